"""Blade-angle design variables and the chain from the adjoint's geometry
gradients to them.

The design variables are offsets, in degrees, of the stagger and of the
inlet and exit metal angles at `nsect` equispaced span sections of every
blade row (30 for the two-row stage at 5 sections), applied on top of
seeded base offsets drawn uniformly in +-1 degree.  They change the blade
surfaces, hence the node angles THETA and through them the face areas and
volumes that the time step reads: AQX, AQR, ABX, ABR, ASX, ASR, VOLOR (ABT,
a meridional area, does not depend on them).

mgpu_adjoint_gradient returns dJ/dA for those arrays.  The derivatives
dA/d(alpha) of the host-side geometry generator are central differences of
the double-precision metrics (`build_common(..., metrics64=True)`), and
dJ/d(alpha_i) = sum over A of dJ/dA . dA/d(alpha_i).  Everything the
frozen step holds fixed (time steps, body forces, smoothing and corner
weights) is held at the base deck's values in the finite-difference checks
as well.
"""
from __future__ import annotations

import copy
import dataclasses
import os
from concurrent.futures import ThreadPoolExecutor
from typing import Callable, Dict, List

import numpy as np

from . import case as _case
from . import common_setup as _cs

KINDS = ("stagger", "inlet", "exit")
GEOM = ("AQX", "AQR", "ABX", "ABR", "ABT", "ASX", "ASR", "VOLOR")


@dataclasses.dataclass
class DesignSpace:
    make_spec: Callable[[], _case.CaseSpec]
    alpha0: np.ndarray            # base offsets, degrees
    nrows: int
    nsect: int

    @classmethod
    def seeded(cls, make_spec, seed: int = 2, nsect: int = 5) -> "DesignSpace":
        spec = make_spec()
        nrows = len(spec.rows)
        rng = np.random.default_rng(seed)
        alpha0 = rng.uniform(-1.0, 1.0, nrows * len(KINDS) * nsect)
        return cls(make_spec=make_spec, alpha0=alpha0, nrows=nrows, nsect=nsect)

    @property
    def size(self) -> int:
        return self.nrows * len(KINDS) * self.nsect

    def index(self, row: int, kind: str, sect: int) -> int:
        return (row * len(KINDS) + KINDS.index(kind)) * self.nsect + sect

    def names(self) -> List[str]:
        return [f"row{r + 1}_{k}_s{s + 1}" for r in range(self.nrows) for k in KINDS for s in range(self.nsect)]

    def spec(self, alpha: np.ndarray) -> _case.CaseSpec:
        spec = self.make_spec()
        a = np.asarray(alpha, np.float64).reshape(self.nrows, len(KINDS), self.nsect)
        for r, row in enumerate(spec.rows):
            row.nsect = self.nsect
            row.d_stag = tuple(a[r, 0])
            row.d_in = tuple(a[r, 1])
            row.d_out = tuple(a[r, 2])
        return spec

    def deck(self, alpha: np.ndarray) -> _cs.CommonData:
        """The REAL*4 COMMON deck of the design alpha."""
        return _cs.build_common(self.spec(alpha))

    def geometry64(self, alpha: np.ndarray) -> Dict[str, np.ndarray]:
        return _cs.build_common(self.spec(alpha), metrics64=True, metrics_only=True).geom64

    def theta64(self, alpha: np.ndarray) -> np.ndarray:
        """The node angles THETA (KM, JM, IM) of the design, double precision."""
        return _cs.build_common(self.spec(alpha), metrics64=True, theta_only=True).theta

    def theta_sensitivities(self, alpha: np.ndarray, h: float = 1e-3) -> np.ndarray:
        """dTHETA/d(alpha_i) (size, KM, JM, IM), per degree: central
        differences of the generator's node angles, without the metrics
        (on a thread pool for large grids, as sensitivities)."""
        def one(i):
            e = np.zeros(self.size)
            e[i] = h
            return (self.theta64(alpha + e) - self.theta64(alpha - e)) / (2.0 * h)
        first = one(0)
        nt = min(16, os.cpu_count() or 1) if first.size > 100_000 else 1
        if nt <= 1:
            return np.stack([first] + [one(i) for i in range(1, self.size)])
        with ThreadPoolExecutor(nt) as ex:
            return np.stack([first] + list(ex.map(one, range(1, self.size))))

    @staticmethod
    def chain_theta(djdtheta: np.ndarray, sens: np.ndarray) -> np.ndarray:
        """dJ/d(alpha) from dJ/dTHETA (mgpu_adjoint_gradient_theta)."""
        g = djdtheta.astype(np.float64).ravel()
        return sens.reshape(sens.shape[0], -1) @ g

    def sensitivities(self, alpha: np.ndarray, h: float = 1e-3, threads: int | None = None) -> List[Dict[str, np.ndarray]]:
        """dA/d(alpha_i) per design variable (per degree), central differences
        of the double-precision metrics.  The 2 x size geometry evaluations
        are independent and spend their time in NumPy array operations, which
        release the GIL, so they run on a thread pool."""
        def one(i):
            e = np.zeros(self.size)
            e[i] = h
            gp, gm = self.geometry64(alpha + e), self.geometry64(alpha - e)
            return {n: (gp[n] - gm[n]) / (2.0 * h) for n in GEOM}
        first = one(0)
        big = first["VOLOR"].size > 100_000      # small grids: the pool costs more than it saves
        nt = threads if threads is not None else (min(16, os.cpu_count() or 1) if big else 1)
        if nt <= 1:
            return [first] + [one(i) for i in range(1, self.size)]
        with ThreadPoolExecutor(nt) as ex:
            return [first] + list(ex.map(one, range(1, self.size)))

    @staticmethod
    def chain(dJdA: Dict[str, np.ndarray], sens: List[Dict[str, np.ndarray]]) -> np.ndarray:
        """dJ/d(alpha) from the geometry gradients."""
        return np.array([sum(float(np.sum(dJdA[n].astype(np.float64) * s[n])) for n in GEOM) for s in sens])


def perturbed_state(base: _cs.CommonData, state: Dict[str, np.ndarray], delta64: Dict[str, np.ndarray]):
    """The finite-difference check's restart: the converged state and every
    frozen array of `state` (arrays read back from the converged problem),
    with the face areas and volumes moved by the double-precision geometry
    change delta64 (rounded to REAL*4 once, on the sum)."""
    cd = copy.copy(base)
    cd.arrays = dict(base.arrays)
    cd.ints = dict(base.ints)
    cd.reals = dict(base.reals)
    for n, a in state.items():
        cd.arrays[n] = a
    for n in GEOM:
        cd.arrays[n] = (state.get(n, base.arrays[n]).astype(np.float64) + delta64[n]).astype(np.float32)
    return cd
