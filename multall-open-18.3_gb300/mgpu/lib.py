"""ctypes binding of libmgpu.so (the C ABI in include/mgpu.h).

`Problem` binds one case's COMMON data to a device handle by name, performs
the calls SETUP makes into the hot path (STEPUP(1.0), the first LOSS) and
then marches.  There is no CPU fallback: if the CUDA library cannot be
loaded, or no GPU is present, the constructor raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from . import build as _build

MGPU_OK = 0


class Monitors(ctypes.Structure):
    _fields_ = [("nstep", ctypes.c_int32), ("tail_ran", ctypes.c_int32), ("ifend", ctypes.c_int32),
                ("health", ctypes.c_int32), ("emax", ctypes.c_float), ("imax", ctypes.c_int32),
                ("jmax", ctypes.c_int32), ("kmax", ctypes.c_int32), ("eavg", ctypes.c_float),
                ("econt", ctypes.c_float), ("jcont", ctypes.c_int32), ("vref", ctypes.c_float),
                ("vmax", ctypes.c_float), ("ivmax", ctypes.c_int32), ("jvmax", ctypes.c_int32),
                ("kvmax", ctypes.c_int32), ("flow_in", ctypes.c_double), ("flow_out", ctypes.c_double)]


class Stage(ctypes.Structure):
    """One row of EFICOOL's stage table (mgpu_stage)."""
    _fields_ = [("j1", ctypes.c_int32), ("j2m1", ctypes.c_int32), ("jmix", ctypes.c_int32),
                ("has_reaction", ctypes.c_int32), ("mass_flow_in", ctypes.c_double),
                ("mass_flow_out", ctypes.c_double), ("po_ratio", ctypes.c_double), ("to_ratio", ctypes.c_double),
                ("delta_to", ctypes.c_double), ("eta_tt", ctypes.c_double), ("eta_ts", ctypes.c_double),
                ("eta_poly", ctypes.c_double), ("reac_hub", ctypes.c_double), ("reac_mid", ctypes.c_double),
                ("reac_tip", ctypes.c_double)]


class Integrals(ctypes.Structure):
    _fields_ = [("mass_flow_in", ctypes.c_double), ("mass_flow_out", ctypes.c_double),
                ("eta_tt", ctypes.c_double), ("eta_ts", ctypes.c_double), ("po_ratio", ctypes.c_double),
                ("to_ratio", ctypes.c_double), ("j1", ctypes.c_int32), ("j2m1", ctypes.c_int32)]


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 48), ("launches", ctypes.c_int32), ("total_ms", ctypes.c_double)]


# every entry point include/mgpu.h declares
EXPORTS = ["mgpu_abi_version", "mgpu_last_error", "mgpu_device_count", "mgpu_create", "mgpu_destroy",
           "mgpu_set_int", "mgpu_set_real", "mgpu_set_array", "mgpu_get_array", "mgpu_get_real", "mgpu_get_int",
           "mgpu_commit", "mgpu_stepup", "mgpu_loss_init", "mgpu_step", "mgpu_run", "mgpu_sync",
           "mgpu_integrals_compute", "mgpu_kernels_per_step", "mgpu_bench_steps", "mgpu_profile_steps",
           "mgpu_step_io_bytes", "mgpu_integrals_noalloc", "mgpu_batch_create", "mgpu_batch_destroy",
           "mgpu_batch_run", "mgpu_batch_bench_steps", "mgpu_adjoint_prepare", "mgpu_adjoint_objective",
           "mgpu_adjoint_iterate", "mgpu_adjoint_solve", "mgpu_adjoint_gradient", "mgpu_adjoint_get",
           "mgpu_adjoint_set", "mgpu_adjoint_solve_krylov", "mgpu_autotune", "mgpu_write_flow_out",
           "mgpu_read_flow_out", "mgpu_stage_performance", "mgpu_adjoint_gradient_theta",
           "mgpu_write_grid_out", "mgpu_setup_metrics", "mgpu_setup_metrics64", "mgpu_setup_geometry"]

# SETUP's metric arrays, which mgpu_setup_metrics forms on the device
METRIC_ARRAYS = ("AQX", "AQR", "ABX", "ABR", "VOL", "ASX", "ASR", "VOLOR", "ABT", "WRABT")

_lib = None


def load(build: bool = True):
    """Loads libmgpu.so (building it in-tree first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"libmgpu.so not found at {path}; the CUDA library is required")
    L = ctypes.CDLL(path)
    vp, cp, i32 = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int32
    L.mgpu_abi_version.restype = i32
    L.mgpu_last_error.argtypes = [ctypes.c_char_p, i32]
    L.mgpu_device_count.restype = i32
    L.mgpu_create.argtypes = [i32, i32, i32, i32, ctypes.POINTER(vp)]
    L.mgpu_destroy.argtypes = [vp]
    L.mgpu_destroy.restype = None
    L.mgpu_set_int.argtypes = [vp, cp, i32]
    L.mgpu_set_real.argtypes = [vp, cp, ctypes.c_float]
    L.mgpu_set_array.argtypes = [vp, cp, vp, ctypes.c_int64]
    L.mgpu_get_array.argtypes = [vp, cp, vp, ctypes.c_int64]
    L.mgpu_get_real.argtypes = [vp, cp, ctypes.POINTER(ctypes.c_float)]
    L.mgpu_get_int.argtypes = [vp, cp, ctypes.POINTER(i32)]
    L.mgpu_commit.argtypes = [vp]
    L.mgpu_stepup.argtypes = [vp, ctypes.c_float]
    L.mgpu_loss_init.argtypes = [vp]
    L.mgpu_step.argtypes = [vp, i32, ctypes.POINTER(Monitors)]
    L.mgpu_run.argtypes = [vp, i32, ctypes.POINTER(Monitors)]
    L.mgpu_sync.argtypes = [vp]
    L.mgpu_integrals_compute.argtypes = [vp, ctypes.POINTER(Integrals)]
    L.mgpu_integrals_noalloc.argtypes = [vp, ctypes.POINTER(Integrals)]
    L.mgpu_kernels_per_step.argtypes = [vp, i32]
    L.mgpu_bench_steps.argtypes = [vp, i32, i32, ctypes.POINTER(ctypes.c_double)]
    L.mgpu_profile_steps.argtypes = [vp, i32, ctypes.POINTER(KernelTime), i32, ctypes.POINTER(i32)]
    L.mgpu_step_io_bytes.argtypes = [ctypes.POINTER(i32), ctypes.POINTER(i32)]
    L.mgpu_batch_create.argtypes = [ctypes.POINTER(vp), i32, ctypes.POINTER(vp)]
    L.mgpu_batch_destroy.argtypes = [vp]
    L.mgpu_batch_run.argtypes = [vp, i32, ctypes.POINTER(Monitors)]
    L.mgpu_batch_bench_steps.argtypes = [vp, i32, i32, ctypes.POINTER(ctypes.c_double)]
    dp = ctypes.POINTER(ctypes.c_double)
    L.mgpu_adjoint_prepare.argtypes = [vp]
    L.mgpu_adjoint_objective.argtypes = [vp, i32, dp]
    L.mgpu_adjoint_iterate.argtypes = [vp, i32, dp]
    L.mgpu_adjoint_solve.argtypes = [vp, i32, ctypes.c_double, ctypes.POINTER(i32), dp]
    L.mgpu_adjoint_gradient.argtypes = [vp]
    L.mgpu_autotune.argtypes = [vp, ctypes.POINTER(i32), dp]
    L.mgpu_write_flow_out.argtypes = [vp, cp, vp]
    L.mgpu_write_grid_out.argtypes = [vp, cp]
    L.mgpu_stage_performance.argtypes = [vp, i32, ctypes.POINTER(Stage)]
    L.mgpu_adjoint_gradient_theta.argtypes = [vp, vp, ctypes.c_int64]
    L.mgpu_read_flow_out.argtypes = [vp, cp, ctypes.POINTER(i32)]
    L.mgpu_adjoint_solve_krylov.argtypes = [vp, i32, i32, i32, ctypes.c_double, ctypes.c_double,
                                            ctypes.POINTER(i32), dp]
    L.mgpu_adjoint_get.argtypes = [vp, cp, vp, ctypes.c_int64]
    L.mgpu_adjoint_set.argtypes = [vp, cp, vp, ctypes.c_int64]
    L.mgpu_setup_metrics.argtypes = [vp]
    L.mgpu_setup_geometry.argtypes = [vp, i32, vp, vp, vp]
    L.mgpu_setup_metrics64.argtypes = [vp, vp, vp, vp, vp, ctypes.c_int64]
    for f in EXPORTS:
        fn = getattr(L, f)
        if f in ("mgpu_destroy", "mgpu_batch_destroy"):
            fn.restype = None
        else:
            fn.restype = i32
    _lib = L
    return L


class MgpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"mgpu error {code}: {msg}")
        self.code = code


def step_io_bytes() -> tuple[int, int]:
    """(host->device, device->host) bytes of one mgpu_step call."""
    a, b = ctypes.c_int32(), ctypes.c_int32()
    _chk(load().mgpu_step_io_bytes(ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    load().mgpu_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def _chk(rc: int) -> int:
    if rc < 0:
        raise MgpuError(rc, last_error())
    return rc


class Problem:
    """One flow problem resident on the current GPU."""

    def __init__(self, cd, setup_calls: bool = True, restart: str | None = None, device_metrics: bool = False,
                 device_geometry=None):
        """restart: a flow_out file read after the COMMON data are bound and
        before the commit, as SETUP reads it with IF_RESTART = 1.
        device_metrics: the face areas and volumes are not bound from cd but
        formed on the device from X, R and RTHETA (mgpu_setup_metrics).
        device_geometry: a deck's CaseGeometry whose blade sections give the
        grid and its metrics on the device (mgpu_setup_geometry) in place of
        cd's X, R, RT_THICK, RTHETA and metric arrays."""
        L = load()
        n = L.mgpu_device_count()
        if n <= 0:
            raise MgpuError(n, "no CUDA device visible: the GPU library has no CPU fallback")
        self.cd = cd
        h = ctypes.c_void_p()
        _chk(L.mgpu_create(cd.im, cd.jm, cd.km, cd.nrows, ctypes.byref(h)))
        self.h = h
        for k, v in cd.ints.items():
            _chk(L.mgpu_set_int(self.h, k.encode(), int(v)))
        for k, v in cd.reals.items():
            _chk(L.mgpu_set_real(self.h, k.encode(), float(v)))
        skip = set(METRIC_ARRAYS) if (device_metrics or device_geometry is not None) else set()
        if device_geometry is not None:
            skip |= {"X", "R", "RT_THICK", "RTHETA"}
        for k, a in cd.arrays.items():
            if k in skip:
                continue
            a = np.ascontiguousarray(a)
            _chk(L.mgpu_set_array(self.h, k.encode(), a.ctypes.data, a.nbytes))
        if device_geometry is not None:
            g = device_geometry
            sec = np.ascontiguousarray(g.sections, np.float32)
            fth = np.ascontiguousarray(g.fthick, np.float32)
            frt = np.ascontiguousarray(g.fractip, np.float32)
            _chk(L.mgpu_setup_geometry(self.h, sec.shape[1], sec.ctypes.data, fth.ctypes.data, frt.ctypes.data))
        elif device_metrics:
            _chk(L.mgpu_setup_metrics(self.h))
        self.restart_nstep = None
        if restart is not None:
            ns = ctypes.c_int32()
            _chk(L.mgpu_read_flow_out(self.h, os.fsencode(restart), ctypes.byref(ns)))
            self.restart_nstep = ns.value
        _chk(L.mgpu_commit(self.h))
        if setup_calls:
            self.setup_calls()

    def stage(self, nstg: int) -> Stage:
        """EFICOOL's table for stage nstg (NSTAGES+1: the whole machine)."""
        o = Stage()
        _chk(load().mgpu_stage_performance(self.h, int(nstg), ctypes.byref(o)))
        return o

    def write_flow_out(self, path: str, rosub: np.ndarray | None = None):
        """The restart/plotting file flow_out of the current state."""
        if rosub is not None:
            rosub = np.ascontiguousarray(rosub, np.float32)
        _chk(load().mgpu_write_flow_out(self.h, os.fsencode(path), None if rosub is None else rosub.ctypes.data))

    def write_grid_out(self, path: str):
        """SETUP's plotting file grid_out of the bound geometry."""
        _chk(load().mgpu_write_grid_out(self.h, os.fsencode(path)))

    def setup_calls(self):
        """STEPUP(1.0) and the first LOSS, as SETUP makes them."""
        _chk(load().mgpu_stepup(self.h, 1.0))
        _chk(load().mgpu_loss_init(self.h))

    def metrics64(self, x: np.ndarray, r: np.ndarray, rtheta: np.ndarray) -> dict:
        """SETUP's metrics in double precision on the device from double X,
        R (KM, JM) and RTHETA (KM, JM, IM), with this handle's INDMIX and
        WRAD: {name: array} in the COMMON shapes."""
        IM, JM, KM = self.cd.im, self.cd.jm, self.cd.km
        x, r, rt = (np.ascontiguousarray(a, np.float64) for a in (x, r, rtheta))
        N, JK = IM * JM * KM, JM * KM
        out = np.zeros(8 * N + 2 * JK, np.float64)
        _chk(load().mgpu_setup_metrics64(self.h, x.ctypes.data, r.ctypes.data, rt.ctypes.data, out.ctypes.data,
                                         out.size))
        res = {n: out[q * N:(q + 1) * N].reshape(KM, JM, IM) for q, n in enumerate(METRIC_ARRAYS[:8])}
        res["ABT"] = out[8 * N:8 * N + JK].reshape(KM, JM)
        res["WRABT"] = out[8 * N + JK:].reshape(KM, JM)
        return res

    def close(self):
        if getattr(self, "h", None):
            load().mgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, force_end: bool = False, check: bool = True) -> Monitors:
        m = Monitors()
        rc = load().mgpu_step(self.h, 1 if force_end else 0, ctypes.byref(m))
        if check:
            _chk(rc)
        return m

    def run(self, nsteps: int) -> tuple[int, Monitors]:
        m = Monitors()
        rc = _chk(load().mgpu_run(self.h, int(nsteps), ctypes.byref(m)))
        return rc, m

    def sync(self):
        _chk(load().mgpu_sync(self.h))

    def get(self, name: str) -> np.ndarray:
        ref = self.cd.arrays.get(name)
        if ref is not None:
            out = np.zeros(ref.shape, ref.dtype)
        else:
            out = np.zeros((self.cd.km, self.cd.jm, self.cd.im), np.float32)
        _chk(load().mgpu_get_array(self.h, name.encode(), out.ctypes.data, out.nbytes))
        return out

    def get_into(self, name: str, out: np.ndarray) -> np.ndarray:
        """Copies a COMMON array into a caller's contiguous buffer (e.g. pinned
        host memory), without allocating."""
        if not out.flags["C_CONTIGUOUS"]:
            raise ValueError("get_into needs a contiguous buffer")
        _chk(load().mgpu_get_array(self.h, name.encode(), out.ctypes.data, out.nbytes))
        return out

    def set(self, name: str, a: np.ndarray):
        a = np.ascontiguousarray(a)
        _chk(load().mgpu_set_array(self.h, name.encode(), a.ctypes.data, a.nbytes))

    def get_real(self, name: str) -> float:
        v = ctypes.c_float()
        _chk(load().mgpu_get_real(self.h, name.encode(), ctypes.byref(v)))
        return v.value

    def integrals(self) -> Integrals:
        o = Integrals()
        _chk(load().mgpu_integrals_compute(self.h, ctypes.byref(o)))
        return o

    def integrals_noalloc(self) -> Integrals:
        """The same integrals through mgpu_integrals_noalloc (fixed static
        device scratch, no allocation; calls on one device must not overlap)."""
        o = Integrals()
        _chk(load().mgpu_integrals_noalloc(self.h, ctypes.byref(o)))
        return o

    def kernels_per_step(self, loss: bool = False, tail: bool = False) -> int:
        """Kernel launches of one step (LOSS and tail steps launch more)."""
        return _chk(load().mgpu_kernels_per_step(self.h, (1 if loss else 0) | (2 if tail else 0)))

    TUNE_CANDIDATES = (128, 192, 256, 512)

    def autotune(self) -> tuple[tuple, dict]:
        """((threads per J-plane CTA chosen for the RO/ROE pass, for the
        momentum pass), {"2": [ms per pass of 2 variables for 128, 192, 256,
        512], "3": [the same for the pass of 3]})."""
        c = (ctypes.c_int32 * 2)()
        ms = (ctypes.c_double * 8)()
        _chk(load().mgpu_autotune(self.h, c, ms))
        return (c[0], c[1]), {"2": list(ms[:4]), "3": list(ms[4:])}

    def bench_steps(self, nsteps: int, flush_l2: bool = True) -> float:
        """Sum of the device times (ms) of nsteps iterations."""
        ms = ctypes.c_double()
        _chk(load().mgpu_bench_steps(self.h, int(nsteps), 1 if flush_l2 else 0, ctypes.byref(ms)))
        return ms.value

    def profile_steps(self, nsteps: int) -> list:
        """[(kernel name, launches, total ms)] over nsteps iterations."""
        arr = (KernelTime * 256)()
        n = ctypes.c_int32()
        _chk(load().mgpu_profile_steps(self.h, int(nsteps), arr, 256, ctypes.byref(n)))
        return [(arr[i].name.decode(), arr[i].launches, arr[i].total_ms) for i in range(n.value)]


    # ---- discrete adjoint ---------------------------------------------------
    ADJ_STATE = ["RO", "ROVX", "ROVR", "RORVT", "ROE", "DRO", "DROE", "DROVX", "DROVR", "DRORVT",
                 "P", "HO", "ROVT", "PEFF", "PD"]
    ADJ_GEOM = ["AQX", "AQR", "ABX", "ABR", "ABT", "ASX", "ASR", "VOLOR"]
    OBJECTIVES = {"none": -1, "eta_tt": 0, "mass_flow_in": 1, "mass_flow_out": 2}

    def adjoint_prepare(self):
        """Records the linearisation step at the current state."""
        _chk(load().mgpu_adjoint_prepare(self.h))

    def adjoint_objective(self, which: str) -> float:
        v = ctypes.c_double()
        _chk(load().mgpu_adjoint_objective(self.h, self.OBJECTIVES[which], ctypes.byref(v)))
        return v.value

    def adjoint_iterate(self, n: int = 1) -> float:
        r = ctypes.c_double()
        _chk(load().mgpu_adjoint_iterate(self.h, int(n), ctypes.byref(r)))
        return r.value

    def adjoint_solve(self, max_iters: int, tol: float) -> tuple[bool, int, float]:
        """(converged, iterations, last relative change)."""
        it, r = ctypes.c_int32(), ctypes.c_double()
        rc = _chk(load().mgpu_adjoint_solve(self.h, int(max_iters), float(tol), ctypes.byref(it), ctypes.byref(r)))
        return rc == 0, it.value, r.value

    def adjoint_solve_krylov(self, inner: int = 40, restart: int = 30, max_steps: int = 20000, tol: float = 1e-6,
                             stall: float = 0.0):
        """(converged, transposed steps used, relative residual) of GMRES on
        the inner-step map; stall > 0 stops when a restart cycle lowers the
        residual by less than that fraction."""
        it, r = ctypes.c_int32(), ctypes.c_double()
        rc = _chk(load().mgpu_adjoint_solve_krylov(self.h, int(inner), int(restart), int(max_steps), float(tol),
                                                   float(stall), ctypes.byref(it), ctypes.byref(r)))
        return rc == 0, it.value, r.value

    def adjoint_gradient_theta(self) -> np.ndarray:
        """dJ/dTHETA (KM, JM, IM) on the device from the last adjoint_gradient."""
        out = np.zeros((self.cd.km, self.cd.jm, self.cd.im), np.float32)
        _chk(load().mgpu_adjoint_gradient_theta(self.h, out.ctypes.data, out.nbytes))
        return out

    def adjoint_gradient(self, read: bool = True) -> dict | None:
        """dJ/dA for the geometry arrays (one more reverse step); read=False
        leaves them on the device (for adjoint_gradient_theta)."""
        _chk(load().mgpu_adjoint_gradient(self.h))
        if not read:
            return None
        return {n: self.adjoint_get("d" + n) for n in self.ADJ_GEOM}

    def _adj_shape(self, name: str):
        base = name[1:] if name.startswith("d") and name[1:] in self.ADJ_GEOM else name
        ref = self.cd.arrays.get(base)
        return ref.shape if ref is not None else (self.cd.km, self.cd.jm, self.cd.im)

    def adjoint_get(self, name: str) -> np.ndarray:
        out = np.zeros(self._adj_shape(name), np.float32)
        _chk(load().mgpu_adjoint_get(self.h, name.encode(), out.ctypes.data, out.nbytes))
        return out

    def adjoint_set(self, name: str, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float32)
        _chk(load().mgpu_adjoint_set(self.h, name.encode(), a.ctypes.data, a.nbytes))


class Batch:
    """Several Problems stepped by one CUDA graph launch per iteration (one
    graph branch per problem); each problem's results are the same as when
    it is stepped alone."""

    def __init__(self, problems):
        L = load()
        self.problems = list(problems)
        arr = (ctypes.c_void_p * len(self.problems))(*[p.h.value for p in self.problems])
        b = ctypes.c_void_p()
        _chk(L.mgpu_batch_create(arr, len(self.problems), ctypes.byref(b)))
        self.b = b

    def run(self, nsteps: int):
        """(members whose end test is met, [Monitors per member])."""
        mons = (Monitors * len(self.problems))()
        ended = _chk(load().mgpu_batch_run(self.b, int(nsteps), mons))
        return ended, list(mons)

    def bench_steps(self, nsteps: int, flush_l2: bool = True) -> float:
        ms = ctypes.c_double()
        _chk(load().mgpu_batch_bench_steps(self.b, int(nsteps), 1 if flush_l2 else 0, ctypes.byref(ms)))
        return ms.value

    def close(self):
        if getattr(self, "b", None):
            load().mgpu_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
