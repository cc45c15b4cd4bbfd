"""ctypes driver for the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product path.  The oracle is a
serial C++ restatement of Multall's LOOP (see multall_oracle.cpp) driven
through the same COMMON-name interface as the GPU library, so a test binds
one CommonData to both and compares.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


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


def build(force: bool = False) -> str:
    """Compiles liboracle.so with the recipe in oracle/Makefile."""
    src = os.path.join(HERE, "multall_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, cp = ctypes.c_void_p, ctypes.c_char_p
        L.oref_create.restype = vp
        L.oref_create.argtypes = [ctypes.c_int32] * 5
        L.oref_destroy.argtypes = [vp]
        L.oref_last_error.restype = cp
        L.oref_set_int.argtypes = [vp, cp, ctypes.c_int32]
        L.oref_set_real.argtypes = [vp, cp, ctypes.c_double]
        L.oref_get_real.argtypes = [vp, cp, ctypes.POINTER(ctypes.c_double)]
        L.oref_get_int.argtypes = [vp, cp, ctypes.POINTER(ctypes.c_int32)]
        L.oref_set_array.argtypes = [vp, cp, vp, ctypes.c_int64]
        L.oref_get_array.argtypes = [vp, cp, vp, ctypes.c_int64, ctypes.c_int32]
        L.oref_commit.argtypes = [vp]
        L.oref_stepup.argtypes = [vp, ctypes.c_double]
        L.oref_loss_init.argtypes = [vp]
        L.oref_step.argtypes = [vp, ctypes.c_int32, ctypes.POINTER(Monitors)]
        L.oref_integrals.argtypes = [vp, ctypes.POINTER(Integrals)]
        dp = ctypes.POINTER(ctypes.c_double)
        L.oref_set_array_f64.argtypes = [vp, cp, vp, ctypes.c_int64]
        L.oref_ad_begin.argtypes = [vp]
        L.oref_ad_zero.argtypes = [vp]
        L.oref_ad_seed.argtypes = [vp, cp, vp, ctypes.c_int64]
        L.oref_ad_reverse.argtypes = [vp]
        L.oref_ad_grad.argtypes = [vp, cp, vp, ctypes.c_int64]
        L.oref_ad_tape_size.argtypes = [vp]
        L.oref_ad_tape_size.restype = ctypes.c_int64
        L.oref_write_flow_out.argtypes = [vp, cp, vp]
        L.oref_stage_performance.argtypes = [vp, ctypes.c_int32, ctypes.POINTER(Stage)]
        L.oref_write_grid_out.argtypes = [vp, cp]
        L.oref_read_flow_out.argtypes = [vp, cp, ctypes.POINTER(ctypes.c_int32)]
        for f in ("oref_set_int", "oref_set_real", "oref_get_real", "oref_get_int", "oref_set_array",
                  "oref_get_array", "oref_commit", "oref_stepup", "oref_loss_init", "oref_step",
                  "oref_integrals", "oref_set_array_f64", "oref_ad_begin", "oref_ad_zero", "oref_ad_seed",
                  "oref_ad_reverse", "oref_ad_grad", "oref_write_flow_out", "oref_read_flow_out",
                  "oref_stage_performance", "oref_write_grid_out"):
            getattr(L, f).restype = ctypes.c_int32
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


class Oracle:
    """One oracle problem: float or double arithmetic, or (ad=True) double
    arithmetic recorded on a tape for reverse-mode derivatives."""

    def __init__(self, cd, double: bool = False, ad: bool = False, restart: str | None = None):
        """restart: a flow_out file read before the commit, as SETUP reads it
        with IF_RESTART = 1 (multall-open-18.3.f:6920-6992)."""
        L = lib()
        self.cd = cd
        self.double = double or ad
        self.ad = ad
        self.h = L.oref_create(cd.im, cd.jm, cd.km, cd.nrows, 2 if ad else (1 if double else 0))
        if not self.h:
            raise OracleError(L.oref_last_error().decode())
        for k, v in cd.ints.items():
            self._chk(L.oref_set_int(self.h, k.encode(), int(v)))
        for k, v in cd.reals.items():
            self._chk(L.oref_set_real(self.h, k.encode(), float(v)))
        for k, a in cd.arrays.items():
            a = np.ascontiguousarray(a)
            self._chk(L.oref_set_array(self.h, k.encode(), a.ctypes.data, a.nbytes))
        self.restart_nstep = None
        if restart is not None:
            ns = ctypes.c_int32()
            self._chk(L.oref_read_flow_out(self.h, os.fsencode(restart), ctypes.byref(ns)))
            self.restart_nstep = ns.value
        self._chk(L.oref_commit(self.h))

    def stage(self, nstg: int) -> "Stage":
        """EFICOOL's table for stage nstg (NSTAGES+1: the whole machine)."""
        o = Stage()
        self._chk(lib().oref_stage_performance(self.h, int(nstg), ctypes.byref(o)))
        return o

    def write_grid_out(self, path: str):
        """SETUP's plotting file grid_out (6585-6597) of the bound geometry."""
        self._chk(lib().oref_write_grid_out(self.h, os.fsencode(path)))

    def write_flow_out(self, path: str, rosub: np.ndarray | None = None):
        """OUTPUT's restart/plotting file flow_out (5942-5978) of the state."""
        if rosub is not None:
            rosub = np.ascontiguousarray(rosub, np.float32)
        self._chk(lib().oref_write_flow_out(self.h, os.fsencode(path), None if rosub is None else rosub.ctypes.data))

    def _chk(self, rc):
        if rc != 0:
            raise OracleError(f"oracle error {rc}: {lib().oref_last_error().decode()}")
        return rc

    def close(self):
        if self.h:
            lib().oref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setup_calls(self):
        """The two hot-path calls SETUP makes: STEPUP(1.0), then LOSS."""
        self._chk(lib().oref_stepup(self.h, 1.0))
        self._chk(lib().oref_loss_init(self.h))

    def step(self, force_end: bool = False, check: bool = True) -> Monitors:
        m = Monitors()
        rc = lib().oref_step(self.h, 1 if force_end else 0, ctypes.byref(m))
        if check:
            self._chk(rc)
        return m

    def get(self, name: str, double: bool = True) -> np.ndarray:
        ref = self.cd.arrays.get(name)
        shape = ref.shape if ref is not None else (self.cd.km, self.cd.jm, self.cd.im)
        dt = np.float64 if double else (ref.dtype if ref is not None else np.float32)
        out = np.zeros(shape, dt)
        self._chk(lib().oref_get_array(self.h, name.encode(), out.ctypes.data, out.nbytes, 1 if double else 0))
        return out

    def get_int(self, name: str) -> int:
        """An integer scalar, or one of the oracle's branch counters of the
        last step: ORACLE_NDENS (density-limiter changes), ORACLE_NMACH
        (Mach-limiter changes), ORACLE_NPM (Prandtl-Meyer sweep updates)."""
        v = ctypes.c_int32()
        self._chk(lib().oref_get_int(self.h, name.encode(), ctypes.byref(v)))
        return v.value

    def get_real(self, name: str) -> float:
        v = ctypes.c_double()
        self._chk(lib().oref_get_real(self.h, name.encode(), ctypes.byref(v)))
        return v.value

    def integrals(self) -> Integrals:
        o = Integrals()
        self._chk(lib().oref_integrals(self.h, ctypes.byref(o)))
        return o

    def set_f64(self, name: str, values: np.ndarray):
        """Overwrites a REAL array with double values (finite-difference checks)."""
        a = np.ascontiguousarray(values, dtype=np.float64)
        self._chk(lib().oref_set_array_f64(self.h, name.encode(), a.ctypes.data, a.size))

    # ---- reverse mode (ad=True) -------------------------------------------
    def ad_begin(self):
        """Makes every REAL COMMON array an independent variable; the next
        steps are recorded."""
        self._chk(lib().oref_ad_begin(self.h))

    def ad_reverse(self, seeds: dict) -> None:
        """Output adjoints {array name: values} on the arrays' current values,
        then one reverse sweep of the tape."""
        L = lib()
        self._chk(L.oref_ad_zero(self.h))
        for name, w in seeds.items():
            w = np.ascontiguousarray(w, dtype=np.float64)
            self._chk(L.oref_ad_seed(self.h, name.encode(), w.ctypes.data, w.size))
        self._chk(L.oref_ad_reverse(self.h))

    def ad_grad(self, name: str) -> np.ndarray:
        """Adjoint of an array as it was at ad_begin."""
        ref = self.cd.arrays[name]
        out = np.zeros(ref.shape, np.float64)
        self._chk(lib().oref_ad_grad(self.h, name.encode(), out.ctypes.data, out.size))
        return out

    def ad_tape_size(self) -> int:
        return int(lib().oref_ad_tape_size(self.h))
