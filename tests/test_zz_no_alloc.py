"""mgpu_integrals_noalloc, the integrals through a path that allocates
nothing, against mgpu_integrals_compute on the same state.

Both run the same per-face expressions and the same per-station reduction
order; only the FP64 efficiency formula runs on the device here and on the
host there (device pow against the host C library), so the bar is 1e-12
relative on every returned number.  The file is named to be collected last,
so it also runs after everything else has used the library in the process;
it passes on its own in a fresh process as well.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12
FIELDS = ("mass_flow_in", "mass_flow_out", "eta_tt", "eta_ts", "po_ratio", "to_ratio")
MAX_JM = 4096   # MGPU_NOALLOC_MAX_JM in include/mgpu.h


@pytest.fixture(scope="module")
def mods():
    from mgpu import case, common_setup, lib
    lib.load()
    return case, common_setup, lib


def _close(a, b):
    for f in FIELDS:
        x, y = getattr(a, f), getattr(b, f)
        assert np.isfinite(x) and abs(x - y) <= TOL * max(1.0, abs(y)), (f, x, y)
    assert (a.j1, a.j2m1) == (b.j1, b.j2m1)


@pytest.mark.parametrize("which,nsteps", [("small_stage", 40), ("small_nozzle", 25)])
def test_noalloc_matches_integrals_compute(mods, which, nsteps):
    case, common_setup, lib = mods
    gpu = lib.Problem(common_setup.build_common(getattr(case, which)()))
    gpu.run(nsteps)
    ref = gpu.integrals()
    first = gpu.integrals_noalloc()
    second = gpu.integrals_noalloc()
    _close(first, ref)
    _close(second, ref)
    for f in FIELDS:                      # same state, same fixed scratch: identical
        assert getattr(first, f) == getattr(second, f), f
    # marching on and asking again follows the new state
    gpu.run(5)
    _close(gpu.integrals_noalloc(), gpu.integrals())


def test_noalloc_setup_only_and_no_device_growth(mods):
    """out=NULL performs only the per-device set-up; afterwards repeated calls
    take no device memory (free memory does not drop)."""
    case, common_setup, lib = mods
    torch = pytest.importorskip("torch")
    gpu = lib.Problem(common_setup.build_common(case.small_stage()))
    L = lib.load()
    assert L.mgpu_integrals_noalloc(gpu.h, None) == 0
    gpu.sync()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        gpu.integrals_noalloc()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 >= free0


def test_noalloc_rejects_oversize_and_uncommitted(mods):
    case, common_setup, lib = mods
    L = lib.load()
    h = ctypes.c_void_p()
    out = lib.Integrals()
    assert L.mgpu_create(9, MAX_JM + 1, 7, 1, ctypes.byref(h)) == 0
    try:
        rc = L.mgpu_integrals_noalloc(h, ctypes.byref(out))
        assert rc == -1
        assert "MGPU_NOALLOC_MAX_JM" in lib.last_error()
    finally:
        L.mgpu_destroy(h)
    h = ctypes.c_void_p()
    assert L.mgpu_create(9, 29, 7, 1, ctypes.byref(h)) == 0
    try:
        assert L.mgpu_integrals_noalloc(h, None) == 0        # set-up only
        assert L.mgpu_integrals_noalloc(h, ctypes.byref(out)) == -2
    finally:
        L.mgpu_destroy(h)
    assert L.mgpu_integrals_noalloc(None, ctypes.byref(out)) == -1
