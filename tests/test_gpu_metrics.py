"""SETUP's face areas and volumes formed on the device (mgpu_setup_metrics,
multall-open-18.3.f:6490-6711) against the host restatement of SETUP in
mgpu/common_setup.py: bit for bit in REAL*4, and in double precision
(mgpu_setup_metrics64) within 1e-12 of the host's double-precision metrics."""
import os

import numpy as np
import pytest

from helpers import STATE

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def mods():
    from mgpu import case, common_setup, deck, lib
    lib.load()
    return case, common_setup, deck, lib


def _cd(mods, which):
    case, common_setup, deck, lib = mods
    if which.startswith("deck:"):
        spec, geo = deck.load_fixture(os.path.join(HERE, "golden", "decks", which[5:] + ".npz"))
        return common_setup.build_common(spec, geo)
    return common_setup.build_common(getattr(case, which)())


@pytest.mark.parametrize("which", ["small_stage", "turbine_stage", "compressor_4stage",
                                   "deck:Single-stage-turbine-17.1", "deck:centrif-compr-17.1"])
def test_device_metrics_equal_setup_bitwise(mods, which):
    """The ten metric arrays formed on the device equal SETUP's REAL*4
    values exactly, mixing planes (the extrapolated theta) included."""
    lib = mods[3]
    cd = _cd(mods, which)
    gpu = lib.Problem(cd, setup_calls=False, device_metrics=True)
    for n in lib.METRIC_ARRAYS:
        g, h = gpu.get(n), cd.arrays[n]
        assert np.array_equal(g, h), (n, float(np.max(np.abs(g.astype(np.float64) - h))))
    gpu.close()


def test_device_metrics_step_like_host_metrics(mods):
    """A handle whose metrics were formed on the device steps exactly like
    one that bound SETUP's: every field equal after five steps."""
    lib = mods[3]
    cd = _cd(mods, "small_stage")
    a = lib.Problem(cd)
    b = lib.Problem(cd, device_metrics=True)
    for _ in range(5):
        a.step()
        b.step()
    for n in STATE:
        assert np.array_equal(a.get(n), b.get(n)), n


@pytest.mark.parametrize("which", ["small_stage", "turbine_stage"])
def test_device_metrics64_match_setup64(mods, which):
    """The double-precision metrics of the design sensitivities: within
    1e-12 relative (L-infinity over each array) of the host's."""
    case, common_setup, deck, lib = mods
    cd = common_setup.build_common(getattr(case, which)(), metrics64=True)
    gpu = lib.Problem(cd, setup_calls=False)
    g64 = cd.geom64
    out = gpu.metrics64(g64["X"], g64["R"], g64["RTHETA"])
    for n in ("AQX", "AQR", "ABX", "ABR", "VOL", "ASX", "ASR", "VOLOR", "ABT", "WRABT"):
        ref = g64[n]
        scale = np.max(np.abs(ref))
        if scale == 0.0:            # e.g. AQR on cylindrical stream surfaces
            assert np.max(np.abs(out[n])) == 0.0, n
            continue
        err = np.max(np.abs(out[n] - ref)) / scale
        assert err <= 1e-12, (n, err)
    gpu.close()


DECKS = ["Single-stage-turbine-17.1", "r37+samods-17.5", "Rotor-37-17.1", "Six-stage-compr-17.1",
         "centrif-compr-17.1", "Transonic-fan-rotor-17.1", "Harrison-cascade-17.1", "Shock-test-17.1"]


@pytest.mark.parametrize("name", DECKS)
def test_device_geometry_from_deck_sections_equals_setup(mods, name):
    """The reference's decks: NEW_INTPOL (tip-gap grid included), the
    alignment at mid-span, the pinched-tip thickness, RTHETA and the metrics
    formed on the device from the reader's blade sections equal the host
    restatement (the deck reader's NEW_INTPOL and mgpu/common_setup.py) bit
    for bit."""
    case, common_setup, deck, lib = mods
    spec, geo = deck.load_fixture(os.path.join(HERE, "golden", "decks", name + ".npz"))
    cd = common_setup.build_common(spec, geo)
    gpu = lib.Problem(cd, setup_calls=False, device_geometry=geo)
    for n in ("X", "R", "RT_THICK", "RTHETA") + lib.METRIC_ARRAYS:
        g, h = gpu.get(n), cd.arrays[n]
        assert np.array_equal(g, h), (n, float(np.max(np.abs(g.astype(np.float64) - h))))
    gpu.close()
