"""The restart/plotting file flow_out and EFICOOL's stage table through the C
ABI.  flow_out: the file the GPU writes (OUTPUT, multall-open-18.3.f:
5942-5978) against the FP32 oracle's, and a restart from a file (SETUP's
IF_RESTART branch, 6920-6992) against the oracle's restart from the same
file.  The stage table (11253-11420) against the oracle's."""
import copy

import numpy as np
import pytest

from helpers import STATE, read_flow_out, rel_linf

pytestmark = pytest.mark.gpu

FIELDS = ["RO", "ROVX", "ROVR", "ROVT", "ROE", "ROSUB", "DPDS_CELL*1e-6", "PEFF+PREFF"]


@pytest.fixture(scope="module")
def mods():
    from mgpu import case, common_setup, lib
    import oracle as O
    lib.load()
    return case, common_setup, lib, O


def _restart_deck(cd):
    c = copy.copy(cd)
    c.ints = dict(cd.ints)
    c.ints["IF_RESTART"] = 1
    return c


def test_flow_out_matches_oracle(mods, tmp_path):
    """After three steps the GPU's flow_out has the oracle's record layout,
    the GPU's own arrays exactly, and the oracle's values within 1e-5 (the
    conserved variables) and 1e-4 (the LOSS wall term and PEFF)."""
    case, common_setup, lib, O = mods
    cd = common_setup.build_common(case.small_stage())
    gpu = lib.Problem(cd)
    ref = O.Oracle(cd)
    ref.setup_calls()
    for _ in range(3):
        gpu.step()
        ref.step()
    fg, fr = str(tmp_path / "gpu_flow_out"), str(tmp_path / "ref_flow_out")
    gpu.write_flow_out(fg)
    ref.write_flow_out(fr)
    N = cd.nodes()
    ng, ag = read_flow_out(fg, N)
    nr, ar = read_flow_out(fr, N)
    assert ng == nr == 3
    for a, n in zip(ag[:5], ("RO", "ROVX", "ROVR", "ROVT", "ROE")):
        assert np.array_equal(a, gpu.get(n).ravel()), n
    for a, b, n in zip(ag, ar, FIELDS):
        tol = 1e-4 if n in ("DPDS_CELL*1e-6", "PEFF+PREFF") else 1e-5
        assert rel_linf(a, b) <= tol, (n, rel_linf(a, b))


def test_restart_matches_oracle_restart(mods, tmp_path):
    """A restart from the oracle's file: the secondary variables, PEFF = P,
    the exit pressures PD and LOOP's PREFF are the oracle's bit for bit;
    five steps later every field is within 1e-4."""
    case, common_setup, lib, O = mods
    cd = common_setup.build_common(case.small_stage())
    ref = O.Oracle(cd)
    ref.setup_calls()
    for _ in range(3):
        ref.step()
    f = str(tmp_path / "flow_out")
    ref.write_flow_out(f)
    cdr = _restart_deck(cd)
    gpu = lib.Problem(cdr, restart=f)
    ref2 = O.Oracle(cdr, restart=f)
    ref2.setup_calls()
    assert gpu.restart_nstep == ref2.restart_nstep == 3
    for n in ("RO", "ROVX", "ROVR", "ROVT", "ROE", "RORVT", "VX", "VR", "VT", "T_STATIC", "HO", "P", "PEFF", "PD"):
        assert np.array_equal(gpu.get(n).ravel(), ref2.get(n, double=False).ravel()), n
    assert gpu.get_real("PREFF") == ref2.get_real("PREFF")
    for _ in range(5):
        gpu.step()
        ref2.step()
    for n in STATE:
        assert rel_linf(gpu.get(n), ref2.get(n)) <= 1e-4, (n, rel_linf(gpu.get(n), ref2.get(n)))


def test_gpu_checkpoint_round_trip(mods, tmp_path):
    """The GPU's own checkpoint: a new handle restarted from it holds the
    writer's conserved variables exactly."""
    case, common_setup, lib, O = mods
    cd = common_setup.build_common(case.small_nozzle())
    gpu = lib.Problem(cd)
    gpu.run(7)
    f = str(tmp_path / "flow_out")
    gpu.write_flow_out(f)
    back = lib.Problem(_restart_deck(cd), restart=f)
    assert back.restart_nstep == 7
    for n in ("RO", "ROVX", "ROVR", "ROVT", "ROE"):
        assert np.array_equal(back.get(n), gpu.get(n)), n
    back.run(3)


def test_stage_table_matches_oracle(mods):
    """EFICOOL's stage table of a 4-stage compressor after 30 steps: the
    stations are the oracle's, the mass flows and ratios agree to 1e-4
    relative (FP64 per-J sums on the GPU, REAL*4 in the oracle), the
    efficiencies and reactions to 1e-3."""
    case, common_setup, lib, O = mods
    cd = common_setup.build_common(case.compressor_4stage(im=9, jm_row=25, km=7))
    gpu = lib.Problem(cd)
    ref = O.Oracle(cd)
    ref.setup_calls()
    for _ in range(30):
        gpu.step()
        ref.step()
    for s in range(1, cd.ints["NSTAGES"] + 2):
        g, r = gpu.stage(s), ref.stage(s)
        assert (g.j1, g.j2m1, g.jmix, g.has_reaction) == (r.j1, r.j2m1, r.jmix, r.has_reaction), s
        for f in ("mass_flow_in", "mass_flow_out", "po_ratio", "to_ratio"):
            assert abs(getattr(g, f) - getattr(r, f)) <= 1e-4 * abs(getattr(r, f)), (s, f)
        for f in ("eta_tt", "eta_ts", "eta_poly", "reac_hub", "reac_mid", "reac_tip"):
            assert abs(getattr(g, f) - getattr(r, f)) <= 1e-3, (s, f, getattr(g, f), getattr(r, f))


def test_grid_out_matches_oracle(mods, tmp_path):
    """grid_out holds only bound constants, so the GPU's file is the
    oracle's byte for byte."""
    case, common_setup, lib, O = mods
    cd = common_setup.build_common(case.small_stage())
    gpu = lib.Problem(cd, setup_calls=False)
    ref = O.Oracle(cd)
    fg, fr = str(tmp_path / "gpu_grid_out"), str(tmp_path / "ref_grid_out")
    gpu.write_grid_out(fg)
    ref.write_grid_out(fr)
    assert open(fg, "rb").read() == open(fr, "rb").read()


def test_flow_out_of_another_grid_is_refused(mods, tmp_path):
    case, common_setup, lib, O = mods
    cd = common_setup.build_common(case.small_stage())
    ref = O.Oracle(cd)
    f = str(tmp_path / "flow_out")
    ref.write_flow_out(f)
    other = common_setup.build_common(case.small_nozzle())
    with pytest.raises(lib.MgpuError):
        lib.Problem(other, restart=f)
