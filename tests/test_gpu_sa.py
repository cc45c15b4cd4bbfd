"""GPU parity of the Spalart-Allmaras model (ILOS 200-299): SPAL_LOSS
(multall-open-18.3.f:13586-14832) and the transport of its cell-centred
turbulent viscosity through the loop (4279-4347, TSTEP's NCALL = 2 branch
5736-5777, the inlet value 4679-4689), called through the C ABI and compared
with the FP32 oracle.

Bars, as for the other loss models: SETUP's call and one step within 1e-5
L-infinity relative, ten steps within 1e-4, a 300-step run within 1e-3.
Option sets: the reader's defaults; the helicity and pressure-gradient
factors with the mixing-length pull (FAC_VORT, FAC_PGRAD, FAC_STMIX);
temperature-dependent viscosity (REYNO < 0); laminar lines from the
transition inputs; the Shih wall functions with the pressure term; SPAL_LOSS
on every step (NLOS = 1, so step 1 re-initialises the viscosity); no tip gap.
"""
import numpy as np
import pytest

from helpers import FORCES, STATE, rel_linf

pytestmark = pytest.mark.gpu

SA_FIELDS = ["TRANS_DYN_VIS", "TRANS_KVIS", "DEL_DYNVIS", "T_SOURCE"]
SA_OPTS = ["defaults", "helicity_pgrad", "reyno_temperature", "transition", "wall_functions", "every_step",
           "no_tip_gap"]


@pytest.fixture(scope="module")
def mods():
    from mgpu import case, common_setup, lib
    import oracle as O
    lib.load()
    return case, common_setup, lib, O


def sa_spec(case, opt, **kw):
    spec = case.small_stage(**kw)
    spec.ilos = 200
    if opt == "helicity_pgrad":
        spec.fac_vort = 1.0
        spec.fac_pgrad = 1.0
        spec.fac_stmix = 1.0
        spec.fac_sfvis = 1.0
    elif opt == "reyno_temperature":
        spec.reyno = -4.0
    elif opt == "wall_functions":
        spec.ypluswall = -15.0
    elif opt == "every_step":
        spec.nlos = 1
    elif opt == "no_tip_gap":
        for r in spec.rows:
            r.tip_gap = 0.0
    return spec


def sa_pair(mods, opt):
    case, common_setup, lib, O = mods
    cd = common_setup.build_common(sa_spec(case, opt))
    if opt == "transition":
        nr = cd.arrays["JTRAN_I1"].size
        for n, v in (("JTRAN_I1", 8), ("JTRAN_IM", 12), ("JTRAN_K1", 4), ("JTRAN_KM", 20)):
            cd.arrays[n] = np.full(nr, v, np.int32)
        cd.reals["FTRANS"] = 2.0
    gpu = lib.Problem(cd)
    ref = O.Oracle(cd)
    ref.setup_calls()
    return cd, gpu, ref


def compare(gpu, ref, names, tol, label):
    worst = {n: rel_linf(gpu.get(n), ref.get(n, double=False)) for n in names}
    bad = {k: v for k, v in worst.items() if not v <= tol}
    assert not bad, f"{label}: fields above {tol}: {bad}"
    return worst


@pytest.mark.parametrize("opt", SA_OPTS)
def test_sa_setup_call(mods, opt):
    """SPAL_LOSS as SETUP calls it (NSTEP = 1): the initial transported
    viscosity from FSTURB, the S-A viscosity of every cell, the source term
    (relaxation 1), the wall and face stresses and the body forces."""
    cd, gpu, ref = sa_pair(mods, opt)
    compare(gpu, ref, FORCES + ["VISC_RAT", "VISC_LAM", "VISC_TURB", "TRANS_DYN_VIS", "TRANS_KVIS", "T_SOURCE"],
            1e-5, f"SPAL_LOSS setup ({opt})")
    assert np.abs(gpu.get("T_SOURCE")).max() > 0.0
    assert gpu.get("TRANS_DYN_VIS").max() > 0.0


@pytest.mark.parametrize("opt", SA_OPTS)
def test_sa_one_step(mods, opt):
    """One step: the transported viscosity's fluxes, its TSTEP (flux sum,
    SCREE, multigrid, damping, cell update, mixing-plane transfer, residual
    smoothing, periodic and mixing-plane averages), its floor, and the inlet
    value, beside the five conserved variables."""
    cd, gpu, ref = sa_pair(mods, opt)
    gpu.step()
    ref.step()
    compare(gpu, ref, STATE + SA_FIELDS, 1e-5, f"S-A step 1 ({opt})")


@pytest.mark.parametrize("opt", SA_OPTS)
def test_sa_ten_steps(mods, opt):
    """Ten steps with SPAL_LOSS on steps 5 and 10 (every step with NLOS=1)."""
    cd, gpu, ref = sa_pair(mods, opt)
    for _ in range(10):
        gpu.step()
        ref.step()
    compare(gpu, ref, STATE + FORCES + SA_FIELDS + ["VISC_RAT"], 1e-4, f"S-A ten steps ({opt})")


def test_sa_long_run(mods):
    """300 steps with the reader's defaults: within 1e-3 of the oracle."""
    cd, gpu, ref = sa_pair(mods, "defaults")
    gpu.run(300)
    for _ in range(300):
        mr = ref.step()
    compare(gpu, ref, ["RO", "ROVX", "ROE", "TRANS_DYN_VIS", "XFORCE"], 1e-3, "S-A 300 steps")
    assert mr.econt < 1.0


def test_sa_stage_config_reference_order(mods):
    """The single-stage turbine at full size (65 x 242 x 49) with the S-A
    model: SETUP's call and one step in the reference's summation order
    (REDUCE_ORDER=1) within 1e-5."""
    case, common_setup, lib, O = mods
    spec = case.turbine_stage()
    spec.ilos = 200
    cd = common_setup.build_common(spec)
    cd.ints["REDUCE_ORDER"] = 1
    gpu = lib.Problem(cd)
    ref = O.Oracle(cd)
    ref.setup_calls()
    compare(gpu, ref, ["TRANS_DYN_VIS", "T_SOURCE", "VISC_RAT", "XFORCE", "TFORCE"], 1e-5, "stage S-A setup")
    gpu.step()
    ref.step()
    compare(gpu, ref, ["RO", "ROVX", "ROE", "TRANS_DYN_VIS", "TRANS_KVIS"], 1e-5, "stage S-A step 1")


def test_sa_restart_carries_the_transported_viscosity(mods, tmp_path):
    """flow_out's seventh array is TRANS_DYN_VIS with the S-A model, and a
    restart reads it back (OUTPUT 5966-5972, SETUP 6934)."""
    case, common_setup, lib, O = mods
    cd, gpu, ref = sa_pair(mods, "defaults")
    gpu.run(10)
    path = str(tmp_path / "flow_out")
    gpu.write_flow_out(path)
    tdv = gpu.get("TRANS_DYN_VIS")
    cd2 = common_setup.build_common(sa_spec(case, "defaults"))
    cd2.ints["IF_RESTART"] = 1
    g2 = lib.Problem(cd2, setup_calls=False, restart=path)
    assert np.array_equal(g2.get("TRANS_DYN_VIS"), tdv)
    g2.close()
    gpu.close()
