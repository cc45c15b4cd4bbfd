"""GPU parity: the sm_103a library, called through its C ABI, against the
CPU oracle on the same seeded cases.

Tolerance (the stated bar for the plain FP32 path): after one step every
updated field agrees with the FP32 oracle to an L-infinity relative
difference <= 1e-5.  Residual differences come only from the order of the
long reductions (superblock multigrid sums and row averages in FP64 on the
GPU, sequential REAL*4 in the reference) and from the last-ulp differences of
CUDA's pow/asin/atan2/sin/cos against the host C library; every other
expression keeps the reference's evaluation order without FMA.
"""
import numpy as np
import pytest

from helpers import FORCES, STATE, rel_linf

pytestmark = pytest.mark.gpu

STEP1_TOL = 1e-5


@pytest.fixture(scope="module")
def mods():
    from mgpu import case, common_setup, lib
    import oracle as O
    lib.load()
    return case, common_setup, lib, O


def _pair(mods, spec, **over):
    case, common_setup, lib, O = mods
    cd = common_setup.build_common(spec)
    for k, v in over.items():
        if isinstance(v, int):
            cd.ints[k] = v
        else:
            cd.reals[k] = v
    gpu = lib.Problem(cd)
    ref = O.Oracle(cd)
    ref.setup_calls()
    return cd, gpu, ref


def _compare(gpu, ref, names, tol, label):
    worst = {}
    for n in names:
        g = gpu.get(n)
        r = ref.get(n, double=False)
        worst[n] = rel_linf(g, r)
    bad = {k: v for k, v in worst.items() if not (v <= tol)}
    assert not bad, f"{label}: fields above {tol}: {bad}"
    return worst


@pytest.mark.parametrize("which", ["small_nozzle", "small_stage"])
def test_setup_calls_match(mods, which):
    """STEPUP(1.0) and the first LOSS (SETUP's calls into the hot path)."""
    case = mods[0]
    cd, gpu, ref = _pair(mods, getattr(case, which)())
    _compare(gpu, ref, ["STEP", "RSTEP"] + FORCES, STEP1_TOL, "setup calls")


@pytest.mark.parametrize("which", ["small_nozzle", "small_stage"])
@pytest.mark.parametrize("order", [0, 2])
def test_one_step(mods, which, order):
    """One step against the FP32 oracle, on the default precision split
    (REDUCE_ORDER 0) and on the plain FP32 path (2)."""
    case = mods[0]
    cd, gpu, ref = _pair(mods, getattr(case, which)(), REDUCE_ORDER=order)
    gpu.step()
    ref.step()
    _compare(gpu, ref, STATE, STEP1_TOL, "step 1")


@pytest.mark.parametrize("which", ["small_nozzle", "small_stage"])
def test_five_steps_with_loss_and_tail(mods, which):
    """Step 5 runs LOSS, the monitors and STEPUP(0.25)."""
    case = mods[0]
    cd, gpu, ref = _pair(mods, getattr(case, which)())
    for _ in range(5):
        mg = gpu.step()
        mr = ref.step()
    assert mg.tail_ran == 1 and mr.tail_ran == 1
    _compare(gpu, ref, STATE + FORCES, 1e-4, "step 5")
    assert abs(mg.flow_in - mr.flow_in) <= 1e-5 * abs(mr.flow_in)
    assert abs(mg.econt - mr.econt) <= 1e-4
    assert abs(mg.vmax - mr.vmax) <= 1e-5 * mr.vmax
    assert (mg.ivmax, mg.jvmax, mg.kvmax) == (mr.ivmax, mr.jvmax, mr.kvmax)


@pytest.mark.parametrize("ypluswall", [-15.0, -10.0])
def test_pressure_gradient_wall_functions(mods, ypluswall):
    """YPLUSWALL <= -10: the Shih wall functions with the pressure-gradient
    term, DPDS_CELL from SET_PWALLGRAD when YPLUSWALL < -10 (at exactly -10
    the term runs on the stored DPDS_CELL, which WALLFUN raises to 1.0).
    After SETUP's LOSS every field is within 1e-5, after five steps (LOSS
    again at step 5) within 1e-4 of the FP32 oracle."""
    case, common_setup, lib, O = mods
    spec = case.small_stage()
    spec.ypluswall = ypluswall
    cd, gpu, ref = _pair(mods, spec)
    _compare(gpu, ref, FORCES + ["DPDS_CELL", "YPLUS_K1", "YPLUS_I1"], STEP1_TOL, "setup LOSS")
    for _ in range(5):
        gpu.step()
        ref.step()
    _compare(gpu, ref, STATE + FORCES + ["DPDS_CELL", "YPLUS_K1", "YPLUS_KM", "YPLUS_I1", "YPLUS_IM"], 1e-4,
             "step 5")


def _option_spec(case, opt):
    spec = case.small_stage()
    if opt == "ipout_minus1":
        spec.ipout = -1
    elif opt == "plate_loss":
        spec.plate_loss = 2.0
    elif opt == "setflo_mean":
        spec.in_flow, spec.rflow = 2, 0.05
    elif opt == "setflo_target":
        spec.in_flow, spec.rflow, spec.flowin = 3, 0.05, 12.0
    elif opt == "cusp2":
        for r in spec.rows:
            r.if_cusp, r.nup_i1, r.nup_im, r.n_wake, r.sep_thik, r.sep_drag = 2, 3, 3, 2, 0.2, 0.9
    return spec


@pytest.mark.parametrize("opt", ["ipout_minus1", "plate_loss", "setflo_mean", "setflo_target", "cusp2"])
def test_optional_branches(mods, opt):
    """The loop's optional branches: IPOUT=-1 (tip-pressure offset, with the
    K=1 exit update using the offset PD(1) before the next K resets it),
    the exit plate loss, SETFLO towards the mean flow (IN_FLOW=2) and
    towards FLOWIN (IN_FLOW=3), and the forced trailing-edge separation of
    IF_CUSP=2.  One step within 1e-5, five steps within 1e-4."""
    case = mods[0]
    cd, gpu, ref = _pair(mods, _option_spec(case, opt))
    gpu.step()
    ref.step()
    _compare(gpu, ref, STATE, STEP1_TOL, f"{opt} step 1")
    for _ in range(4):
        gpu.step()
        ref.step()
    _compare(gpu, ref, STATE + FORCES, 1e-4, f"{opt} step 5")


def test_throttle_exit(mods):
    """THROTTLE_EXIT: from step 101 the exit pressures follow the exit mass
    flow of the last tail (4488-4505).  After 120 steps PDOWN_HUB, PDOWN_TIP
    and THROTTLE_PRES agree with the FP32 oracle to 1e-5 and the flow field
    to 1e-3."""
    case = mods[0]
    spec = case.small_stage()
    spec.throttle_exit, spec.throttle_pres, spec.throttle_mas, spec.rfthrotl = 1.0, spec.pdown_hub, 14.08, 0.05
    cd, gpu, ref = _pair(mods, spec)
    gpu.run(120)
    for _ in range(120):
        ref.step()
    for n in ("PDOWN_HUB", "PDOWN_TIP", "THROTTLE_PRES"):
        g, r = gpu.get_real(n), ref.get_real(n)
        assert abs(g - r) <= 1e-5 * abs(r), (n, g, r)
    assert abs(ref.get_real("PDOWN_HUB") - spec.pdown_hub) > 100.0     # the throttle did move it
    _compare(gpu, ref, ["RO", "ROVX", "ROE", "P"], 1e-3, "throttle step 120")


def test_sss_scheme_one_step(mods):
    """ITIMST=-3 (SSS): F2/F3 history terms and SMOOTH_RESID."""
    case = mods[0]
    cd, gpu, ref = _pair(mods, case.small_stage(), NRSMTH=1, F2=-1.65, F3=-0.65)
    for _ in range(2):
        gpu.step()
        ref.step()
    _compare(gpu, ref, STATE, 1e-5, "SSS step 2")


def test_stage_config_one_step_reference_order(mods):
    """The single-stage turbine at its full size, 65 x 242 x 49, with the
    long sums in the reference's sequential REAL*4 order (REDUCE_ORDER=1):
    every field within 1e-5 of the FP32 oracle after one step."""
    case = mods[0]
    cd, gpu, ref = _pair(mods, case.turbine_stage(), REDUCE_ORDER=1)
    gpu.step()
    ref.step()
    _compare(gpu, ref, STATE, STEP1_TOL, "stage step 1 (reference order)")


def test_nozzle_config_one_step_reference_order(mods):
    """The single nozzle row at its full size, 37 x 97 x 33 (one row, JLE=18,
    JTE=74), long sums in reference order: every field within 1e-5."""
    case = mods[0]
    cd, gpu, ref = _pair(mods, case.nozzle_row(), REDUCE_ORDER=1)
    gpu.step()
    ref.step()
    _compare(gpu, ref, STATE, STEP1_TOL, "nozzle step 1 (reference order)")


@pytest.fixture(scope="module")
def compressor(mods):
    case, common_setup, lib, O = mods
    return common_setup.build_common(case.compressor_4stage())


def test_compressor_config_reference_order(mods, compressor):
    """The 4-stage compressor, 73 x 752 x 57, 8 rows with a mixing plane at
    every row interface, sums in reference order.  After one step every field
    is within 1e-5 of the FP32 oracle, or no farther from the FP64 oracle
    than the FP32 oracle itself is: at the low-speed inlet the velocity comes
    from 2*CP*(TO1 - TSTATIC) with TSTATIC = TO1*(P/PO1)**FGA, which turns the
    last-ulp difference between CUDA's powf and the host's into ~1e-5 of VX,
    the same size as the FP32 oracle's own error there.  After five steps
    (LOSS, tail, STEPUP) every field is within 1e-4 of the FP32 oracle."""
    case, common_setup, lib, O = mods
    cd = compressor
    cd.ints["REDUCE_ORDER"] = 1
    try:
        gpu = lib.Problem(cd)
        ref = O.Oracle(cd)
        ref.setup_calls()
        ref64 = O.Oracle(cd, double=True)
        ref64.setup_calls()
    finally:
        cd.ints["REDUCE_ORDER"] = 0
    gpu.step()
    ref.step()
    ref64.step()
    for n in STATE:
        g, r32, r64 = gpu.get(n), ref.get(n, double=False), ref64.get(n, double=True)
        e32 = rel_linf(g, r32)
        if e32 > STEP1_TOL:
            assert rel_linf(g, r64) <= 1.05 * rel_linf(r32, r64), (n, e32, rel_linf(g, r64), rel_linf(r32, r64))
    del ref64
    for _ in range(4):
        mg = gpu.step()
        mr = ref.step()
    assert mg.tail_ran == 1 and mr.tail_ran == 1
    _compare(gpu, ref, STATE + FORCES, 1e-4, "compressor step 5")
    assert abs(mg.flow_in - mr.flow_in) <= 1e-5 * abs(mr.flow_in)


def test_stage_config_one_step_fp64_sums(mods):
    """Default path (FP64 tree sums for the superblock and row-average
    reductions): against the FP64 oracle it is at least as close as the
    FP32 oracle is, field by field (the reference's 380k-term sequential
    REAL*4 sum of |change| is what separates the two FP32 results)."""
    case, common_setup, lib, O = mods
    cd, gpu, ref = _pair(mods, case.turbine_stage())
    ref64 = O.Oracle(cd, double=True)
    ref64.setup_calls()
    gpu.step()
    ref.step()
    ref64.step()
    for n in STATE:
        g, r32, r64 = gpu.get(n), ref.get(n), ref64.get(n)
        e_gpu, e_ref = rel_linf(g, r64), rel_linf(r32, r64)
        assert e_gpu <= max(1e-5, 1.05 * e_ref), (n, e_gpu, e_ref)


def test_converged_mass_flow_and_efficiency(mods):
    """Converged small stage: mass flow within 1e-4 relative, efficiency
    within 1e-4 absolute of the FP32 oracle run the same number of steps."""
    case = mods[0]
    cd, gpu, ref = _pair(mods, case.small_stage(), NCHANGE=200, NMIXUP=200)
    n = 1500
    rc, mg = gpu.run(n)
    for _ in range(n):
        mr = ref.step()
    ig, ir = gpu.integrals(), ref.integrals()
    assert mg.econt < 0.01 and mr.econt < 0.01
    assert abs(ig.mass_flow_in - ir.mass_flow_in) <= 1e-4 * abs(ir.mass_flow_in)
    assert abs(ig.eta_tt - ir.eta_tt) <= 1e-4


def test_precision_split_against_fp64_oracle(mods):
    """The reported quantities against the FP64 oracle after 1500 steps of
    the small stage: the default path (FP32 field arithmetic, FP64 for the
    multigrid, row-mean, mixing-plane, monitor and integral sums), the
    reference-order path (REDUCE_ORDER=1: the long sums sequential in
    REAL*4) and the plain FP32 path (REDUCE_ORDER=2: the default path's
    parallel trees with FP32 adds) all keep mass flow within 1e-4 relative
    and total-to-total efficiency within 1e-4 absolute."""
    case, common_setup, lib, O = mods
    spec = case.small_stage()
    cd = common_setup.build_common(spec)
    cd.ints.update(NCHANGE=200, NMIXUP=200)
    ref64 = O.Oracle(cd, double=True)
    ref64.setup_calls()
    n = 1500
    for _ in range(n):
        ref64.step()
    i64 = ref64.integrals()
    errs = {}
    for order in (0, 1, 2):
        cd.ints["REDUCE_ORDER"] = order
        gpu = lib.Problem(cd)
        gpu.run(n)
        ig = gpu.integrals()
        errs[order] = (abs(ig.mass_flow_in - i64.mass_flow_in) / abs(i64.mass_flow_in), abs(ig.eta_tt - i64.eta_tt))
        gpu.close()
    cd.ints["REDUCE_ORDER"] = 0
    print("mass-flow rel / eta abs error vs FP64 oracle: FP64 sums", errs[0], "reference order", errs[1],
          "plain FP32", errs[2])
    for order, (em, ee) in errs.items():
        assert em <= 1e-4 and ee <= 1e-4, (order, em, ee)


@pytest.mark.parametrize("limit", ["nsteps_max", "conlim"])
def test_run_stops_after_the_final_step(mods, limit):
    """mgpu_run stops right after the step on which IFEND is set, where LOOP
    stops: NSTEP reaching NSTEPS_MAX (12, between two tails) or the
    convergence test met at a tail (CONLIM=1e3, so ECONT < 0.01 decides; the
    oracle's ECONT is 0.0104 at the tail of step 340 and 0.0096 at 345, so
    step 346 is the final one).  The state is the oracle's after the same
    final step, and a further run returns at once without stepping."""
    case = mods[0]
    over, final, tol = ({"NSTEPS_MAX": 12}, 12, 1e-4) if limit == "nsteps_max" else ({"CONLIM": 1e3}, 346, 1e-3)
    cd, gpu, ref = _pair(mods, case.small_stage(), **over)
    rc, mg = gpu.run(1000)
    for _ in range(1000):
        mr = ref.step()
        if mr.ifend:
            break
    assert mr.nstep == final and mr.tail_ran == 1
    assert rc == 1 and mg.ifend == 1 and mg.tail_ran == 1 and mg.nstep == final
    _compare(gpu, ref, STATE, tol, f"final step {final}")
    ro = gpu.get("RO")
    rc2, m2 = gpu.run(10)
    assert rc2 == 1 and m2.nstep == final
    assert np.array_equal(gpu.get("RO"), ro)


def test_deterministic(mods):
    """Two runs of the same case are bitwise identical (no float atomics)."""
    case = mods[0]
    outs = []
    for _ in range(2):
        cd, gpu, ref = _pair(mods, case.small_stage())
        gpu.run(20)
        outs.append([gpu.get(n) for n in ("RO", "ROE", "ROVX")])
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("which", ["small_stage", "small_nozzle"])
@pytest.mark.parametrize("bs", [128, 192, 256, 512])
def test_pair_update_matches_single_plane_update(mods, which, bs):
    """TSTEP's damping and corner gather over pairs of J-planes (TS_PAIR=1,
    the default) give bitwise the state of the one-CTA-per-plane kernel
    (TS_PAIR=0) after 12 steps, at every CTA size.  The nozzle's JM = 29 is
    odd, so its last pair holds a single plane."""
    case, common_setup, lib, O = mods
    spec = getattr(case, which)()
    outs = []
    for pair in (0, 1):
        cd = common_setup.build_common(spec)
        cd.ints["TS_PAIR"] = pair
        cd.ints["TS_THREADS"] = bs
        gpu = lib.Problem(cd)
        gpu.run(12)
        outs.append([gpu.get(n) for n in ("RO", "ROE", "ROVX", "RORVT", "ROVR", "DRO", "DROE")])
        gpu.close()
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_batch_matches_members_stepped_alone(mods):
    """Three uneven problems in one batch graph: after 12 steps (two tails,
    two LOSS steps) every member's state is bitwise the state of the same
    problem stepped on its own, and the monitors agree."""
    case, common_setup, lib, O = mods
    specs = [case.small_stage(), case.small_nozzle(), case.small_stage(im=11, jm_row=21, km=9, seed=7)]
    cds = [common_setup.build_common(sp) for sp in specs]
    alone = [lib.Problem(cd) for cd in cds]
    for p in alone:
        p.run(12)
    members = [lib.Problem(cd) for cd in cds]
    batch = lib.Batch(members)
    ended, mons = batch.run(12)
    assert ended == 0
    for p, q, m in zip(alone, members, mons):
        assert m.nstep == 12
        for n in ("RO", "ROVX", "ROVR", "RORVT", "ROE", "DRO", "XFORCE", "STEP"):
            assert np.array_equal(p.get(n), q.get(n)), n
    batch.close()


def test_health_check_reports_nonfinite(mods):
    """A NaN planted in the host copy of RO comes back as MGPU_E_NONFINITE
    from the next tail step; the handle stays usable."""
    case, common_setup, lib, O = mods
    cd = common_setup.build_common(case.small_nozzle())
    gpu = lib.Problem(cd)
    ro = cd.arrays["RO"].copy()
    ro[2, 10, 3] = np.nan
    gpu.set("RO", ro)
    with pytest.raises(lib.MgpuError) as e:
        gpu.run(5)
    assert e.value.code == -5
    gpu.set("RO", cd.arrays["RO"])          # still usable afterwards
    assert gpu.get("RO").shape == cd.arrays["RO"].shape


def test_api_errors(mods):
    case, common_setup, lib, O = mods
    cd = common_setup.build_common(case.small_nozzle())
    gpu = lib.Problem(cd)
    with pytest.raises(lib.MgpuError) as e:
        gpu.set("RO", np.zeros(7, np.float32))
    assert e.value.code == -1
    with pytest.raises(lib.MgpuError):
        gpu.set("NOT_A_COMMON_NAME", np.zeros(7, np.float32))
    with pytest.raises(lib.MgpuError) as e:
        gpu.set("AQX", cd.arrays["AQX"])      # geometry is fixed after commit
    assert e.value.code == -2
    gpu.close()
    cd.ints["REDUCE_ORDER"] = 3                # 0, 1 and 2 are the only orders
    with pytest.raises(lib.MgpuError) as e:
        lib.Problem(cd)
    assert e.value.code == -1


@pytest.mark.parametrize("bs", [128, 192, 512])
def test_tstep_cta_sizes_match_oracle(mods, bs):
    """Every CTA size the autotuner can choose gives the oracle's step: the
    small stage after one step within 1e-5 and after five steps (LOSS and
    tail) within 1e-4, with TSTEP set to each size through TS_THREADS."""
    case, common_setup, lib, O = mods
    cd = common_setup.build_common(case.small_stage())
    probe = lib.Problem(cd)
    chosen, ms = probe.autotune()
    assert all(c in (128, 192, 256, 512) for c in chosen)
    assert all(m > 0 for p in ("2", "3") for m in ms[p])
    probe.close()
    cd.ints["TS_THREADS"] = bs
    gpu = lib.Problem(cd)
    ref = O.Oracle(cd)
    ref.setup_calls()
    for n in range(5):
        gpu.step()
        ref.step()
        if n == 0:
            for name in ("RO", "ROE", "ROVX", "RORVT", "ROVR"):
                assert rel_linf(gpu.get(name), ref.get(name)) <= 1e-5, (bs, name)
    for name in ("RO", "ROE", "ROVX", "RORVT", "ROVR"):
        assert rel_linf(gpu.get(name), ref.get(name)) <= 1e-4, (bs, name)


def test_handles_of_different_sizes_keep_their_launch_limits(mods):
    """A kernel's dynamic shared-memory limit is per function, not per
    handle: committing a small problem after a large one must not lower the
    limit the large one needs (k_bc_sums takes 49 KB at IM = 65).  Both
    step, alone and in one batch, with the large one's values the same
    either way."""
    case, common_setup, lib, O = mods
    big = common_setup.build_common(case.turbine_stage(im=65, jm_row=30, km=9, seed=6))
    small = common_setup.build_common(case.turbine_stage(im=33, jm_row=30, km=9, seed=7))
    pb = lib.Problem(big)
    ps = lib.Problem(small)
    pb.run(6)
    ps.run(6)
    alone = pb.get("RO").copy()
    pb2 = lib.Problem(big)
    ps2 = lib.Problem(small)
    b = lib.Batch([pb2, ps2])
    b.run(6)
    assert np.array_equal(pb2.get("RO"), alone)
    b.close()


def _new_loss_spec(case, opt):
    spec = case.small_stage()
    spec.ilos = 100
    if opt == "wall_functions":
        spec.ypluswall = -15.0
    elif opt == "reyno_temperature":
        spec.reyno = -4.0
    elif opt == "no_tip_gap":
        for r in spec.rows:
            r.tip_gap = 0.0
    return spec


NEW_LOSS_OPTS = ["log_law", "wall_functions", "reyno_temperature", "rough_transition", "ibound1", "no_tip_gap"]


def _new_loss_pair(mods, opt):
    case, common_setup, lib, O = mods
    cd = common_setup.build_common(_new_loss_spec(case, opt))
    if opt == "rough_transition":
        nr = cd.arrays["ROUGH_H"].size
        for n, v in (("ROUGH_H", 2e-5), ("ROUGH_T", 1e-5), ("ROUGH_L", 3e-5), ("ROUGH_U", 5e-6)):
            cd.arrays[n] = np.full(nr, v, np.float32)
        for n, v in (("JTRAN_I1", 8), ("JTRAN_IM", 12), ("JTRAN_K1", 4), ("JTRAN_KM", 20)):
            cd.arrays[n] = np.full(nr, v, np.int32)
        cd.reals["FTRANS"] = 2.0
    elif opt == "ibound1":
        cd.ints["IBOUND"] = 1
    gpu = lib.Problem(cd)
    ref = O.Oracle(cd)
    ref.setup_calls()
    return cd, gpu, ref


@pytest.mark.parametrize("opt", NEW_LOSS_OPTS)
def test_new_loss_setup_call(mods, opt):
    """NEW_LOSS (ILOS=100) as SETUP calls it: the eddy viscosity, the wall
    shear stresses (log law with roughness, or the Shih wall functions with
    the pressure-gradient term), transition, the stresses summed over the I
    and K faces, and the relaxed body forces, within 1e-5 of the FP32 oracle."""
    cd, gpu, ref = _new_loss_pair(mods, opt)
    _compare(gpu, ref, FORCES + ["VISC_RAT", "VISC_LAM", "ROAVG_CELL"], STEP1_TOL, f"NEW_LOSS setup ({opt})")
    if opt == "wall_functions":
        _compare(gpu, ref, ["YPLUS_I1", "YPLUS_IM", "YPLUS_K1", "YPLUS_KM", "DPDS_CELL"], STEP1_TOL, "wall functions")
    if opt == "rough_transition":
        v = gpu.get("VISC_RAT")
        assert np.count_nonzero(v == 1.0) > 0          # some lines were made laminar
    assert np.abs(gpu.get("XFORCE")).max() > 0.0


@pytest.mark.parametrize("opt", NEW_LOSS_OPTS)
def test_new_loss_ten_steps(mods, opt):
    """Ten steps with NEW_LOSS on steps 5 and 10 and the cell-average
    density formed after TSTEP(RO) on every step: state, forces, viscosity
    ratios and ROAVG_CELL within 1e-4 of the FP32 oracle."""
    cd, gpu, ref = _new_loss_pair(mods, opt)
    for _ in range(10):
        mg = gpu.step()
        ref.step()
    assert mg.tail_ran == 1
    _compare(gpu, ref, STATE + FORCES + ["VISC_RAT", "VISC_LAM", "ROAVG_CELL"], 1e-4, f"NEW_LOSS step 10 ({opt})")


def test_new_loss_long_run(mods):
    """300 steps of the small stage under NEW_LOSS through the graph
    (mgpu_run): the flow field within 1e-3 and the mass flow within 1e-4 of
    the FP32 oracle."""
    cd, gpu, ref = _new_loss_pair(mods, "log_law")
    gpu.run(300)
    for _ in range(300):
        mr = ref.step()
    _compare(gpu, ref, ["RO", "ROVX", "ROE", "P", "VISC_RAT"], 1e-3, "NEW_LOSS step 300")
    ig, ir = gpu.integrals(), ref.integrals()
    assert abs(ig.mass_flow_in - ir.mass_flow_in) <= 1e-4 * abs(ir.mass_flow_in)


def test_new_loss_stage_config_setup_call(mods):
    """NEW_LOSS at the single-stage turbine's full size, 65 x 242 x 49, with
    the long sums in the reference's sequential REAL*4 order (REDUCE_ORDER=1,
    as the other full-size parity tests): SETUP's call and then one step
    within 1e-5 of the FP32 oracle."""
    case, common_setup, lib, O = mods
    spec = case.turbine_stage()
    spec.ilos = 100
    cd = common_setup.build_common(spec)
    cd.ints["REDUCE_ORDER"] = 1
    gpu = lib.Problem(cd)
    ref = O.Oracle(cd)
    ref.setup_calls()
    _compare(gpu, ref, FORCES + ["VISC_RAT", "VISC_LAM"], STEP1_TOL, "stage NEW_LOSS setup")
    gpu.step()
    ref.step()
    _compare(gpu, ref, STATE + ["ROAVG_CELL"], STEP1_TOL, "stage NEW_LOSS step 1")
    gpu.close()
