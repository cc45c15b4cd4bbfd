"""CPU tests: the oracle's own invariants, the host-side setup, and the C
ABI library's symbol table (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from helpers import rel_linf


@pytest.fixture(scope="module")
def mods():
    from mgpu import case, common_setup
    import oracle as O
    O.build()
    return case, common_setup, O


def test_setup_geometry_closes(mods):
    """Face areas close each cell: the divergence of a constant field is
    zero in x (the reference checks this, commented out, at
    multall-open-18.3.f:6727-6733).  The mixing-plane cell J=JMIX+1 is
    excluded: its upstream faces use the theta extrapolated from the next
    row (TEMP1, multall-open-18.3.f:3025-3035), so it does not close."""
    case, common_setup, O = mods
    cd = common_setup.build_common(case.small_stage())
    a = cd.arrays
    K, J, I = cd.km, cd.jm, cd.im
    xarea = (a["AQX"][:K - 1, 1:, :I - 1] - a["AQX"][:K - 1, :-1, :I - 1] + a["ABX"][:K - 1, 1:, :I - 1]
             - a["ABX"][:K - 1, 1:, 1:] + a["ASX"][:K - 1, 1:, :I - 1] - a["ASX"][1:, 1:, :I - 1])
    scale = np.abs(a["AQX"]).max()
    for jmix in a["JMIX"][:-1]:
        xarea[:, int(jmix) + 1 - 2, :] = 0.0
    assert np.abs(xarea).max() <= 1e-4 * scale
    assert (a["VOL"][:K - 1, 1:, :I - 1] > 0).all()


def test_oracle_float_vs_double_one_step(mods):
    """REAL*4 and REAL*8 restatements agree to 1e-4 after one step (the
    FP32 rounding of cancelling face fluxes, not a code difference)."""
    case, common_setup, O = mods
    cd = common_setup.build_common(case.small_stage())
    of, od = O.Oracle(cd), O.Oracle(cd, double=True)
    of.setup_calls()
    od.setup_calls()
    of.step()
    od.step()
    for n in ("RO", "ROE", "ROVX", "RORVT", "ROVR"):
        assert rel_linf(of.get(n), od.get(n)) < 1e-4, n


def test_oracle_pressure_gradient_wall_functions(mods):
    """YPLUSWALL < -10 (SET_PWALLGRAD + Shih with the pressure term): REAL*4
    and REAL*8 agree to 1e-4 over ten steps (two LOSS calls), DPDS_CELL is
    set on the cells and stays within the DPDS_LIM bound."""
    case, common_setup, O = mods
    spec = case.small_stage()
    spec.ypluswall = -15.0
    cd = common_setup.build_common(spec)
    of, od = O.Oracle(cd), O.Oracle(cd, double=True)
    of.setup_calls()
    od.setup_calls()
    for _ in range(10):
        of.step()
        od.step()
    for n in ("RO", "ROE", "ROVX", "XFORCE", "TFORCE"):
        assert rel_linf(of.get(n), od.get(n)) < 1e-4, n
    dp = of.get("DPDS_CELL")
    nr = cd.nrows
    lim = abs(20.0 * (cd.arrays["PO1"][cd.km // 2 - 1] - 0.5 * (cd.reals["PDOWN_HUB"] + cd.reals["PDOWN_TIP"]) / nr /
                      (cd.arrays["CHORD"][0] + cd.arrays["CHORD"][nr - 1])))
    assert np.count_nonzero(dp) > 0 and np.abs(dp).max() <= lim * (1 + 1e-6)


def test_oracle_periodic_and_mixing_plane(mods):
    """After a step, non-blade J-planes are periodic (D(1)=D(IM)) and the
    two faces of the mixing plane are pitchwise uniform.  The exit plane
    J=JM is excluded: the exit condition, applied after TSTEP, rebuilds it
    from HO(JM-1) of the step's start (multall-open-18.3.f:4701-4728)."""
    case, common_setup, O = mods
    cd = common_setup.build_common(case.small_stage())
    o = O.Oracle(cd)
    o.setup_calls()
    o.step()
    ro = o.get("RO", double=False)
    ind = cd.arrays["IND"]
    indle = cd.arrays["INDLE"]
    for j in range(cd.jm - 1):
        if ind[j] != 1 and indle[j] != 1:
            assert np.array_equal(ro[:, j, 0], ro[:, j, -1]), j
    jmix = int(cd.arrays["JMIX"][0])
    for jj in (jmix, jmix + 1):
        plane = ro[:, jj - 1, :]
        assert np.all(plane == plane[:, :1])


def test_oracle_converges(mods):
    """The small stage converges: continuity error below 1 % and the
    residual EAVG falls by orders of magnitude."""
    case, common_setup, O = mods
    cd = common_setup.build_common(case.small_stage())
    cd.ints["NCHANGE"] = 200
    cd.ints["NMIXUP"] = 200
    o = O.Oracle(cd)
    o.setup_calls()
    first = None
    for n in range(1500):
        m = o.step()
        if m.tail_ran and first is None:
            first = m.eavg
    assert m.econt < 0.01
    assert m.eavg < 0.01 * first
    it = o.integrals()
    assert 0.5 < it.eta_tt < 1.0


def test_oracle_rejects_uncovered_options(mods):
    case, common_setup, O = mods
    cd = common_setup.build_common(case.small_nozzle())
    cd.ints["IFGAS"] = 1
    with pytest.raises(O.OracleError):
        O.Oracle(cd)


def test_golden_regression(mods):
    """The oracle reproduces the committed fixture (tests/golden, made by
    tests/golden/make_golden.py) bit for bit: a guard against unintended
    changes to the restatement."""
    case, common_setup, O = mods
    path = os.path.join(os.path.dirname(__file__), "golden", "small_stage_10steps.npz")
    g = np.load(path)
    cd = common_setup.build_common(case.small_stage())
    o = O.Oracle(cd)
    o.setup_calls()
    for _ in range(10):
        o.step()
    for n in g.files:
        assert np.array_equal(o.get(n, double=False), g[n]), n


def test_golden_regression_new_loss(mods):
    """The same guard for NEW_LOSS (ILOS=100): ten steps of the small stage
    reproduce tests/golden/small_stage_newloss_10steps.npz bit for bit."""
    case, common_setup, O = mods
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "small_stage_newloss_10steps.npz"))
    spec = case.small_stage()
    spec.ilos = 100
    o = O.Oracle(common_setup.build_common(spec))
    o.setup_calls()
    for _ in range(10):
        o.step()
    for n in g.files:
        assert np.array_equal(o.get(n, double=False), g[n]), n


def test_abi_library_exports_every_declared_symbol():
    """libmgpu.so loads without a GPU and exports each function
    include/mgpu.h declares."""
    from mgpu import build, lib
    path = build.build()
    L = ctypes.CDLL(path)
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "mgpu.h")).read()
    declared = set(re.findall(r"\b(mgpu_[a-z0-9_]+)\s*\(", hdr))
    assert declared == set(lib.EXPORTS)
    for name in declared:
        assert hasattr(L, name), name
    assert L.mgpu_abi_version() == 1


def test_gloo_two_ranks_shard_instances():
    """Batched instances shard across ranks with no data-path collective:
    each of two gloo ranks steps its own instance on the CPU oracle and the
    ranks only gather the per-instance node counts."""
    import torch.multiprocessing as mp
    mp.spawn(_rank_main, args=(2,), nprocs=2, join=True)


def _rank_main(rank, world):
    import os
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "..", "multall-open-18.3_gb300"))
    sys.path.insert(0, os.path.join(here, "..", "oracle"))
    import torch
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    os.environ.setdefault("MASTER_PORT", "29533")
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from mgpu import case, common_setup
    import oracle as O
    spec = case.small_stage(seed=10 + rank)
    cd = common_setup.build_common(spec)
    o = O.Oracle(cd)
    o.setup_calls()
    for _ in range(5):
        m = o.step()
    t = torch.tensor([float(cd.nodes()), float(m.flow_in)])
    out = [torch.zeros(2) for _ in range(world)]
    dist.all_gather(out, t)
    assert all(x[0] > 0 for x in out)
    dist.destroy_process_group()


def test_oracle_reverse_mode_matches_finite_differences(mods):
    """The oracle's tape (reverse mode over one frozen step, the checker of
    the GPU adjoint) against central differences of the double oracle: the
    dot-product identity w . (G(x+ev) - G(x-ev)) / 2e = (G'^T w) . v holds
    to 1e-7 on a developing stage flow."""
    case, common_setup, O = mods
    cd = common_setup.build_common(case.small_stage())
    of = O.Oracle(cd)
    of.setup_calls()
    for _ in range(20):
        of.step()
    for n, a in list(cd.arrays.items()):
        if a.dtype == np.float32:
            cd.arrays[n] = of.get(n, double=False).astype(np.float32)
    cd.ints["NSTEP"] = 20
    cd.ints["FROZEN"] = 1
    names = ["RO", "ROVX", "ROVR", "RORVT", "ROE", "DRO", "DROE", "DROVX", "DROVR", "DRORVT", "P", "HO",
             "ROVT", "PEFF", "PD"]
    rng = np.random.default_rng(3)
    w = {n: rng.standard_normal(cd.arrays[n].shape) for n in names}
    v = {n: rng.standard_normal(cd.arrays[n].shape) * float(np.abs(cd.arrays[n]).mean()) for n in names}
    oa = O.Oracle(cd, ad=True)
    oa.ad_begin()
    oa.step()
    oa.ad_reverse(w)
    rhs = sum(float(np.sum(oa.ad_grad(n) * v[n])) for n in names)
    eps = 1e-6
    out = []
    for sgn in (1.0, -1.0):
        od = O.Oracle(cd, double=True)
        for n in names:
            od.set_f64(n, cd.arrays[n].astype(np.float64) + sgn * eps * v[n])
        od.step()
        out.append({n: od.get(n) for n in names})
    lhs = sum(float(np.sum(w[n] * (out[0][n] - out[1][n]))) for n in names) / (2 * eps)
    assert abs(lhs - rhs) <= 1e-7 * abs(rhs), (lhs, rhs)


def test_design_space_and_geometry_sensitivities(mods):
    """The 30 blade-angle design variables of the adjoint configuration:
    the double-precision metrics agree with the REAL*4 deck, a zero offset
    leaves the deck bitwise unchanged, every variable moves the blade-wise
    areas of its own row only, and the chain rule is linear."""
    case, common_setup, O = mods
    from mgpu import design
    ds = design.DesignSpace.seeded(case.small_stage)
    assert ds.size == 30 and len(ds.names()) == 30
    base = common_setup.build_common(case.small_stage())
    zero = common_setup.build_common(ds.spec(np.zeros(ds.size)))
    for n in ("AQX", "ABX", "VOLOR", "RO", "STEP"):
        assert np.array_equal(base.arrays[n], zero.arrays[n]), n
    cd = ds.deck(ds.alpha0)
    g64 = ds.geometry64(ds.alpha0)
    for n in ("AQX", "ABX", "ABR", "VOLOR"):
        scale = np.abs(g64[n]).max()
        assert np.abs(cd.arrays[n] - g64[n]).max() <= 1e-5 * scale, n
    sens = ds.sensitivities(ds.alpha0)
    j_row2 = int(cd.arrays["JSTART"][1])
    i_row1 = ds.index(0, "stagger", 2)
    own = np.abs(sens[i_row1]["ABX"][:, :j_row2 - 2, :]).max()
    assert own > 0.0
    assert np.abs(sens[i_row1]["ABX"][:, j_row2 + 1:, :]).max() <= 1e-9 * own
    rng = np.random.default_rng(0)
    g1 = {n: rng.standard_normal(g64[n].shape) for n in design.GEOM}
    g2 = {n: 2.0 * g1[n] for n in design.GEOM}
    c1, c2 = ds.chain(g1, sens), ds.chain(g2, sens)
    assert np.allclose(c2, 2.0 * c1)


def test_flow_out_and_restart_follow_the_reference(mods, tmp_path):
    """OUTPUT's flow_out (multall-open-18.3.f:5942-5978) from the FP32
    oracle: nine gfortran records holding NSTEP and the eight fields, with
    DPDS_CELL*1.0E-6 and PEFF+PREFF formed in REAL*4.  Read back as SETUP's
    IF_RESTART branch does (6920-6992): the secondary variables, PEFF = P and
    the shifted exit pressures PD, checked bitwise against the same REAL*4
    expressions in NumPy, and LOOP's prologue (PREFF) taken from the
    restarted pressures."""
    from helpers import read_flow_out
    case, common_setup, O = mods
    cd = common_setup.build_common(case.small_stage())
    ref = O.Oracle(cd)
    ref.setup_calls()
    for _ in range(3):
        ref.step()
    f = str(tmp_path / "flow_out")
    ref.write_flow_out(f)
    N = cd.nodes()
    nstep, (ro, rovx, rovr, rovt, roe, rosub, dpds, peff) = read_flow_out(f, N)
    g = lambda n: ref.get(n, double=False).ravel()
    assert nstep == 3
    for a, n in ((ro, "RO"), (rovx, "ROVX"), (rovr, "ROVR"), (rovt, "ROVT"), (roe, "ROE")):
        assert np.array_equal(a, g(n)), n
    assert np.array_equal(rosub, g("RO"))
    assert np.array_equal(dpds, g("DPDS_CELL") * np.float32(1.0e-6))
    P = g("P").reshape(cd.km, cd.jm, cd.im)
    imid, kmid = int(0.5 * cd.im), int(0.5 * cd.km)
    preff = np.float32(0.5) * (P[kmid - 1, 0, imid - 1] + P[kmid - 1, cd.jm - 1, imid - 1])
    assert np.array_equal(peff, g("PEFF") + preff)

    rs = O.Oracle(cd, restart=f)
    assert rs.restart_nstep == 3
    f32 = np.float32
    cp, ga = f32(cd.reals["CP"]), f32(cd.reals["GA"])
    cv = cp / ga
    rgas = cp - cv
    vx, vr, vt = rovx / ro, rovr / ro, rovt / ro
    eke = f32(0.5) * (vx * vx + vr * vr + vt * vt)
    ts = (roe / ro - eke) / cv
    p = ro * rgas * ts
    r = cd.arrays["R"].reshape(cd.km, cd.jm)[:, :, None]
    want = {"VX": vx, "VR": vr, "VT": vt, "T_STATIC": ts, "HO": cp * ts + eke, "P": p, "PEFF": p,
            "RORVT": (rovt.reshape(cd.km, cd.jm, cd.im) * r).ravel()}
    for n, w in want.items():
        assert np.array_equal(rs.get(n, double=False).ravel(), w), n
    # the exit pressures: PDOWN(K) in the reference's order, shifted by PD(1)
    pk = p.reshape(cd.km, cd.jm, cd.im)[:, cd.jm - 1, :]
    fp = cd.arrays["FP"].ravel()
    pdown = np.zeros(cd.km, np.float32)
    for k in range(cd.km):
        s = f32(0.0)
        for i in range(cd.im - 1):
            s = f32(s + fp[i] * f32(0.5) * (pk[k, i] + pk[k, i + 1]))
        pdown[k] = s
    assert cd.ints["IPOUT"] == 0
    pd = pdown + (cd.arrays["PD"].ravel()[0] - pdown[0])
    assert np.array_equal(rs.get("PD", double=False).ravel(), pd)
    pr = p.reshape(cd.km, cd.jm, cd.im)
    assert rs.get_real("PREFF") == float(f32(0.5) * (pr[kmid - 1, 0, imid - 1] + pr[kmid - 1, cd.jm - 1, imid - 1]))
    rs.setup_calls()
    rs.step()


def test_stage_table_stations_and_whole_machine(mods):
    """EFICOOL's stage table on a 4-stage compressor: the stations follow the
    reader's JSTG_START / JSTG_END (multall-open-18.3.f:1522-1536) and the
    stage loop (11269-11293); the whole-machine row is the integrals' one."""
    case, common_setup, O = mods
    cd = common_setup.build_common(case.compressor_4stage(im=9, jm_row=25, km=7))
    ns = cd.ints["NSTAGES"]
    nstage, jstart, jmix = (cd.arrays[n].ravel() for n in ("NSTAGE", "JSTART", "JMIX"))
    nrow = cd.arrays["NROW"].ravel()
    js, je = {1: 1}, {}
    for n in range(len(nstage)):
        s0 = int(nstage[n])
        s1 = int(nstage[n + 1]) if n + 1 < len(nstage) else ns + 1
        if s0 != s1:
            je[s0] = int(jmix[n])
            if s1 <= ns:
                js[s1] = int(jstart[n + 1])
    ref = O.Oracle(cd)
    ref.setup_calls()
    for _ in range(10):
        ref.step()
    for s in range(1, ns + 1):
        st = ref.stage(s)
        j2 = je[s] + 1
        assert (st.j1, st.j2m1, st.jmix, st.has_reaction) == (
            js[s], cd.jm - 1 if s == ns else j2, int(jmix[nrow[js[s]] - 1]), 1), s
    whole, ig = ref.stage(ns + 1), ref.integrals()
    assert (whole.j1, whole.j2m1, whole.has_reaction) == (ig.j1, ig.j2m1, 0) == (2, cd.jm - 1, 0)
    for f in ("mass_flow_in", "mass_flow_out", "eta_tt", "eta_ts", "po_ratio", "to_ratio"):
        assert getattr(whole, f) == getattr(ig, f), f
    with pytest.raises(O.OracleError):
        ref.stage(ns + 2)


def test_grid_out_follows_setup(mods, tmp_path):
    """SETUP's plotting file grid_out (multall-open-18.3.f:6585-6597) from the
    FP32 oracle: NSTEPS_MAX; IM, JM, KM; CP, GA; INDLETE; WRAD; NBLADE; then
    X, R and RTHETA(1..IM) per (J, K) with K fastest, each a gfortran record."""
    case, common_setup, O = mods
    cd = common_setup.build_common(case.small_stage())
    ref = O.Oracle(cd)
    f = str(tmp_path / "grid_out")
    ref.write_grid_out(f)
    raw = open(f, "rb").read()
    recs, pos = [], 0
    while pos < len(raw):
        m = int(np.frombuffer(raw, np.int32, 1, pos)[0])
        assert int(np.frombuffer(raw, np.int32, 1, pos + 4 + m)[0]) == m
        recs.append(raw[pos + 4: pos + 4 + m])
        pos += m + 8
    im, jm, km = cd.im, cd.jm, cd.km
    assert len(recs) == 6 + jm * km
    assert np.frombuffer(recs[0], np.int32)[0] == cd.ints["NSTEPS_MAX"]
    assert list(np.frombuffer(recs[1], np.int32)) == [im, jm, km]
    assert np.array_equal(np.frombuffer(recs[2], np.float32), np.float32([cd.reals["CP"], cd.reals["GA"]]))
    indlete = np.zeros(jm, np.int32)
    indlete[cd.arrays["INDLE"].ravel() == 1] = 1
    indlete[cd.arrays["JTE"].ravel() - 1] = 1
    assert np.array_equal(np.frombuffer(recs[3], np.int32), indlete)
    assert np.array_equal(np.frombuffer(recs[4], np.float32), cd.arrays["WRAD"].ravel())
    assert np.array_equal(np.frombuffer(recs[5], np.int32), cd.arrays["NBLADE"].ravel())
    X = cd.arrays["X"].reshape(km, jm)
    R = cd.arrays["R"].reshape(km, jm)
    RT = cd.arrays["RTHETA"].reshape(km, jm, im)
    for j in (0, jm // 2, jm - 1):
        for k in (0, km - 1):
            rec = np.frombuffer(recs[6 + j * km + k], np.float32)
            assert rec[0] == X[k, j] and rec[1] == R[k, j] and np.array_equal(rec[2:], RT[k, j])


def test_flow_out_of_another_grid_is_refused(mods, tmp_path):
    """A restart file of another grid is refused (the record lengths do not
    match), before anything of the new problem is changed."""
    case, common_setup, O = mods
    cd = common_setup.build_common(case.small_stage())
    ref = O.Oracle(cd)
    f = str(tmp_path / "flow_out")
    ref.write_flow_out(f)
    other = common_setup.build_common(case.small_nozzle())
    with pytest.raises(O.OracleError, match="not a flow_out file of this grid"):
        O.Oracle(other, restart=f)


def test_new_loss_oracle_float_vs_double(mods):
    """NEW_LOSS (ILOS=100) in the oracle: the mixing lengths SETUP derives
    are zero on the first cell of each row and FST_RAT stays within FSTURB;
    after SETUP's call and ten steps (NEW_LOSS on steps 5 and 10) the FP32
    restatement agrees with the FP64 one to 1e-4 on the state, forces and
    viscosity ratios."""
    case, common_setup, O = mods[0], mods[1], mods[2]
    spec = case.small_stage()
    spec.ilos = 100
    cd = common_setup.build_common(spec)
    JS = cd.arrays["JSTART"]
    for j0 in JS[1:]:
        assert not cd.arrays["XLENGTH"][:-1, j0 - 1, :-1].any()
    assert cd.arrays["FST_RAT"].max() <= 1.0 and cd.arrays["XLENGTH"].max() > 0.0
    assert cd.reals["VORT_MAX"] > 0.0
    of, od = O.Oracle(cd), O.Oracle(cd, double=True)
    of.setup_calls()
    od.setup_calls()
    for n in ("XFORCE", "QSOURCE", "VISC_RAT", "Y_PLUS"):
        assert rel_linf(of.get(n, double=False), od.get(n)) <= 1e-5, n
    for _ in range(10):
        of.step()
        od.step()
    for n in ("RO", "ROVX", "ROE", "XFORCE", "RFORCE", "TFORCE", "QSOURCE", "VISC_RAT", "ROAVG_CELL"):
        assert rel_linf(of.get(n, double=False), od.get(n)) <= 1e-4, n


def test_new_loss_inputs_are_required(mods):
    """ILOS 100-299 needs the SETUP-made mixing lengths and VORT_MAX, and
    ILOS 300 and above is refused as not covered, as mgpu_commit does."""
    case, common_setup, O = mods[0], mods[1], mods[2]
    spec = case.small_nozzle()
    spec.ilos = 100
    cd = common_setup.build_common(spec)
    bad = common_setup.build_common(spec)
    del bad.arrays["XLENGTH"]
    with pytest.raises(O.OracleError, match="XLENGTH"):
        O.Oracle(bad)
    bad = common_setup.build_common(spec)
    bad.reals["VORT_MAX"] = 0.0
    with pytest.raises(O.OracleError, match="VORT_MAX"):
        O.Oracle(bad)
    cd.ints["ILOS"] = 300
    with pytest.raises(O.OracleError, match="ILOS"):
        O.Oracle(cd)


@pytest.mark.parametrize("branch", ["density_limiter", "mach_limiter", "supersonic_mixing_plane"])
def test_branch_cases_make_the_oracle_take_each_branch(mods, branch):
    """The inputs of the GPU branch tests make the oracle take the density
    limiter, the Mach limiter and the Prandtl-Meyer sweep on step 1."""
    from helpers import BRANCH_CASES
    case, common_setup, O = mods
    make, counter = BRANCH_CASES[branch]
    o = O.Oracle(make(case, common_setup))
    o.setup_calls()
    o.step()
    assert o.get_int(counter) > 0
    assert O.Oracle(common_setup.build_common(case.small_stage())).get_int(counter) == 0
    o.close()


def test_gloo_two_ranks_run_the_bench_replica_logic():
    """bench.py's multi-rank path on two gloo ranks with the GPU calls
    stubbed: each rank sees only its own GPU (CUDA_VISIBLE_DEVICES = its
    local rank), marches its own instance (here the CPU oracle, timed on the
    host), and both report the slowest rank's time and the whole-job
    throughput; the reference arm does no work on rank 1."""
    import torch.multiprocessing as mp
    mp.spawn(_bench_rank_main, args=(2,), nprocs=2, join=True)


def _bench_rank_main(rank, world):
    import os
    import sys
    import time
    here = os.path.dirname(os.path.abspath(__file__))
    for p in ("..", os.path.join("..", "multall-open-18.3_gb300"), os.path.join("..", "oracle")):
        sys.path.insert(0, os.path.join(here, p))
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT="29547")
    import torch
    import bench
    from mgpu import case, common_setup
    import oracle as O
    dist = bench.replica_setup(world, rank, rank)
    assert os.environ["CUDA_VISIBLE_DEVICES"] == str(rank)
    cd = common_setup.build_common(case.small_stage(seed=20 + rank))
    o = O.Oracle(cd)
    o.setup_calls()
    bench.dist_barrier(dist)
    t0 = time.perf_counter()
    for _ in range(2 + 3 * rank):          # rank 1 is the slow one
        o.step()
    ms = (time.perf_counter() - t0) * 1e3
    ms_max, value = bench.replica_value(dist, world, cd.nodes(), 5, ms)
    both = [torch.zeros(2, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(both, torch.tensor([ms, ms_max], dtype=torch.float64))
    assert all(abs(b[1].item() - max(x[0].item() for x in both)) < 1e-9 for b in both)
    assert abs(value - cd.nodes() * 5 * world / (ms_max / 1e3) / 1e9) < 1e-12
    if rank == 1:
        class A:
            steps, warmup, gpus = 1, 1, world
        assert bench.run_reference(A, rank, world) == 0
    o.close()
    dist.destroy_process_group()


def test_sa_oracle_float_vs_double(mods):
    """The Spalart-Allmaras restatement (SPAL_LOSS, the transported viscosity
    and TSTEP's NCALL = 2 branch): the FP32 instance stays within 1e-4 of the
    FP64 one over 20 steps (SPAL_LOSS on steps 5, 10, 15, 20), and the
    transported viscosity of every cell is positive."""
    case, common_setup, O = mods
    sp = case.small_stage()
    sp.ilos = 200
    cd = common_setup.build_common(sp)
    outs = []
    for dbl in (False, True):
        o = O.Oracle(cd, double=dbl)
        o.setup_calls()
        for _ in range(20):
            o.step()
        outs.append({n: o.get(n) for n in ("RO", "ROVX", "ROE", "TRANS_DYN_VIS", "T_SOURCE", "XFORCE")})
        tdv = o.get("TRANS_DYN_VIS")[:-1, 1:, :-1]          # the cells
        assert tdv.min() > 0.0
        o.close()
    for n in outs[0]:
        assert rel_linf(outs[0][n], outs[1][n]) <= 1e-4, n


def test_sa_oracle_flow_out_round_trip(mods, tmp_path):
    """With ILOS >= 200 the oracle's flow_out carries TRANS_DYN_VIS as its
    seventh array and a restart reads it back (5966-5972, 6934)."""
    case, common_setup, O = mods
    sp = case.small_stage()
    sp.ilos = 200
    cd = common_setup.build_common(sp)
    o = O.Oracle(cd)
    o.setup_calls()
    for _ in range(6):
        o.step()
    path = str(tmp_path / "flow_out")
    o.write_flow_out(path)
    tdv = o.get("TRANS_DYN_VIS", double=False)
    cd.ints["IF_RESTART"] = 1
    o2 = O.Oracle(cd, restart=path)
    assert np.array_equal(o2.get("TRANS_DYN_VIS", double=False), tdv)
    o.close()
    o2.close()
