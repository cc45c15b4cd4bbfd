"""The discrete adjoint on the GPU against the oracle's reverse mode.

The transposed step (mgpu_adjoint_iterate with no objective) maps output
adjoints of one frozen step to input adjoints; the oracle instantiated with
its tape type gives the same product exactly, in double precision, for the
same linearisation state.  The GPU's reverse kernels work in FP32 with
atomic scatters, so agreement is to FP32 rounding of the adjoint chain."""
import numpy as np
import pytest

from helpers import rel_linf

pytestmark = pytest.mark.gpu

# the state arrays the adjoint carries between steps, and the parts of them
# that are state (the rest are recomputed every step)
ADJ_STATE = ["RO", "ROVX", "ROVR", "RORVT", "ROE", "DRO", "DROE", "DROVX", "DROVR", "DRORVT", "PEFF", "P", "HO",
             "ROVT", "PD"]


def _state_mask(name, cd):
    shape = cd.arrays[name].shape
    m = np.ones(shape, bool)
    if name in ("P", "ROVT"):
        m[:] = False
        m[:, 0, :] = True        # J = 1
    if name == "HO":
        m[:] = False
        m[:, -1, :] = True       # J = JM
    return m


@pytest.fixture(scope="module")
def mods():
    from mgpu import case, common_setup, lib
    import oracle as O
    O.build()
    lib.load()
    return case, common_setup, lib, O


def _stepped(mods, spec, nsteps=30):
    """A deck advanced nsteps by the float oracle (a developing flow), frozen."""
    case, common_setup, lib, O = mods
    cd = common_setup.build_common(spec)
    of = O.Oracle(cd)
    of.setup_calls()
    for _ in range(nsteps):
        of.step()
    for n, a in list(cd.arrays.items()):
        if a.dtype == np.float32:
            cd.arrays[n] = of.get(n, double=False).astype(np.float32)
    cd.ints["NSTEP"] = nsteps
    cd.ints["FROZEN"] = 1
    return cd


def _medium_stage(case):
    """33 x 122 x 25: the stage's multigrid blocks (3 and 9), leading-edge
    smoothing and a multi-point tip gap, small enough for the oracle's tape."""
    spec = case.turbine_stage(im=33, jm_row=61, km=25, seed=5)
    spec.name = "medium_stage_33x122x25"
    return spec


@pytest.mark.parametrize("which", ["small_nozzle", "small_stage", "medium_stage"])
def test_transposed_step_matches_oracle_reverse(mods, which):
    case, common_setup, lib, O = mods
    spec = _medium_stage(case) if which == "medium_stage" else getattr(case, which)()
    cd = _stepped(mods, spec, nsteps=30 if which != "medium_stage" else 20)
    rng = np.random.default_rng(7)
    seeds = {}
    for n in ADJ_STATE:
        w = rng.standard_normal(cd.arrays[n].shape) * _state_mask(n, cd)
        seeds[n] = w
    oa = O.Oracle(cd, ad=True)
    oa.ad_begin()
    oa.step()
    oa.ad_reverse(seeds)
    gp = lib.Problem(cd, setup_calls=False)
    gp.adjoint_prepare()
    gp.adjoint_objective("none")
    for n in ADJ_STATE:
        gp.adjoint_set(n, seeds[n].astype(np.float32))
    gp.adjoint_iterate(1)
    worst = {}
    for n in ADJ_STATE:
        ref = oa.ad_grad(n) * _state_mask(n, cd)
        got = gp.adjoint_get(n) * _state_mask(n, cd)
        worst[n] = rel_linf(got, ref)
    bad = {n: e for n, e in worst.items() if e > 1e-3}
    assert not bad, f"{which}: {bad} (all: {worst})"


def _restart(cd, state, frozen=1):
    """The converged problem restarted with LOSS and STEPUP held: NSTEP set
    so that the first step re-forms the final smoothing ramp values."""
    import copy
    c = copy.copy(cd)
    c.arrays, c.ints, c.reals = dict(cd.arrays), dict(cd.ints), dict(cd.reals)
    c.arrays.update(state)
    c.ints["NSTEP"] = cd.ints["NCHANGE"] - 1
    c.ints["FROZEN"] = frozen
    return c


def _state(p, cd):
    return {n: p.get(n) for n, a in cd.arrays.items() if a.dtype == np.float32}


@pytest.fixture(scope="module")
def converged_small_stage(mods):
    """The small stage with SFXIN = SFTIN = 0.02 converged with LOSS (EAVG at
    its FP32 floor, ~6e-6), then 2000 frozen steps."""
    case, common_setup, lib, O = mods
    from mgpu import design

    def make():
        sp = case.small_stage()
        sp.sfxin = sp.sftin = 0.02
        return sp

    ds = design.DesignSpace.seeded(make)
    cd = ds.deck(ds.alpha0)
    cd.ints["NSTEPS_MAX"] = 10 ** 9
    cd.reals["CONLIM"] = 1e-9
    p = lib.Problem(cd)
    p.run(3000)
    st = _state(p, cd)
    p.close()
    cdf = _restart(cd, st)
    pf = lib.Problem(cdf, setup_calls=False)
    _, m = pf.run(2000)
    assert m.eavg < 2e-5
    return ds, cdf, pf, _state(pf, cdf)


def test_adjoint_gradient_matches_frozen_finite_differences(mods, converged_small_stage):
    """dJ/d(alpha) of eta_tt and of the inlet mass flow from the adjoint
    (fixed-point iteration) against central differences of the frozen
    primal restarted from the converged state with the perturbed geometry
    (h = 0.2 degree, 3000 steps), for a stagger and an exit-angle variable
    of each row: within 3 % (the finite differences' own noise), and the
    GMRES solve gives the same gradient within 1 %."""
    case, common_setup, lib, O = mods
    from mgpu import design
    ds, cdf, pf, stf = converged_small_stage
    alpha = ds.alpha0
    sens = ds.sensitivities(alpha)
    g64 = ds.geometry64(alpha)
    grads, kgrads = {}, {}
    for obj in ("eta_tt", "mass_flow_in"):
        pf.adjoint_prepare()
        pf.adjoint_objective(obj)
        for _ in range(8):
            pf.adjoint_iterate(1000)
        grads[obj] = ds.chain(pf.adjoint_gradient(), sens)
        pf.adjoint_prepare()
        pf.adjoint_objective(obj)
        ok, steps, res = pf.adjoint_solve_krylov(inner=50, restart=30, max_steps=6000, tol=1e-6)
        kgrads[obj] = ds.chain(pf.adjoint_gradient(), sens)
    h = 0.2
    for i in (ds.index(0, "stagger", 0), ds.index(0, "exit", 2), ds.index(1, "stagger", 2), ds.index(1, "exit", 2)):
        js = []
        for sgn in (1.0, -1.0):
            a = alpha.copy()
            a[i] += sgn * h
            gp = ds.geometry64(a)
            cdp = design.perturbed_state(cdf, stf, {n: gp[n] - g64[n] for n in design.GEOM})
            pp = lib.Problem(cdp, setup_calls=False)
            pp.run(3000)
            r = pp.integrals()
            js.append((r.eta_tt, r.mass_flow_in))
            pp.close()
        fd = {"eta_tt": (js[0][0] - js[1][0]) / (2 * h), "mass_flow_in": (js[0][1] - js[1][1]) / (2 * h)}
        for obj in fd:
            adj = grads[obj][i]
            assert abs(adj - fd[obj]) <= 0.03 * abs(fd[obj]), (ds.names()[i], obj, adj, fd[obj])
            assert abs(kgrads[obj][i] - adj) <= 0.01 * abs(adj), (ds.names()[i], obj, kgrads[obj][i], adj)


def test_autograd_wrapper_returns_the_adjoint_gradient(mods):
    """The torch.autograd.Function of the check harness: backward() delivers
    the adjoint gradient of the objective the forward pass computed."""
    torch = pytest.importorskip("torch")
    case = mods[0]
    from mgpu import design
    from mgpu.autograd import AdjointObjective, DesignSolve

    def make():
        sp = case.small_stage()
        sp.sfxin = sp.sftin = 0.02
        return sp

    ds = design.DesignSpace.seeded(make)
    solver = DesignSolve(ds, steps=3000, adjoint_iters=8000)
    alpha = torch.tensor(ds.alpha0, dtype=torch.float64, requires_grad=True)
    eta = AdjointObjective.apply(alpha, solver, "eta_tt")
    eta.backward()
    value, grad = solver.last
    assert abs(float(eta) - value) < 1e-12
    assert np.allclose(alpha.grad.numpy(), grad)
    assert np.abs(grad).max() > 0.0


def test_theta_gradient_matches_metric_chain(mods):
    """dJ/dTHETA from the transposed SETUP metrics on the device, chained
    with the generator's dTHETA/d(alpha), gives the design gradient that
    dJ/dA chained with the metrics' dA/d(alpha) gives (small stage, with a
    mixing plane and a tip gap)."""
    case, common_setup, lib, O = mods
    from mgpu import design
    ds = design.DesignSpace.seeded(case.small_stage)
    alpha = ds.alpha0
    p = lib.Problem(ds.deck(alpha))
    p.run(60)
    p.adjoint_prepare()
    p.adjoint_objective("eta_tt")
    p.adjoint_iterate(20)
    ga = ds.chain(p.adjoint_gradient(), ds.sensitivities(alpha))
    gt = ds.chain_theta(p.adjoint_gradient_theta(), ds.theta_sensitivities(alpha))
    scale = float(np.max(np.abs(ga)))
    assert scale > 0.0
    assert float(np.max(np.abs(gt - ga))) <= 1e-3 * scale, (ga, gt)
