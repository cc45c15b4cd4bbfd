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


@pytest.mark.parametrize("which", ["small_nozzle", "small_stage"])
def test_transposed_step_matches_oracle_reverse(mods, which):
    case, common_setup, lib, O = mods
    cd = _stepped(mods, getattr(case, which)())
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
