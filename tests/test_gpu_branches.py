"""GPU parity on the loop's branches that the configured cases never take:
the density limiter's sequential J walk (multall-open-18.3.f:5115-5122), the
Mach limiter (5127-5168) and NEW_MIXPLAN's Prandtl-Meyer sweep for a
supersonic relative flow at the mixing plane (15151-15173).

Each case is built so that the branch fires (tests/helpers.py).  Every test
first reads the oracle's counter of the branch for each step and requires it
to be non-zero, then compares the library, called through its C ABI, with
the FP32 oracle: every state field within 1e-5 L-infinity relative after one
step and within 1e-4 after five, the bars of the other parity tests.
"""
import pytest

from helpers import BRANCH_CASES, STATE, rel_linf

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    from mgpu import case, common_setup, lib
    import oracle as O
    lib.load()
    return case, common_setup, lib, O


def _worst(gpu, ref):
    return {n: rel_linf(gpu.get(n), ref.get(n, double=False)) for n in STATE}


@pytest.mark.parametrize("branch", sorted(BRANCH_CASES))
def test_branch_fires_and_matches_oracle(mods, branch):
    case, common_setup, lib, O = mods
    make, counter = BRANCH_CASES[branch]
    cd = make(case, common_setup)
    gpu = lib.Problem(cd)
    ref = O.Oracle(cd)
    ref.setup_calls()
    fired = []
    for s in range(1, 6):
        gpu.step()
        ref.step()
        fired.append(ref.get_int(counter))
        if s == 1:
            assert fired[0] > 0, f"{branch}: the branch did not fire on step 1"
            w = _worst(gpu, ref)
            bad = {k: v for k, v in w.items() if not v <= 1e-5}
            assert not bad, f"{branch}, step 1: {bad}"
    w = _worst(gpu, ref)
    bad = {k: v for k, v in w.items() if not v <= 1e-4}
    assert not bad, f"{branch}, step 5: {bad} (branch counts {fired})"
    gpu.close()
    ref.close()


def test_run_without_multigrid(mods):
    """IR = JR = KR = 1 (and IRBB = JRBB = KRBB = 1): TSTEP skips the block
    restriction and its block changes stay zero (multall-open-18.3.f:5613,
    5490-5498).  One step within 1e-5 and ten steps within 1e-4 of the
    oracle, which takes the same branch."""
    case, common_setup, lib, O = mods
    spec = case.small_stage()
    spec.ir = spec.jr = spec.kr = 1
    spec.irbb = spec.jrbb = spec.krbb = 1
    cd = common_setup.build_common(spec)
    gpu = lib.Problem(cd)
    ref = O.Oracle(cd)
    ref.setup_calls()
    gpu.step()
    ref.step()
    for n in STATE:
        assert rel_linf(gpu.get(n), ref.get(n, double=False)) <= 1e-5, n
    for _ in range(9):
        gpu.step()
        ref.step()
    for n in ["RO", "ROVX", "ROVR", "RORVT", "ROE"]:
        assert rel_linf(gpu.get(n), ref.get(n, double=False)) <= 1e-4, n
