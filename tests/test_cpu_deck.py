"""The deck reader (mgpu.deck: NEW_READIN's cards, the grid of the gaps
between rows, INPINT and NEW_INTPOL) and the fixtures it made from the
reference's own input decks.  CPU only."""
import glob
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "decks", "*.npz")))
DECK_DIR = "/root/reference/Multall-open-18.3/multall-test-cases"


@pytest.fixture(scope="module")
def deck():
    from mgpu import deck
    return deck


def test_intp_is_the_four_point_lagrange_interpolant(deck):
    """INTP (7801-7872) reproduces a cubic from any four neighbouring table
    points, and is linear through two points."""
    f32 = np.float32
    xs = np.array([0, 0.0, 0.1, 0.25, 0.45, 0.6, 0.8, 1.0], f32)     # 1-based
    ys = (f32(2.0) * xs ** 3 - xs ** 2 + f32(0.5) * xs + f32(3.0)).astype(f32)
    for x in (0.05, 0.3, 0.5, 0.71, 0.99, 1.2, -0.1):
        want = 2 * x ** 3 - x ** 2 + 0.5 * x + 3
        assert abs(float(deck.intp(7, xs, ys, f32(x))) - want) < 2e-5
    assert float(deck.intp(2, np.array([0, 1.0, 3.0], f32), np.array([0, 2.0, 6.0], f32), f32(2.5))) == 5.0


@pytest.mark.parametrize("n,total,first", [(20, 0.05, 0.001), (15, 0.01, 0.002), (30, 0.2, 0.0005)])
def test_solve_gives_the_progression_that_fills_the_gap(deck, n, total, first):
    """SOLVE (9513-9540): n intervals growing by the returned ratio from the
    first one add up to the gap."""
    rat = float(deck.solve(n, np.float32(total), np.float32(first)))
    s = first * (rat ** n - 1.0) / (rat - 1.0)
    assert abs(s - total) / total < 1e-3


def test_reader_refuses_options_outside_the_path(deck):
    text = " TITLE\n CP GA\n -1.0 1.4\n"
    with pytest.raises(deck.DeckError, match="real-gas"):
        deck.read_deck(text)
    with pytest.raises(deck.DeckError, match="ends early"):
        deck.read_deck(" TITLE\n CP GA\n 1005.0 1.4\n ITIMST\n")


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_fixture_matches_its_deck(deck, path):
    """Each committed fixture is what the reader makes of the reference's
    deck today, bit for bit (skipped where the decks are not present)."""
    src = os.path.join(DECK_DIR, os.path.basename(path)[:-4] + ".dat")
    if not os.path.exists(src):
        pytest.skip("the reference's decks are not on this machine")
    spec, geo = deck.read_deck_file(src)
    s2, g2 = deck.load_fixture(path)
    for k in deck._GEO_ARRAYS:
        assert np.array_equal(getattr(geo, k), getattr(g2, k)), k
    for k in spec.inlet:
        assert np.array_equal(spec.inlet[k], s2.inlet[k]), k
    assert [r.jm for r in spec.rows] == [r.jm for r in s2.rows]
    assert spec.ilos == s2.ilos and spec.reyno == s2.reyno and spec.cfl == s2.cfl


def test_single_stage_turbine_deck_geometry():
    """The reference's single-stage turbine (46 x 282 x 46): rows of 141 J
    points with the leading and trailing edges where the deck puts them, the
    hub at r = 0.5 m, the mixing plane's two J planes 1 % of a spacing apart
    (GRID_UP 9465), and the section of row 1's inlet along the deck's -35
    degree yaw."""
    from mgpu import deck
    spec, geo = deck.load_fixture(os.path.join(HERE, "golden", "decks", "Single-stage-turbine-17.1.npz"))
    assert (geo.im, geo.jm, geo.km) == (46, 282, 46)
    assert [(r.jm, r.jle, r.jte, r.nblade) for r in spec.rows] == [(141, 26, 126, 71), (141, 16, 116, 83)]
    assert abs(float(geo.r[0, 0]) - 0.5) < 1e-6
    assert np.all(np.diff(geo.x, axis=1) > 0.0)            # x increases along every stream surface
    gap = geo.x[:, 141] - geo.x[:, 140]
    assert np.all(gap > 0.0) and np.all(gap < 0.02 * (geo.x[:, 142] - geo.x[:, 141]) + 1e-7)
    assert np.all(spec.inlet["BS"] == np.float32(-35.0))
    assert np.all(geo.rt_thick[:, :25] == 0.0) and np.all(geo.rt_thick[:, 126:156] == 0.0)


@pytest.mark.parametrize("name", ["Single-stage-turbine-17.1", "Shock-test-17.1", "r37+samods-17.5"])
def test_oracle_steps_a_deck(name):
    """The COMMON state built from a deck fixture commits in the oracle and
    steps: the monitors after 5 steps are finite (the end test of step 5 has
    run) and the mass flow is positive."""
    from mgpu import common_setup, deck
    import oracle as O
    spec, geo = deck.load_fixture(os.path.join(HERE, "golden", "decks", name + ".npz"))
    cd = common_setup.build_common(spec, geo)
    o = O.Oracle(cd)
    o.setup_calls()
    for _ in range(5):
        m = o.step()
    assert np.isfinite([m.eavg, m.emax, m.econt]).all() and m.eavg > 0.0
    assert o.integrals().mass_flow_in > 0.0
    o.close()
