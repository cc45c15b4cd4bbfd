"""The Stagen restatement (mgpu.stagen) against the reference's own data:
the blade sections generated from the reference's Stagen sample inputs
equal, to the printed precision, the sections of the MULTALL test-case decks
the reference ships for them (tests/golden/stagen, made by
make_stagen_fixtures.py), and every generated deck reads back through
mgpu.deck with the sections it was written with."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "stagen")

# the decks print F10.6: half a unit in the sixth decimal, plus the float32
# rounding of values up to ~2 and of the REAL*4 transcendentals
TOL = 1.5e-6

INPUTS = sorted(f[:-5] for f in os.listdir(GOLD) if f.endswith(".json")) if os.path.isdir(GOLD) else []
PAIRED = [n for n in INPUTS if os.path.exists(os.path.join(GOLD, n + "_deck.npz"))]


def _input(name):
    from mgpu import stagen
    return stagen.input_from_dict(json.load(open(os.path.join(GOLD, name + ".json"))))


@pytest.mark.parametrize("name", PAIRED)
def test_generated_sections_equal_the_reference_decks(name):
    from mgpu import stagen
    inp = _input(name)
    ref = np.load(os.path.join(GOLD, name + "_deck.npz"))
    tol = TOL
    worst = 0.0
    n = 0
    for nr, row in enumerate(inp.rows, start=1):
        g = stagen.generate_row(row, inp.km)
        assert g.jm == row.nintup + row.ninton + 1 + row.nintdn
        for ns in range(1, len(row.sections) + 1):
            for key in ("x", "y", "tk", "r"):
                mine = getattr(g, key)[ns - 1]
                theirs = ref[f"{key}_{nr}_{ns}"]
                assert mine.shape == theirs.shape
                worst = max(worst, float(np.max(np.abs(mine.astype(np.float64) - theirs))))
                n += 1
    assert n == 4 * sum(len(r.sections) for r in inp.rows)
    assert worst <= tol, f"{name}: max |generated - deck| = {worst:.3e}"


@pytest.mark.parametrize("name", INPUTS)
def test_written_deck_reads_back(name):
    """write_deck prints every generated section to the deck's precision,
    and mgpu.deck reads the deck back with the rows and grid it describes."""
    from mgpu import deck, stagen
    inp = _input(name)
    text = stagen.write_deck(inp)
    jms = [r.nintup + r.ninton + 1 + r.nintdn for r in inp.rows]
    printed = stagen.deck_sections(text, jms)
    assert len(printed) == sum(len(r.sections) for r in inp.rows)
    for nr, row in enumerate(inp.rows, start=1):
        g = stagen.generate_row(row, inp.km)
        for ns in range(1, len(row.sections) + 1):
            for q, key in enumerate(("x", "y", "tk", "r")):
                want = getattr(g, key)[ns - 1].astype(np.float64)
                assert np.max(np.abs(printed[(nr, ns)][q] - want)) <= 6e-7
    spec, geo = deck.read_deck(text)
    assert geo.im == inp.im and geo.km == inp.km
    assert geo.jm == sum(jms)
    assert [r.nblade for r in spec.rows] == [r.nblade for r in inp.rows]
    assert [r.jm for r in spec.rows] == jms


def test_deck_header_follows_stagen_defaults():
    from mgpu import deck, stagen
    inp = _input("stagen-single-stg-turbine")
    spec, geo = deck.read_deck(stagen.write_deck(inp, CFL=0.35, NMAX=1234))
    assert spec.cfl == pytest.approx(0.35)
    assert spec.nsteps_max == 1234
    assert spec.ilos == 10
    assert spec.cp == pytest.approx(287.5 * 1.4 / 0.4, rel=1e-6)
    with pytest.raises(stagen.StagenError):
        stagen.write_deck(inp, NOT_A_VARIABLE=1)


def test_interpolation_helpers():
    from mgpu import stagen
    f32 = np.float32
    x = np.array([0, 0, 1, 2, 3, 4], f32)
    y = np.array([0, 0, 1, 8, 27, 64], f32)       # x**3: the 4-point Lagrange form is exact
    assert stagen.intp(5, x, y, f32(1.5)) == pytest.approx(3.375, rel=1e-6)
    assert stagen.intp(5, x, y, f32(3.5)) == pytest.approx(42.875, rel=1e-6)
    assert stagen.linint(5, x, y, f32(1.5)) == pytest.approx(4.5)
    assert stagen.linint(5, x, y, f32(5.0)) == pytest.approx(101.0)   # extrapolated from the last interval
    assert stagen.linint(5, x, y, f32(-1.0)) == pytest.approx(-1.0)   # and from the first
    sp = stagen.pitch_spacing(9, 1.25, 1.5)
    assert list(sp) == pytest.approx([1.0, 1.25, 1.5, 1.5, 1.5, 1.5, 1.25, 1.0])


# a one-row vane of this test's own, with Stagen's control-variable block
# (IFDEF = 1), in Stagen's input layout
SYNTHETIC_IFDEF = """287.5  1.4               RGAS, GAMMA
 37  37                  IM, KM
 1.25  20.0              FPRAT, FPMAX
 1.25  20.0              FRRAT, FRMAX
 1                       IFDEF
 4000  500               NMAX, NCHANGE
 0 0 2 1 3 0 1 0 10 5 0 1 0 2
 3 3 3 9 9 9 1 3 1 1 0
 0 0 0 0
 0 0 3 0 0 0
 1005.0 1.4 0.45 0.006 0.006 0.8 2.0
 10.0 0.4 0.2 0.1 0.0 0.001 0.5
 1 0.025 1.0 0.8 0.8 10 10
 1.0 0.5 1000.0 800000.0 1.0 0.5 0.0001 0.0 5.0 25.0
 0.0 1.0 1.0 1.0 1.0 2.0 0.0 0.0
 0.05 0.05 0.03 0.02 0.03 0.03 0.04
 1  2                    NROWS, NOSECT
 1.0                     scale
blank
 VANE ROW
blank
 20  60  20
 0.0    1.0
 0.5    1.2
 1.001  1.0
 50
 0.0  100000.  100000.  90000.  90000.
 0  0  10  70  10  70  0.0  0.0
blank
 HUB SECTION
blank
 1
 5  200  2
 0.0    0.0
 0.25  10.0
 0.5   25.0
 0.75  40.0
 1.0   55.0
 0.02  0.01  0.10  0.40  0.05  0.02  2.0
 0.0  0.0  1.0
 0.0  0.5  0.5
 0.5  0.5  0.0  55.0
blank
 2
 -0.1  0.2
  0.5  0.5
 0.0  0.05  0.5  0.5
 0.0  0.0  0  0  0
 1.0  0
blank
 TIP SECTION
blank
 1
 5  200  2
 0.0    0.0
 0.25  12.0
 0.5   28.0
 0.75  44.0
 1.0   60.0
 0.02  0.01  0.08  0.40  0.05  0.02  2.0
 0.0  0.0  1.0
 0.0  0.5  0.5
 0.5  0.5  0.0  60.0
blank
 2
 -0.1  0.2
  0.6  0.6
 0.0  0.05  0.6  0.6
 1.0  0.0  0  0  0
 1.0  0
blank
 95000.  95000.  90000.  90000.
blank
 2
 0.0  1.0
 100000.  100000.
 300.  300.
 0.0  0.0
 100.  100.
 0.0  0.0
 0.0  0.0
"""


def test_control_block_input():
    """IFDEF != 0: the control cards are read by name, the deck carries
    them, and the variables the block does not set are zero (Stagen skips
    its defaults then)."""
    from mgpu import deck, stagen
    inp = stagen.read_stagen(SYNTHETIC_IFDEF)
    assert inp.controls["NMAX"] == 4000 and inp.controls["ILOS"] == 10
    assert inp.controls["CFL"] == pytest.approx(0.45) and inp.controls["TURBVIS_LIM"] == pytest.approx(1000.0)
    g = stagen.generate_row(inp.rows[0], inp.km)
    assert (g.jm, g.jle, g.jte) == (101, 21, 81)
    assert np.all(np.isfinite(np.concatenate(g.x + g.y + g.tk + g.r)))
    assert g.tk[0].max() == pytest.approx(0.05 * 0.10, rel=0.01)    # TKMAX of the axial chord x its length
    text = stagen.write_deck(inp)
    spec, geo = deck.read_deck(text)
    assert spec.nsteps_max == 4000 and spec.cfl == pytest.approx(0.45) and spec.cp == pytest.approx(1005.0)
    assert geo.jm == 101 and spec.ilos == 10
    assert "FACTOR TO INCREASE" in text and text.rstrip().endswith("0")   # FACMIXUP, NMIXUP left at zero


def test_unsupported_inputs_are_refused():
    from mgpu import stagen
    with pytest.raises(stagen.StagenError):
        stagen.read_stagen("287.5 1.4\n37 2\n1.2 5\n1.2 5\n0\n1 2\n1.0\n")
    with pytest.raises(stagen.StagenError):
        stagen.read_stagen("287.5 1.4\n37 37\n1.2 5\n1.2 5\n1\n")      # the control block ends early


def _turbine_section():
    from mgpu import stagen
    inp = _input("stagen-single-stg-turbine")
    return inp, inp.rows[0], inp.rows[0].sections[0]


def test_coordinate_input_reproduces_the_generated_section():
    """INTYPE 0 (blade coordinates read in) fed with the surface points an
    INTYPE 1 section generates gives the same section on the grid: the
    rescaling to unit axial chord is the only step between them."""
    import copy
    from mgpu import stagen
    inp, row, s1 = _turbine_section()
    nin, xs, ys, _ = stagen._generated_surface(s1)
    s0 = copy.copy(s1)
    s0.intype = 0
    s0.xyin = (xs[:nin + 1].copy(), ys[:nin + 1].copy(), 0, 0)
    r1 = copy.copy(row)
    r1.sections = [s1]
    r0 = copy.copy(row)
    r0.sections = [s0]
    g1 = stagen.generate_row(r1, inp.km)
    g0 = stagen.generate_row(r0, inp.km)
    chord = float(g1.x[0][g1.jte - 1] - g1.x[0][g1.jle - 1])
    for key in ("x", "y", "tk", "r"):
        a, b = getattr(g0, key)[0], getattr(g1, key)[0]
        assert np.max(np.abs(a - b)) <= 1e-4 * chord, key


@pytest.mark.parametrize("intype", [2, 3])
def test_thickness_and_surface_slope_inputs(intype):
    """INTYPE 2 (camber slopes with thicknesses above and below) and INTYPE 3
    (the two surface slopes), on a turbine vane: a closed section whose
    tangential thickness peaks at TKMAX of the meridional chord (FTKSCALE = 1
    scales it there) and vanishes off the blade."""
    import copy
    from mgpu import stagen
    f32 = np.float32
    inp, row, s1 = _turbine_section()
    s = copy.copy(s1)
    s.intype = intype
    npin = len(s1.fracx) - 1
    x = s1.fracx[1:]
    half = f32(0.5) * np.sin(np.pi * x).astype(f32) * f32(0.1)       # a thickness shape; rescaled to TKMAX
    if intype == 2:
        s.tkh = stagen._tab(half)
        s.tkl = stagen._tab(half)
    else:
        slope = s1.slope[1:]
        dt = np.gradient(half.astype(np.float64), x.astype(np.float64)).astype(f32)
        s.slpup = stagen._tab(slope + dt)
        s.slplow = stagen._tab(slope - dt)
        s.slope = np.zeros(npin + 1, f32)
    s.fchord = (f32(0.0), f32(0.0), f32(1.0))
    r = copy.copy(row)
    r.sections = [s]
    g = stagen.generate_row(r, inp.km)
    tk = g.tk[0]
    assert np.all(np.isfinite(np.concatenate([g.x[0], g.y[0], tk, g.r[0]])))
    chord = float(g.x[0][g.jte - 1] - g.x[0][g.jle - 1])
    # the 4-point interpolation onto the grid may undershoot zero at the
    # rounded trailing edge by a few millionths of the chord, as Stagen's does
    assert np.all(tk >= -1e-4 * chord)
    assert np.all(tk[:g.jle - 1] == 0.0) and np.all(tk[g.jte + 1:] == 0.0)
    tkmax = float(s.thick[2])
    assert tk.max() == pytest.approx(tkmax * chord, rel=0.05)


@pytest.mark.parametrize("name", ["stagen-single-stg-turbine", "stagen-18.1-intype=4-test"])
def test_written_deck_steps_in_the_oracle(name):
    """Stagen input -> deck -> the test-side SETUP -> five oracle steps: a
    finite, positive density field and a falling residual."""
    import oracle as O
    from mgpu import common_setup, deck, stagen
    inp = _input(name)
    spec, geo = deck.read_deck(stagen.write_deck(inp))
    cd = common_setup.build_common(spec, geo)
    ref = O.Oracle(cd)
    ref.setup_calls()
    for _ in range(5):
        m = ref.step()
    ro = ref.get("RO", double=False)
    assert np.all(np.isfinite(ro)) and ro.min() > 0.0
    assert np.isfinite(m.eavg) and m.eavg > 0.0


def test_command_line_writes_the_deck(tmp_path):
    """python -m mgpu.stagen input -o deck: the deck write_deck gives."""
    from mgpu import stagen
    src = tmp_path / "stagen.dat"
    src.write_text(SYNTHETIC_IFDEF)
    out = tmp_path / "stage_new.dat"
    assert stagen.main([str(src), "-o", str(out)]) == 0
    assert out.read_text() == stagen.write_deck(stagen.read_stagen(SYNTHETIC_IFDEF))
    spec, geo = stagen.case_from_input(stagen.read_stagen(SYNTHETIC_IFDEF))
    assert geo.jm == 101
