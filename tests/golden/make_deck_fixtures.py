"""Generates tests/golden/decks/*.npz from the reference's own input decks
(Multall-open-18.3/multall-test-cases/*.dat): each is the deck read by
mgpu.deck (the NEW_READIN subset with the grid of the gaps, INPINT and
NEW_INTPOL), stored as the float32 geometry and the cards that SETUP takes.
The GPU tests rebuild the COMMON state from these files, so they need no
copy of the reference at run time.

From the repository root, with the reference unpacked beside it:
    python tests/golden/make_deck_fixtures.py /path/to/Multall-open-18.3/multall-test-cases
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "multall-open-18.3_gb300"))

from mgpu import deck  # noqa: E402

# one deck per kind of input the path accepts: the mixing-length model on a
# stage (the reference's single-stage turbine), NEW_LOSS and Spalart-Allmaras
# on a transonic rotor with a tip gap, inviscid flow, a radial compressor,
# a transonic fan, a linear cascade and a twelve-row compressor
DECKS = [
    "Single-stage-turbine-17.1",
    "Six-stage-compr-17.1",
    "r37+samods-17.5",
    "Rotor-37-17.1",
    "Shock-test-17.1",
    "Staggered-wedge-exact-17.1",
    "Harrison-cascade-17.1",
    "centrif-compr-17.1",
    "Transonic-fan-rotor-17.1",
]


def main(src):
    out = os.path.join(HERE, "decks")
    os.makedirs(out, exist_ok=True)
    for name in DECKS:
        spec, geo = deck.read_deck_file(os.path.join(src, name + ".dat"))
        deck.save_fixture(os.path.join(out, name + ".npz"), spec, geo, source=name + ".dat")
        print(name, geo.im, geo.jm, geo.km)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else
         "/root/reference/Multall-open-18.3/multall-test-cases")
