"""Generates tests/golden/stagen/: the reference's Stagen sample inputs
(Stagen-18.1/sample-stagen-data-sets/*.dat) parsed by mgpu.stagen and stored
as JSON, and, for each input whose deck the reference ships among its MULTALL
test cases (Multall-open-18.3/multall-test-cases), that deck's blade-section
arrays exactly as printed (X, R*THETA of the suction surface, the tangential
thickness and R for every section of every row).  The CPU tests generate the
sections from the JSON and compare them with these arrays, so they need no
copy of the reference at run time.

From the repository root, with the reference unpacked beside it:
    python tests/golden/make_stagen_fixtures.py /path/to/reference
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "multall-open-18.3_gb300"))

from mgpu import stagen  # noqa: E402

# Stagen input -> the MULTALL test-case deck written from it (None: no deck)
PAIRS = {
    "stagen-single-stg-turbine": "Single-stage-turbine-17.1",
    "stagen-4stg-turbine": "four-stg-turbine-17.1",
    "stagen-6stg-compr": "Six-stage-compr-17.1",
    "stagen-RI-turbine-from-meangen": "RI-turbine-from-meangen-17.1",
    "stagen-centr-compr-hispeed": "centr-compr-hispeed-17.1",
    "stagen-simple-axial-compr": "simple-axial-compr-17.1",
    "stagen-centrif-compr": "centrif-compr-17.1",
    "stagen-18.1-intype=4-test": None,
}


def main(ref):
    src = os.path.join(ref, "Stagen-18.1", "sample-stagen-data-sets")
    decks = os.path.join(ref, "Multall-open-18.3", "multall-test-cases")
    out = os.path.join(HERE, "stagen")
    os.makedirs(out, exist_ok=True)
    for name, deck_name in PAIRS.items():
        inp = stagen.read_stagen(open(os.path.join(src, name + ".dat")).read())
        with open(os.path.join(out, name + ".json"), "w") as f:
            json.dump(stagen.input_to_dict(inp), f, separators=(",", ":"))
        if deck_name is None:
            print(name, "(no deck)")
            continue
        jms = [r.nintup + r.ninton + 1 + r.nintdn for r in inp.rows]
        secs = stagen.deck_sections(open(os.path.join(decks, deck_name + ".dat")).read(), jms)
        arrays = {}
        for (nr, ns), (x, y, tk, r) in secs.items():
            for key, a in (("x", x), ("y", y), ("tk", tk), ("r", r)):
                arrays[f"{key}_{nr}_{ns}"] = a
        np.savez_compressed(os.path.join(out, name + "_deck.npz"), source=deck_name + ".dat", **arrays)
        print(name, "->", deck_name, len(secs), "sections")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
