"""Generates the regression fixture small_stage_10steps.npz: the FP32
oracle's state after SETUP's calls and 10 LOOP iterations on the seeded
small stage case.  The reference ships no outputs, so this fixture pins the
oracle against itself (a guard against accidental changes), not against the
reference.  Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "multall-open-18.3_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from mgpu import case, common_setup  # noqa: E402
import oracle as O  # noqa: E402


def main():
    cd = common_setup.build_common(case.small_stage())
    o = O.Oracle(cd)
    o.setup_calls()
    for _ in range(10):
        o.step()
    out = {n: o.get(n, double=False) for n in ("RO", "ROVX", "ROVR", "RORVT", "ROE", "XFORCE", "STEP")}
    np.savez_compressed(os.path.join(HERE, "small_stage_10steps.npz"), **out)


if __name__ == "__main__":
    main()
