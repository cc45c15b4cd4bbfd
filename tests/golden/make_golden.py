"""Generates the regression fixtures small_stage_10steps.npz and
small_stage_newloss_10steps.npz: the FP32 oracle's state after SETUP's calls
and 10 LOOP iterations on the seeded small stage case, with LOSS (ILOS=10)
and with NEW_LOSS (ILOS=100).  The reference ships no outputs, so this fixture pins the
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


def run(ilos, names, fname):
    spec = case.small_stage()
    spec.ilos = ilos
    o = O.Oracle(common_setup.build_common(spec))
    o.setup_calls()
    for _ in range(10):
        o.step()
    np.savez_compressed(os.path.join(HERE, fname), **{n: o.get(n, double=False) for n in names})


def main():
    run(10, ("RO", "ROVX", "ROVR", "RORVT", "ROE", "XFORCE", "STEP"), "small_stage_10steps.npz")
    run(100, NEW_LOSS_FIELDS, "small_stage_newloss_10steps.npz")


NEW_LOSS_FIELDS = ("RO", "ROVX", "ROE", "XFORCE", "TFORCE", "QSOURCE", "VISC_RAT", "Y_PLUS")


if __name__ == "__main__":
    main()
