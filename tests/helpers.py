"""Shared helpers for the parity tests."""
import numpy as np

# the arrays one LOOP iteration updates and the tests compare
STATE = ["RO", "ROVX", "ROVR", "RORVT", "ROE", "P", "HO", "T_STATIC", "VX", "VR", "VT", "WT", "PEFF",
         "DRO", "DROE", "DROVX", "DROVR", "DRORVT", "STEP", "RSTEP"]
FORCES = ["XFORCE", "RFORCE", "TFORCE", "QSOURCE", "Y_PLUS"]


def rel_linf(a: np.ndarray, b: np.ndarray) -> float:
    """max |a-b| / max |b|: the per-field L-infinity relative difference."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.max(np.abs(b))
    if scale == 0.0:
        return float(np.max(np.abs(a - b)))
    return float(np.max(np.abs(a - b)) / scale)
