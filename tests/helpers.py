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


def read_flow_out(path: str, n: int, dtype=np.float32):
    """(NSTEP, [8 arrays]) of a flow_out file: gfortran sequential unformatted
    records, each payload between two 4-byte byte counts."""
    raw = open(path, "rb").read()
    pos, recs = 0, []
    while pos < len(raw):
        m = int(np.frombuffer(raw, np.int32, 1, pos)[0])
        body = raw[pos + 4: pos + 4 + m]
        assert int(np.frombuffer(raw, np.int32, 1, pos + 4 + m)[0]) == m, "record markers differ"
        recs.append(body)
        pos += m + 8
    assert len(recs) == 9 and len(recs[0]) == 4, [len(r) for r in recs]
    nstep = int(np.frombuffer(recs[0], np.int32)[0])
    arrays = [np.frombuffer(r, dtype).copy() for r in recs[1:]]
    assert all(a.size == n for a in arrays)
    return nstep, arrays
