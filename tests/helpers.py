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


# ---- inputs that make the loop take branches the configured cases never take
def density_spike_case(case, common_setup):
    """The small stage with its initial density cut to 35 % on three
    consecutive J planes of one column and raised 2.5x on two planes of
    another: the density limiter (multall-open-18.3.f:5115-5122) changes
    values on the first steps, and the changes of one plane feed the
    4-plane average of the next, which exercises its sequential J walk."""
    cd = common_setup.build_common(case.small_stage())
    ro = cd.arrays["RO"]                 # (KM, JM, IM)
    for j in (10, 11, 12):
        ro[3, j - 1, 4] *= np.float32(0.35)
    for j in (30, 31):
        ro[2, j - 1, 2] *= np.float32(2.5)
    return cd


def mach_limit_case(case, common_setup):
    """The small stage with MACHLIM = 0.45, below the flow's relative Mach
    number: the Mach limiter (5127-5168) rescales the mass fluxes and raises
    densities to RO_LIMIT on every step."""
    cd = common_setup.build_common(case.small_stage())
    cd.reals["MACHLIM"] = 0.45
    return cd


def supersonic_mixing_plane_case(case, common_setup):
    """The small stage with its rotor turning backwards at 20000 rpm: the
    relative flow entering the rotor is supersonic across the pitch, so
    NEW_MIXPLAN takes its Prandtl-Meyer branch (15151-15173)."""
    sp = case.small_stage()
    sp.rows[1].rpm = sp.rows[1].rpm_hub = -20000.0
    return common_setup.build_common(sp)


BRANCH_CASES = {"density_limiter": (density_spike_case, "ORACLE_NDENS"),
                "mach_limiter": (mach_limit_case, "ORACLE_NMACH"),
                "supersonic_mixing_plane": (supersonic_mixing_plane_case, "ORACLE_NPM")}
