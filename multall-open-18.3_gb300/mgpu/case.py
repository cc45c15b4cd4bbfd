"""Synthetic turbomachinery cases: the geometry and control data a Multall
input deck would carry, generated from seeded blade-section parameters.

The reference reads this data from an input deck (NEW_READIN,
multall-open-18.3.f:148-2161) and interpolates the blade sections onto the
KM stream surfaces (NEW_INTPOL, 7493-7613).  There is no public benchmark
suite behind the configurations this library is measured on, so the cases
are generated here instead: an H-mesh per blade row whose pitchwise lines
follow a circular-arc camber line (extended upstream / downstream along the
inlet / exit metal angle, as the reference's sheared H-meshes do), a
thickness distribution with given maximum, position and LE/TE values, and
seeded Gaussian per-section angle noise.  The generator produces directly
what the reader + NEW_INTPOL leave in COMMON: X(J,K), R(J,K), RT_UPP(J,K),
RT_THICK(J,K) plus the per-row cards.  The geometric series used for the
FP/FR spacings follows the reader's own rule (multall-open-18.3.f:1961-2028).

Arrays use numpy's C order with shape (KM, JM) for A(J,K), so that a flat
copy is the packed Fortran layout with J fastest.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Callable, List, Optional

import numpy as np

f32 = np.float32


@dataclasses.dataclass
class RowSpec:
    """One blade row, the reader's per-row cards (multall-open-18.3.f:792-1503)."""
    nblade: int
    jm: int                 # JMROW: streamwise points of this row
    jle: int                # JLEROW, row-relative (1-based)
    jte: int                # JTEROW, row-relative
    rpm: float = 0.0        # RPMROW
    rpm_hub: float = 0.0    # RPMHUB
    chi_in: float = 0.0     # metal angle at the leading edge, degrees
    chi_out: float = 70.0   # metal angle at the trailing edge, degrees
    tmax: float = 0.20      # max thickness / axial chord
    xtmax: float = 0.40     # chord fraction of max thickness
    tle: float = 0.015      # LE thickness / chord
    tte: float = 0.008      # TE thickness / chord
    chord: float = 0.04     # axial chord, m
    up_len: float = 0.04    # axial length upstream of the LE, m
    dn_len: float = 0.04    # axial length downstream of the TE, m
    tip_gap: float = 0.0    # tip clearance as a fraction of span (casing side)
    noise_deg: float = 0.5  # std-dev of per-section angle noise, degrees
    nsect: int = 5          # sections carrying independent noise
    pup: float = 0.0        # PUPROW, PLEROW, PTEROW, PDNROW (initial guess)
    ple: float = 0.0
    pte: float = 0.0
    pdn: float = 0.0
    stage: int = 1          # NSTAGE(NR)
    xllim: tuple = (0.03, 0.03, 0.03, 0.03, 0.03, 0.02)  # XLLIM_I1,IM,K1,KM,DWN,UP
    xllim_new: tuple = (0.03, 0.03, 0.03, 0.03)  # ILOS >= 100: XLLIM_IN,LE,TE,DN
    fsturb: float = 1.0     # ILOS >= 100: FSTURB, free-stream turbulent viscosity ratio
    turbvis_damp: float = 0.5   # ILOS >= 200: TURBVIS_DAMP, decay of the transported viscosity across a mixing plane
    # IF_CUSP = 2: forced trailing-edge separation (multall-open-18.3.f:987-1005)
    if_cusp: int = 0
    nup_i1: int = 0         # NUP_I1, NUP_IM: points before the TE where it starts
    nup_im: int = 0
    n_wake: int = 0         # N_WAKE: points into the wake
    sep_thik: float = 0.0   # SEP_THIK: fraction of the blade thickness
    sep_drag: float = 1.0   # SEP_DRAG: momentum factor in the separated region
    # design offsets (degrees) at the nsect span sections, interpolated across
    # the span like the noise: inlet and exit metal angle (pivot at the
    # leading edge) and stagger (all metal angles, pivot at mid-chord)
    d_in: tuple = ()
    d_out: tuple = ()
    d_stag: tuple = ()
    # JROTHS, JROTHE, JROTTS, JROTTE, row-relative (reader 940-960); None:
    # the hub rotates with the row over its whole length, the casing not
    jrot: Optional[tuple] = None
    jtran: tuple = (0, 0, 0, 0)     # JTRAN_I1, JTRAN_IM, JTRAN_K1, JTRAN_KM
    rough: tuple = (0.0, 0.0, 0.0, 0.0)   # ROUGH_H, ROUGH_T, ROUGH_L, ROUGH_U (m)


@dataclasses.dataclass
class CaseSpec:
    name: str
    im: int
    km: int
    rows: List[RowSpec]
    hub: Callable[[np.ndarray], np.ndarray]
    casing: Callable[[np.ndarray], np.ndarray]
    po1: float
    to1: float
    pdown_hub: float
    pdown_tip: float
    seed: int = 0
    cp: float = 1005.0
    ga: float = 1.4
    cfl: float = 0.4
    itimst: int = 3
    nsteps_max: int = 5000
    conlim: float = 0.001
    dampin: float = 10.0
    machlim: float = 2.0
    sfxin: float = 0.005
    sftin: float = 0.005
    fac_4th: float = 0.8
    nchange: int = 1000
    fp_ratio: float = 1.2       # geometric ratio of pitchwise spacing
    fp_max: float = 20.0
    fr_ratio: float = 1.2
    fr_max: float = 20.0
    ir: int = 3
    jr: int = 3
    kr: int = 3
    irbb: int = 9
    jrbb: int = 9
    krbb: int = 9
    fblk: tuple = (0.4, 0.2, 0.1)
    ifmix: int = 1
    rfmix: float = 0.025
    fextrap: float = 0.8
    fsmthb: float = 1.0
    fangle: float = 0.8
    rfin: float = 0.25
    ipout: int = 0
    reyno: float = 4.0          # 0 < REYNO < 99.99 -> VISLAM = REYNO*1e-5
    rf_vis: float = 0.5
    ftrans: float = 0.0001
    prandtl: float = 1.0
    ypluswall: float = 0.0
    facmixup: float = 2.0
    nmixup: int = 1000
    nlos: int = 5
    ilos: int = 10              # 10: LOSS; 100-199: NEW_LOSS; 200-299: Spalart-Allmaras (SPAL_LOSS)
    # Spalart-Allmaras source-term factors FAC_STMIX, FAC_ST0..3, FAC_SFVIS,
    # FAC_VORT, FAC_PGRAD (the reader's defaults, 631-639)
    fac_stmix: float = 0.0
    fac_st: tuple = (1.0, 1.0, 1.0, 1.0)
    fac_sfvis: float = 2.0
    fac_vort: float = 0.0
    fac_pgrad: float = 0.0
    turbvis_lim: float = 3000.0
    in_vr: int = 0
    in_flow: int = 0            # IN_FLOW: 0 off, 3 towards FLOWIN, otherwise towards the mean flow
    flowin: float = 0.0         # FLOWIN (kg/s through all blade passages)
    rflow: float = 0.0          # RFLOW relaxation
    plate_loss: float = 0.0     # PLATE_LOSS (exit spanwise loss)
    throttle_exit: float = 0.0  # THROTTLE_EXIT marker, with THROTTLE_PRES, THROTTLE_MAS, RFTHROTL
    throttle_pres: float = 0.0
    throttle_mas: float = 0.0
    rfthrotl: float = 0.0
    # inlet data on the KM grid points as INPINT leaves it (PO1, TO1, VTIN,
    # VM1, BS, BR); None: uniform po1 / to1, no swirl or pitch, and VM1 from
    # the isentropic expansion to the first row's upstream pressure guess
    inlet: Optional[dict] = None
    ibound: int = 0
    in_vtan: int = 0
    in_press: int = 0
    f_pdown: float = 0.0
    sfexit: float = 0.0
    nsfexit: int = 0
    yplam: float = 5.0
    ypturb: float = 25.0


def geometric_spacing(n_intervals: int, ratio: float, fmax: float) -> np.ndarray:
    """FP/FR as the reader expands them when FP(3)=0 (multall-open-18.3.f:
    1961-2028): a geometric series from both walls, capped at fmax; returned
    un-normalised, length n_intervals+1 with a trailing zero (FP(IM)=0)."""
    m = n_intervals + 1
    f = np.zeros(m + 1, dtype=f32)          # 1-based
    f[1] = f32(1.0)
    f[m] = f32(0.0)
    for k in range(2, m):
        f[k] = f32(f[k - 1] * f32(ratio))
    for k in range(1, m):
        frev = f[m - k]
        if frev < f[k]:
            f[k] = frev
        if f[k] > f32(fmax):
            f[k] = f32(fmax)
    return f[1:].copy()


def _stretch(n: int, length: float, first: float) -> np.ndarray:
    """n intervals over `length`, smallest interval ~first at the start,
    growing geometrically; returns cumulative positions (n+1,)."""
    if n <= 0:
        return np.zeros(1)
    if first * n >= length:
        return np.linspace(0.0, length, n + 1)
    lo, hi = 1.0 + 1e-9, 2.0
    for _ in range(200):
        q = 0.5 * (lo + hi)
        s = first * (q ** n - 1.0) / (q - 1.0)
        if s > length:
            hi = q
        else:
            lo = q
    q = 0.5 * (lo + hi)
    d = first * q ** np.arange(n)
    d *= length / d.sum()
    return np.concatenate([[0.0], np.cumsum(d)])


def row_axial_grid(row: RowSpec, x_le: float) -> np.ndarray:
    """Axial positions of the row's JM points (LE at JLE, TE at JTE)."""
    nb = row.jte - row.jle
    s = np.linspace(0.0, 1.0, nb + 1)
    sb = 0.75 * s + 0.25 * 0.5 * (1.0 - np.cos(math.pi * s))
    xb = x_le + row.chord * sb
    d0 = xb[1] - xb[0]
    d1 = xb[-1] - xb[-2]
    up = _stretch(row.jle - 1, row.up_len, d0)
    dn = _stretch(row.jm - row.jte, row.dn_len, d1)
    xu = x_le - up[::-1]
    xd = xb[-1] + dn
    x = np.concatenate([xu[:-1], xb, xd[1:]])
    assert x.size == row.jm, (x.size, row.jm)
    return x


def thickness(s: np.ndarray, row: RowSpec) -> np.ndarray:
    """Normal thickness / chord along the chord fraction s in [0,1]."""
    t = np.empty_like(s)
    a = s <= row.xtmax
    t[a] = row.tle + (row.tmax - row.tle) * (1.0 - ((row.xtmax - s[a]) / row.xtmax) ** 2)
    b = ~a
    t[b] = row.tte + (row.tmax - row.tte) * (1.0 - ((s[b] - row.xtmax) / (1.0 - row.xtmax)) ** 2)
    return t


@dataclasses.dataclass
class CaseGeometry:
    """What the reader leaves in COMMON for SETUP (geometry and row cards)."""
    spec: CaseSpec
    im: int
    jm: int
    km: int
    x: np.ndarray          # X(J,K)       (KM, JM)
    r: np.ndarray          # R(J,K)
    rt_upp: np.ndarray     # RT_UPP(J,K)
    rt_thick: np.ndarray   # RT_THICK(J,K)
    fp: np.ndarray         # FP(1:IM), un-normalised
    fr: np.ndarray         # FR(1:KM), un-normalised
    row_first_j: List[int]
    ktips: List[int]
    ktipe: List[int]
    fthick: np.ndarray     # FTHICK(NR,K)  (NROWS, KM)
    # a deck's NSECS_IN blade sections before NEW_INTPOL, XSURF, RSURF,
    # RT_UPP, RT_THICK (4, NSECS_IN, JM), and FRACTIP1/2 (NROWS, 2); None
    # for the generated cases
    sections: Optional[np.ndarray] = None
    fractip: Optional[np.ndarray] = None


def build_geometry(spec: CaseSpec, dtype=f32) -> CaseGeometry:
    im, km = spec.im, spec.km
    rng = np.random.default_rng(spec.seed)
    nrows = len(spec.rows)
    fp = geometric_spacing(im - 1, spec.fp_ratio, spec.fp_max)
    fr = geometric_spacing(km - 1, spec.fr_ratio, spec.fr_max)
    frs = np.concatenate([[0.0], np.cumsum(fr[:-1].astype(np.float64))])
    frs /= frs[-1]                                   # fractional span of each K
    jm = sum(r.jm for r in spec.rows)
    x = np.zeros((km, jm))
    rt_c = np.zeros((km, jm))
    thick = np.zeros((km, jm))
    first_j = []
    ktips, ktipe = [], []
    fthick = np.ones((nrows, km))
    xcur = 0.0
    j0 = 0
    for nr, row in enumerate(spec.rows):
        x_le = xcur + row.up_len
        xr = row_axial_grid(row, x_le)
        if nr > 0:
            # first point of this row 1% of the neighbouring spacings
            # downstream of the last point of the previous row (the
            # reader's ISHIFT=1 rule, multall-open-18.3.f:1564-1576)
            prev_last = x[0, j0 - 1]
            d_prev = x[0, j0 - 1] - x[0, j0 - 2]
            d_next = xr[1] - xr[0]
            xr = xr - xr[0] + prev_last + 0.01 * (d_prev + d_next)
            x_le = xr[row.jle - 1]
        x_te = xr[row.jte - 1]
        first_j.append(j0 + 1)
        # per-section angle noise, interpolated across the span
        sec_span = np.linspace(0.0, 1.0, row.nsect)
        n_in = rng.normal(0.0, row.noise_deg, row.nsect)
        n_out = rng.normal(0.0, row.noise_deg, row.nsect)
        zero = np.zeros(row.nsect)
        d_in = np.asarray(row.d_in, np.float64) if len(row.d_in) else zero
        d_out = np.asarray(row.d_out, np.float64) if len(row.d_out) else zero
        d_stag = np.asarray(row.d_stag, np.float64) if len(row.d_stag) else zero
        jmid = (row.jle + row.jte) // 2 - 1

        def camber(ch):
            # r*theta of the camber line: integrate tan(chi) dx (trapezoids)
            tanc = np.tan(ch)
            rt = np.concatenate([[0.0], np.cumsum(0.5 * (tanc[1:] + tanc[:-1]) * np.diff(xr))])
            return rt - rt[row.jle - 1]

        for k in range(km):
            chi1 = math.radians(row.chi_in + np.interp(frs[k], sec_span, n_in + d_in))
            chi2 = math.radians(row.chi_out + np.interp(frs[k], sec_span, n_out + d_out))
            stag = math.radians(float(np.interp(frs[k], sec_span, d_stag)))
            s = np.clip((xr - x_le) / (x_te - x_le), 0.0, 1.0)
            chi = chi1 + (chi2 - chi1) * s
            rtc = camber(chi)
            if stag != 0.0:
                # the section turned by the stagger offset about its mid-chord point
                rts = camber(chi + stag)
                rtc = rts - (rts[jmid] - rtc[jmid])
                chi = chi + stag
            t = np.zeros_like(xr)
            on = (np.arange(row.jm) >= row.jle - 1) & (np.arange(row.jm) <= row.jte - 1)
            t[on] = row.chord * thickness(s[on], row) / np.cos(chi[on])
            # the reader takes the LE and TE points as zero thickness
            t[row.jle - 1] = 0.0
            t[row.jte - 1] = 0.0
            x[k, j0:j0 + row.jm] = xr
            rt_c[k, j0:j0 + row.jm] = rtc
            thick[k, j0:j0 + row.jm] = t
        if row.tip_gap > 0.0:
            kt = int(np.argmax(frs >= 1.0 - row.tip_gap - 1e-12)) + 1   # 1-based
            kt = min(max(kt, 2), km - 1)
            ktips.append(kt)
            ktipe.append(km)
            fthick[nr, kt - 1:] = 0.0
        else:
            ktips.append(0)
            ktipe.append(0)
        xcur = xr[-1]
        j0 += row.jm
    xf = x.astype(np.float64)
    rh = spec.hub(xf)
    rc = spec.casing(xf)
    r = rh + frs[:, None] * (rc - rh)
    rt_upp = rt_c + 0.5 * thick
    return CaseGeometry(spec=spec, im=im, jm=jm, km=km,
                        x=x.astype(dtype), r=r.astype(dtype), rt_upp=rt_upp.astype(dtype),
                        rt_thick=thick.astype(dtype), fp=fp, fr=fr,
                        row_first_j=first_j, ktips=ktips, ktipe=ktipe,
                        fthick=fthick.astype(f32))


# --------------------------------------------------------------------------
# The benchmark configurations: single nozzle row, single stage, batch of
# stages, four-stage compressor.
# --------------------------------------------------------------------------

def _const(v):
    return lambda x: np.full_like(x, v, dtype=np.float64)


def nozzle_row(im=37, jm=97, km=33, seed=0, jle=18, jte=74) -> CaseSpec:
    """One axial-turbine nozzle row: 48 vanes, hub r 0.30 m, casing 0.36 m,
    axial chord 0.04 m, circular-arc camber 0 -> 70 deg, t/c 0.20 at 40 %
    chord, LE/TE 1.5 % / 0.8 %, +-0.5 deg section noise; 37x97x33 H-mesh
    (17 upstream, 57 on blade, 23 downstream), wall expansion ratio 1.2;
    P0 2.0e5 Pa, T0 1200 K, exit hub static 1.1e5 Pa with radial
    equilibrium; mixing length 0.02 x span, mu = 4e-5, CFL 0.4."""
    row = RowSpec(nblade=48, jm=jm, jle=jle, jte=jte, chi_in=0.0, chi_out=70.0,
                  tmax=0.20, xtmax=0.40, tle=0.015, tte=0.008, chord=0.04,
                  up_len=0.03, dn_len=0.03, noise_deg=0.5,
                  pup=1.98e5, ple=1.95e5, pte=1.12e5, pdn=1.10e5,
                  xllim=(0.03, 0.03, 0.02, 0.02, 0.03, 0.02))
    return CaseSpec(name="nozzle_37x97x33", im=im, km=km, rows=[row],
                    hub=_const(0.30), casing=_const(0.36), po1=2.0e5, to1=1200.0,
                    pdown_hub=1.1e5, pdown_tip=1.1e5, seed=seed, nsteps_max=5000,
                    nchange=1000, ir=3, jr=3, kr=3, irbb=9, jrbb=9, krbb=9,
                    fblk=(0.4, 0.0, 0.1))


def turbine_stage(im=65, jm_row=121, km=49, seed=1, pexit=0.85e5, rpm=9000.0) -> CaseSpec:
    """Single-stage axial turbine: the nozzle row above and a 60-blade rotor
    at 9000 rpm, metal angles 40 -> -62 deg, t/c 0.15, tip clearance 1 %
    span; mixing plane between the rows; 65 x 242 (121 per row) x 49,
    3-level multigrid with block sizes 3 and 9; exit static 0.85e5 Pa."""
    jle = int(round(jm_row * 18 / 97))
    jte = int(round(jm_row * 74 / 97))
    stator = RowSpec(nblade=48, jm=jm_row, jle=jle, jte=jte, chi_in=0.0, chi_out=70.0,
                     tmax=0.20, xtmax=0.40, tle=0.015, tte=0.008, chord=0.04,
                     up_len=0.03, dn_len=0.012, noise_deg=0.5,
                     pup=1.98e5, ple=1.95e5, pte=1.25e5, pdn=1.22e5, stage=1,
                     xllim=(0.03, 0.03, 0.02, 0.02, 0.03, 0.02))
    rotor = RowSpec(nblade=60, jm=jm_row, jle=jle, jte=jte, rpm=rpm, rpm_hub=rpm,
                    chi_in=40.0, chi_out=-62.0, tmax=0.15, xtmax=0.35, tle=0.012,
                    tte=0.008, chord=0.035, up_len=0.012, dn_len=0.03, tip_gap=0.01,
                    noise_deg=0.5, pup=1.22e5, ple=1.18e5, pte=0.88e5, pdn=pexit, stage=1,
                    xllim=(0.03, 0.03, 0.02, 0.02, 0.03, 0.02))
    return CaseSpec(name=f"stage_{im}x{2 * jm_row}x{km}", im=im, km=km, rows=[stator, rotor],
                    hub=_const(0.30), casing=_const(0.36), po1=2.0e5, to1=1200.0,
                    pdown_hub=pexit, pdown_tip=pexit, seed=seed, nsteps_max=20000,
                    nchange=1000, conlim=0.00001)


def compressor_4stage(im=73, jm_row=89, km=57, seed=4, pr_row=1.10, chi_rotor=(-66.0, -54.0),
                      chi_stator=(39.0, 8.0)) -> CaseSpec:
    """Four-stage axial compressor, 8 rows (36,52,40,56,44,60,48,64 blades),
    12000 rpm, hub 0.25 m, casing tapering 0.40 -> 0.33 m, P0 1.013e5 Pa,
    T0 288.15 K; double-circular-arc sections with t/c 0.08 and +-0.3 deg
    noise; 73 x 752 x 57 with mixing planes between all rows.  The metal
    angles follow the mean-radius velocity triangles at 12000 rpm (blade
    speed ~390 m/s, axial velocity ~160 m/s: relative inflow ~-68 deg, de
    Haller ratio ~0.72; stator inflow ~39 deg), and the exit static pressure
    is the inlet's times pr_row per row (2.14 over the 8 rows)."""
    counts = [36, 52, 40, 56, 44, 60, 48, 64]
    rows = []
    npts = []
    extra = 752 - 8 * jm_row          # 40 inlet/exit points
    for nr, nb in enumerate(counts):
        n = jm_row + (extra // 2 if nr in (0, 7) else 0)
        npts.append(n)
    p = 1.0e5
    for nr, nb in enumerate(counts):
        rotor = nr % 2 == 0
        n = npts[nr]
        lead = n - jm_row if nr == 0 else 0
        jle = lead + int(round(jm_row * 0.25))
        jte = lead + int(round(jm_row * 0.75))
        p_in, p_out = p, p * pr_row
        rows.append(RowSpec(nblade=nb, jm=n, jle=jle, jte=jte,
                            rpm=12000.0 if rotor else 0.0, rpm_hub=12000.0 if rotor else 0.0,
                            chi_in=(chi_rotor[0] if rotor else chi_stator[0]),
                            chi_out=(chi_rotor[1] if rotor else chi_stator[1]),
                            tmax=0.08, xtmax=0.5, tle=0.01, tte=0.01, chord=0.03,
                            up_len=0.012 + (0.03 if nr == 0 else 0.0),
                            dn_len=0.012 + (0.03 if nr == 7 else 0.0),
                            noise_deg=0.3, pup=p_in, ple=p_in, pte=p_out, pdn=p_out,
                            stage=nr // 2 + 1))
        p = p_out
    return CaseSpec(name=f"compressor_{im}x752x{km}", im=im, km=km, rows=rows,
                    hub=_const(0.25),
                    casing=lambda x: 0.40 - (0.40 - 0.33) * np.clip((x - x.min()) / (x.max() - x.min()), 0, 1),
                    po1=1.013e5, to1=288.15, pdown_hub=p, pdown_tip=p, seed=seed,
                    nsteps_max=20000, nchange=1000)


def batch_instance(seed: int) -> CaseSpec:
    """One member of the 64-instance batch: I in {33,49,65}, K in {33,49},
    J in [97,161] split between two rows, exit P/P0 in [0.45,0.70],
    rotor speed in [7000,10000] rpm, otherwise the single stage."""
    rng = np.random.default_rng(1000 + seed)
    im = int(rng.choice([33, 49, 65]))
    km = int(rng.choice([33, 49]))
    jtot = int(rng.integers(97, 162))
    jrow = max(jtot // 2, 48)
    pexit = float(rng.uniform(0.45, 0.70)) * 2.0e5
    rpm = float(rng.uniform(7000.0, 10000.0))
    return turbine_stage(im=im, jm_row=jrow, km=km, seed=seed, pexit=pexit, rpm=rpm)


CONFIGS = {
    "nozzle": nozzle_row,
    "stage": turbine_stage,
    "compressor": compressor_4stage,
}


def small_stage(im=9, jm_row=25, km=7, seed=3) -> CaseSpec:
    """A small two-row stage for fast tests (same physics as the stage)."""
    spec = turbine_stage(im=im, jm_row=jm_row, km=km, seed=seed)
    spec.name = f"small_stage_{im}x{2 * jm_row}x{km}"
    spec.ir = spec.jr = spec.kr = 2
    spec.irbb = spec.jrbb = spec.krbb = 4
    for r in spec.rows:
        r.up_len *= 0.7
        r.dn_len *= 0.7
    return spec


def small_nozzle(im=9, jm=29, km=7, seed=2) -> CaseSpec:
    spec = nozzle_row(im=im, jm=jm, km=km, seed=seed, jle=7, jte=21)
    spec.name = f"small_nozzle_{im}x{jm}x{km}"
    spec.ir = spec.jr = spec.kr = 2
    spec.irbb = spec.jrbb = spec.krbb = 4
    return spec
