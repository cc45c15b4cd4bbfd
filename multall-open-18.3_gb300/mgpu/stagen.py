"""Blade-section generator restating Stagen 18.1 (Stagen-18.1/Stagen-18.1.f,
the reference's pre-processor that turns a blade-design input file into a
MULTALL deck): for every blade row the J grid along the axial chord with its
upstream and downstream extensions, and for every input section the
camber-line / thickness construction, the leading- and trailing-edge
rounding, the rotation, the projection onto the stream surface and the
stacking, giving per section the four arrays a MULTALL deck holds for it
(X, the suction-surface R*THETA, the tangential thickness and R at each J).

REAL*4 throughout, as Stagen computes (numpy float32 scalars, each operation
rounded to float32).  Built for the design chain and for batches of
generated machines; it produces the same (CaseSpec-independent) geometry
arrays that `mgpu.deck` reads from a deck's sections.

Not restated: the interactive prompts (the thick-blade factor FACTK is taken
as 1, every generated section is accepted), the HGRAPH plotting, the
quasi-3D (KM = 2) and throughflow (IM = 2) branches, and the stage_old.dat
writer.  In Stagen 18.1 as distributed the loop that samples the suction
surface and the thickness at the cosine-spaced chord points before the grid
interpolation is commented out (Stagen-18.1.f:1469-1490), which leaves that
surface unset; the loop's own text is restated here (with the linear
interpolation it names as the safer choice), and the reference's
Single-stage-turbine-17.1 deck, which Stagen wrote from the sample input
stagen-single-stg-turbine.dat, is the check that this is what produced it.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .deck import _Cards, DeckError

f32 = np.float32
PI = f32(3.1415927)                        # Stagen-18.1.f:71
DEGRAD = f32(PI / f32(180.0))              # :72


class StagenError(ValueError):
    pass


# ---------------------------------------------------------------------------
# the three interpolation / geometry helpers (Stagen-18.1.f:2379-2590)
# ---------------------------------------------------------------------------

def intp(n: int, xn, yn, x) -> np.float32:
    """INTP (2379-2414): Lagrange interpolation through the four table
    points around x (all n when n < 4); xn increasing, 1-based arrays."""
    y = f32(0.0)
    L = 1
    nm = n
    if n >= 4:
        nm = 4
        while True:
            if x < xn[L]:
                if L > 2:
                    L = n - 3 if L == n else L - 2
                else:
                    L = 1
                break
            if L == n:
                L = n - 3
                break
            L += 1
    for l1 in range(1, nm + 1):
        co = f32(1.0)
        for l2 in range(1, nm + 1):
            temp = f32(1.0) if l1 == l2 else f32(f32(x - xn[L + l2 - 1]) / f32(xn[L + l1 - 1] - xn[L + l2 - 1]))
            co = f32(co * temp)
        y = f32(y + f32(co * yn[L + l1 - 1]))
    return y


def linint(npoints: int, x, y, xarg) -> np.float32:
    """LININT (2419-2450): linear interpolation, extrapolating from the end
    intervals; 1-based arrays."""
    if x[1] > xarg:
        return f32(y[1] + f32(f32(f32(xarg - x[1]) * f32(y[2] - y[1])) / f32(x[2] - x[1])))
    n = 2
    while True:
        if x[n] > xarg:
            return f32(y[n] + f32(f32(f32(xarg - x[n]) * f32(y[n - 1] - y[n])) / f32(x[n - 1] - x[n])))
        n += 1
        if n > npoints:
            m = npoints
            return f32(y[m] + f32(f32(f32(xarg - x[m]) * f32(y[m] - y[m - 1])) / f32(x[m] - x[m - 1])))


def insect(nxpts: int, nc: int, xc, yc, x0, y0, alpha):
    """INSECT (2454-2540): the intersection of the curve (xc, yc) with the
    line through (x0, y0) at angle alpha to the x axis; near the ends, where
    the line misses the curve, with the curve extrapolated along its end
    chord.  Returns None where the reference leaves XINT, YINT unset."""
    nle = nxpts // 3
    nte = nxpts - nle
    xnorm = f32(np.cos(alpha))
    ynorm = f32(np.sin(alpha))
    perp1 = f32(f32(xnorm * f32(yc[1] - y0)) - f32(ynorm * f32(xc[1] - x0)))
    perpend = f32(f32(xnorm * f32(yc[nxpts] - y0)) - f32(ynorm * f32(xc[nxpts] - x0)))
    if nc < nle and perp1 <= 0.0:
        # the curve's first point and its third give the end chord
        dydxs = f32(f32(yc[3] - yc[1]) / f32(xc[3] - xc[1]))
        dydxn = f32(np.tan(alpha))
        top = f32(f32(f32(f32(x0 * dydxn) - f32(xc[1] * dydxs)) + yc[1]) - y0)
        xint = f32(top / f32(dydxn - dydxs))
        return xint, f32(y0 + f32(f32(xint - x0) * dydxn))
    if nc > nte and perpend >= 0.0:
        dydxs = f32(f32(yc[nxpts - 2] - yc[nxpts]) / f32(xc[nxpts - 2] - xc[nxpts]))
        dydxn = f32(np.tan(alpha))
        top = f32(f32(f32(f32(x0 * dydxn) - f32(xc[nxpts] * dydxs)) + yc[nxpts]) - y0)
        xint = f32(top / f32(dydxn - dydxs))
        return xint, f32(y0 + f32(f32(xint - x0) * dydxn))
    perpp = f32(0.0001)
    for n in range(1, nxpts + 1):
        perp = f32(f32(xnorm * f32(yc[n] - y0)) - f32(ynorm * f32(xc[n] - x0)))
        if perp < 0.0 and perpp > 0.0:
            fac = f32(perpp / f32(perpp - perp))
            xdif = f32(xc[n] - xc[n - 1])
            if 3 <= n <= nxpts - 1:
                dydxl = f32(f32(yc[n + 1] - yc[n - 1]) / f32(xc[n + 1] - xc[n - 1]))
                dydxp = f32(f32(yc[n] - yc[n - 2]) / f32(xc[n] - xc[n - 2]))
                ddy = f32(f32(dydxl - dydxp) / xdif)
            else:
                ddy = f32(0.0)
            xint = f32(xc[n - 1] + f32(fac * xdif))
            yint = f32(f32(yc[n - 1] + f32(fac * f32(yc[n] - yc[n - 1])))
                       + f32(f32(f32(f32(f32(0.5) * fac) * fac) * ddy) * xdif) * xdif)
            return xint, yint
        perpp = perp
    return None


def find_dydx(npoints: int, x, y) -> np.ndarray:
    """FIND_DYDX (2543-2560): central differences, one-sided at the ends."""
    d = np.zeros(npoints + 1, f32)
    for n in range(2, npoints):
        d[n] = f32(f32(y[n + 1] - y[n - 1]) / f32(x[n + 1] - x[n - 1]))
    d[1] = f32(f32(y[2] - y[1]) / f32(x[2] - x[1]))
    d[npoints] = f32(f32(y[npoints] - y[npoints - 1]) / f32(x[npoints] - x[npoints - 1]))
    return d


def smooth(npin: int, nsmooth: int, sfac, fracx, var) -> None:
    """SMOOTH (2564-2590), in place: NSMOOTH passes of a curvature-weighted
    average over the interior points of an unevenly spaced table."""
    sfac = f32(sfac)
    sfacm1 = f32(f32(1.0) - sfac)
    avg = np.zeros(npin + 2, f32)
    curv = np.zeros(npin + 2, f32)
    for _ in range(nsmooth):
        for j in range(2, npin):
            dx1 = f32(fracx[j] - fracx[j - 1])
            dx2 = f32(fracx[j + 1] - fracx[j])
            fac = f32(dx1 / f32(dx1 + dx2))
            avg[j] = f32(var[j - 1] + f32(fac * f32(var[j + 1] - var[j - 1])))
            curv[j] = f32(var[j] - avg[j])
        curv[1] = curv[2]
        curv[npin] = curv[npin - 1]
        for j in range(2, npin):
            vsmth = f32(avg[j] + f32(f32(0.5) * f32(curv[j + 1] + curv[j - 1])))
            var[j] = f32(f32(sfacm1 * var[j]) + f32(sfac * vsmth))


# ---------------------------------------------------------------------------
# input
# ---------------------------------------------------------------------------

@dataclass
class SectionInput:
    label: str
    intype: int
    nxpts: int
    nsmooth: int = 0
    fracx: Optional[np.ndarray] = None       # 1-based tables (index 0 unused)
    slope: Optional[np.ndarray] = None       # INTYPE 1/2/4: tangents after the read
    tkh: Optional[np.ndarray] = None
    tkl: Optional[np.ndarray] = None
    slpup: Optional[np.ndarray] = None
    slplow: Optional[np.ndarray] = None
    curv: Optional[np.ndarray] = None
    xyin: Optional[tuple] = None             # INTYPE 0: (x, y, ifclock, if_reflect)
    thick: tuple = ()                        # TKLE, TKTE, TKMAX, XTMAX, XMODLE, XMODTE, TK_TYP
    fchord: tuple = ()                       # FCHORD, FPERP, FTKSCALE
    rot: tuple = ()                          # ROTN, XROT, YROT
    ext: tuple = ()                          # XCUP, XCDWN, BETUP, BETDN
    xrin: Optional[np.ndarray] = None
    rin: Optional[np.ndarray] = None
    edges: tuple = ()                        # XLE, XTE, RLE, RTE
    stack: tuple = ()                        # FCENTROID, FTANG, FLEAN, FSWEEP, FAXIAL
    scale: tuple = ()                        # FSCALE, FCONST


@dataclass
class RowInput:
    title: str
    nintup: int
    ninton: int
    nintdn: int
    xfrac: np.ndarray
    relspce: np.ndarray
    nblade: int
    rpm_p: tuple                             # RPMROW, PUPROW, PLEROW, PTEROW, PDROW
    tip: tuple                               # KTIPS, KTIPE, JROTHS, JROTHE, JROTTS, JROTTE, FRACTIP, RPMHUB
    sections: List[SectionInput] = field(default_factory=list)


@dataclass
class StagenInput:
    rgas: float
    gamma: float
    im: int
    km: int
    fprat: float
    fpmax: float
    frrat: float
    frmax: float
    ifdef: int
    nrows: int
    nosect: int
    fac_scale: float
    rows: List[RowInput] = field(default_factory=list)
    pressures: tuple = ()                    # PUPHUB, PUPTIP, PDHUB, PDTIP
    controls: Optional[dict] = None          # the IFDEF != 0 control block, by Stagen name
    inlet: Optional[dict] = None             # FSPAN, POIN, TOIN, VTIN, VMIN, B1IN, BRIN (1-based tables)


# the IFDEF != 0 control block (Stagen-18.1.f:145-160), card by card
_CONTROL_CARDS = (
    ("ii", ("NMAX", "NCHANGE")),
    ("i" * 14, ("IN_VTAN", "IN_PRESS", "INPUT", "IN_VR", "ITIMST", "ISMTH", "IPOUT", "IN_FLOW", "ILOS", "NLOS",
                "IF_RESTART", "IOUTST", "IBOUND", "ISHIFT")),
    ("i" * 11, ("IR", "JR", "KR", "IRBB", "JRBB", "KRBB", "NSBUP", "NSBON", "NSBDN", "IFMIX", "NEWGRID")),
    ("iiii", ("JTRANS", "JTRANP", "JTRANH", "JTRANT")),
    ("iiiiii", ("IF_CUSP", "ICUSP", "LCUSP", "LCUSPUP", "IFANGLES", "IF_DESIGN")),
    ("r" * 7, ("CP", "GA", "CFL", "SFT", "SFX", "FAC_4TH", "MACHLIM")),
    ("r" * 7, ("DAMP", "FBLK1", "FBLK2", "FBLK3", "SFEX", "CLIM", "RFIN")),
    ("irrrrii", ("IFMIX", "RFMIX", "FSMTHB", "FEXTRAP", "FANGLE", "NEXTRAP_LE", "NEXTRAP_TE")),
    ("r" * 10, ("FSTURB", "TURBVIS_DAMP", "TURBVIS_LIM", "REYNO", "PRANDTL", "RF_VIS", "FTRANS", "YPLUSWALL",
                "YPLAM", "YPTURB")),
    ("r" * 8, ("FAC_STMIX", "FAC_ST0", "FAC_ST1", "FAC_ST2", "FAC_ST3", "FAC_SFVIS", "FAC_VORT", "FAC_PGRAD")),
    ("r" * 7, ("FRACPB", "FRACPW", "FRACPUP", "FRACPIN", "FRACPLE", "FRACPTE", "FRACPDWN")),
)


def _tab(vals) -> np.ndarray:
    a = np.zeros(len(vals) + 1, f32)
    a[1:] = np.asarray(vals, f32)
    return a


def read_stagen(text: str) -> StagenInput:
    """The input file as Stagen reads it (Stagen-18.1.f:74-1905): list-
    directed reads, each starting on a new line, and the one-line title
    reads (FORMAT 72A) taken as whole lines.  Inputs with IFDEF != 0 (the
    control-variable block) are refused."""
    c = _Cards(text)
    try:
        rgas, gamma = c.reals(2)
        im, km = c.ints(2)
        fprat, fpmax = c.reals(2)
        frrat, frmax = c.reals(2)
        ifdef = c.ints(1)[0]
        controls = None
        if ifdef != 0:
            # the control block (145-160); every card is one list-directed READ
            controls = {}
            for kinds, names in _CONTROL_CARDS:
                for name, v in zip(names, c.mixed(kinds)):
                    controls[name] = v
        nrows, nosect = c.ints(2)
        if km == 2 or im == 2:
            raise StagenError("quasi-3D (KM = 2) and throughflow (IM = 2) inputs are not generated")
        fac_scale = c.reals(1)[0]
        inp = StagenInput(float(rgas), float(gamma), im, km, fprat, fpmax, frrat, frmax, ifdef, nrows, nosect,
                          fac_scale)
        inp.controls = controls
        for _ in range(nrows):
            c.skip()
            title = c.line().strip()
            c.skip()
            nintup, ninton, nintdn = c.ints(3)
            xf, rs = [], []
            while True:
                a, b = c.reals(2)
                xf.append(a)
                rs.append(b)
                if a > 0.999999:
                    break
            nblade = c.ints(1)[0]
            rpm_p = tuple(c.reals(5))
            tip = tuple(c.mixed("iiiiiirr"))
            row = RowInput(title, nintup, ninton, nintdn, _tab(xf), _tab(rs), nblade, rpm_p, tip)
            for _ in range(nosect):
                c.skip()
                label = c.line().strip()
                c.skip()
                intype = c.ints(1)[0]
                if intype == 0:
                    npoints, nxpts, ifclock, if_reflect = c.ints(4)
                    pts = [c.reals(2) for _ in range(npoints)]
                    s = SectionInput(label, 0, nxpts,
                                     xyin=(_tab([p[0] for p in pts]), _tab([p[1] for p in pts]), ifclock, if_reflect))
                else:
                    if intype not in (1, 2, 3, 4):
                        raise StagenError(f"INTYPE {intype}")
                    npin, nxpts, nsmooth = c.ints(3)
                    s = SectionInput(label, intype, nxpts, nsmooth)
                    fx, a1, a2, a3 = [], [], [], []
                    s1 = sn = None
                    for n in range(1, npin + 1):
                        if intype == 1:
                            x, sl = c.reals(2)
                            fx.append(x)
                            a1.append(f32(np.tan(f32(sl * DEGRAD))))
                        elif intype == 2:
                            x, sl, th, tl = c.reals(4)
                            fx.append(x)
                            a1.append(f32(np.tan(f32(sl * DEGRAD))))
                            a2.append(th)
                            a3.append(tl)
                        elif intype == 3:
                            x, su, sl = c.reals(3)
                            fx.append(x)
                            a2.append(f32(np.tan(f32(su * DEGRAD))))
                            a3.append(f32(np.tan(f32(sl * DEGRAD))))
                        else:
                            if n == 1:
                                s1, sn = c.reals(2)
                            x, cv = c.reals(2)
                            fx.append(x)
                            a1.append(cv)
                    s.fracx = _tab(fx)
                    if intype in (1, 2):
                        s.slope = _tab(a1)
                    if intype == 2:
                        s.tkh, s.tkl = _tab(a2), _tab(a3)
                    if intype == 3:
                        s.slpup, s.slplow = _tab(a2), _tab(a3)
                        s.slope = np.zeros(npin + 1, f32)
                    if intype == 4:
                        s.curv = _tab(a1)
                        s.slope = np.zeros(npin + 1, f32)
                        s.slope[1], s.slope[npin] = s1, sn
                    s.thick = tuple(c.reals(7))
                    s.fchord = tuple(c.reals(3))
                s.rot = tuple(c.reals(3))
                s.ext = tuple(c.reals(4))
                c.skip()
                nss = c.ints(1)[0]
                s.xrin = _tab(c.reals(nss))
                s.rin = _tab(c.reals(nss))
                s.edges = tuple(c.reals(4))
                s.stack = tuple(c.reals(5))
                s.scale = tuple(c.reals(2))
                row.sections.append(s)
            inp.rows.append(row)
        # the machine's inlet and exit pressures and the inlet tables (2167-2186)
        c.skip()
        inp.pressures = tuple(c.reals(4))
        c.skip()
        (ninlet,) = c.ints(1)
        inp.inlet = {name: _tab(c.reals(ninlet)) for name in ("FSPAN", "POIN", "TOIN", "VTIN", "VMIN", "B1IN", "BRIN")}
        return inp
    except DeckError as e:
        raise StagenError(str(e)) from None


# ---------------------------------------------------------------------------
# generation
# ---------------------------------------------------------------------------

@dataclass
class RowGrid:
    """One blade row as Stagen writes it: the J indices and, per section,
    X, R*THETA of the suction (upper) surface, the tangential thickness and
    R at every J (0-based arrays of length jm)."""
    title: str
    nblade: int
    jm: int
    jle: int
    jte: int
    x: List[np.ndarray] = field(default_factory=list)
    y: List[np.ndarray] = field(default_factory=list)
    tk: List[np.ndarray] = field(default_factory=list)
    r: List[np.ndarray] = field(default_factory=list)


def pitch_spacing(n: int, rat, fmax) -> np.ndarray:
    """FP or FR (Stagen-18.1.f:95-130): geometric growth from both ends,
    capped at FMAX; n-1 relative spacings (0-based)."""
    nm1 = n - 1
    f1 = np.zeros(n + 1, f32)
    f1[1] = f32(1.0)
    for i in range(2, nm1 + 1):
        f1[i] = f32(f1[i - 1] * f32(rat))
    out = np.zeros(nm1, f32)
    for i in range(1, nm1 + 1):
        v = f1[i]
        f2 = f1[n - i]
        if v > f2:
            v = f2
        if v > f32(fmax):
            v = f32(fmax)
        out[i - 1] = v
    return out


def _blade_xy(s: SectionInput):
    """The section's surface points clockwise from the leading edge as
    (xup, yup, nsuct, xlow, ylow, npres, xchord, fthick) after the
    construction, the edge rounding and the rotation (Stagen-18.1.f:700-1450)."""
    nxpts = s.nxpts
    if s.intype == 0:
        xin_raw, yin_raw, ifclock, if_reflect = s.xyin
        npoints = len(xin_raw) - 1
        xmax, xmin = f32(-1000000.0), f32(1000000.0)
        fy = f32(-1.0) if if_reflect != 0 else f32(1.0)
        yle = f32(0.0)
        for n in range(1, npoints + 1):
            if xin_raw[n] > xmax:
                xmax = xin_raw[n]
            if xin_raw[n] < xmin:
                xmin = xin_raw[n]
                yle = yin_raw[n]
        xdiff = f32(xmax - xmin)
        xsurf = np.zeros(2 * max(npoints, nxpts) + 2, f32)
        ysurf = np.zeros_like(xsurf)
        for n in range(1, npoints + 1):
            nn = npoints - n + 1 if ifclock != 0 else n
            xsurf[nn] = f32(f32(xin_raw[n] - xmin) / xdiff)
            ysurf[nn] = f32(f32(fy * f32(yin_raw[n] - yle)) / xdiff)
        fthick = np.ones(2 * nxpts + 2, f32)
        nin = npoints
    else:
        nin, xsurf, ysurf, fthick = _generated_surface(s)
    # rotation about (XROT, YROT), clockwise (9999-32)
    rotn, xrot, yrot = s.rot
    if abs(rotn) >= 0.0001:
        rotn = f32(rotn * DEGRAD)
        for n in range(1, nin + 1):
            xdif = f32(xsurf[n] - xrot)
            ydif = f32(ysurf[n] - yrot)
            dist = f32(np.sqrt(f32(f32(xdif * xdif) + f32(ydif * ydif))))
            angl = f32(np.arctan(f32(ydif / xdif)))
            if xdif < 0.0:
                angl = f32(angl + PI)
            anew = f32(angl - rotn)
            xsurf[n] = f32(f32(dist * f32(np.cos(anew))) + xrot)
            ysurf[n] = f32(f32(dist * f32(np.sin(anew))) + yrot)
    # leading and trailing edge points (33), the last match of each test
    nle = nt = None
    for i in range(1, nin + 1):
        im1 = nin if i == 1 else i - 1
        ip1 = 1 if i == nin else i + 1
        if xsurf[ip1] > xsurf[i] and xsurf[im1] >= xsurf[i]:
            nle = i
        if xsurf[ip1] < xsurf[i] and xsurf[im1] <= xsurf[i]:
            nt = i
    if nle is None or nt is None:
        raise StagenError(f"section '{s.label}': no leading or trailing edge point")
    xclock = np.zeros(nin + 2, f32)
    yclock = np.zeros(nin + 2, f32)
    nte = None
    for i in range(1, nin + 1):
        n = nle + i - 1
        if n > nin:
            n -= nin
        if n == nt:
            nte = i
        xclock[i] = xsurf[n]
        yclock[i] = ysurf[n]
    xclock[nin + 1] = xclock[1]
    yclock[nin + 1] = yclock[1]
    xup = np.zeros(nin + 2, f32)
    yup = np.zeros(nin + 2, f32)
    xlow = np.zeros(nin + 2, f32)
    ylow = np.zeros(nin + 2, f32)
    for i in range(1, nte + 1):
        xup[i], yup[i] = xclock[i], yclock[i]
    for i in range(nte, nin + 2):
        ir = nin + 2 - i
        xlow[ir], ylow[ir] = xclock[i], yclock[i]
    nsuct = nte
    npres = nin + 2 - nte
    xmin = min(xlow[1], xup[1])
    xmax = max(xup[nsuct], xlow[npres])
    xchord = f32(xmax - xmin)
    # trailing-edge points must not coincide
    if f32(xup[nsuct] - xup[nsuct - 1]) < 0.000001:
        xup[nsuct - 1] = f32(f32(0.5) * f32(xup[nsuct] + xup[nsuct - 2]))
    if f32(xlow[npres] - xlow[npres - 1]) < 0.000001:
        xlow[npres - 1] = f32(f32(0.5) * f32(xlow[npres] + xlow[npres - 2]))
    return xup, yup, nsuct, xlow, ylow, npres, xmin, xchord, fthick


def _generated_surface(s: SectionInput):
    """INTYPE 1-4: camber line (or surfaces) from the slope table, the
    thickness distribution, and the edge rounding (Stagen-18.1.f:760-1420);
    returns (nin, xsurf, ysurf, fthick) with the 2*NXPTS points going round
    the blade."""
    intype, nxpts = s.intype, s.nxpts
    fracx = s.fracx
    npin = len(fracx) - 1
    slope = s.slope.copy() if s.slope is not None else np.zeros(npin + 1, f32)
    tkh = s.tkh.copy() if s.tkh is not None else None
    tkl = s.tkl.copy() if s.tkl is not None else None
    slpup = s.slpup.copy() if s.slpup is not None else np.zeros(npin + 1, f32)
    slplow = s.slplow.copy() if s.slplow is not None else np.zeros(npin + 1, f32)
    if intype == 4:
        # the slope from the inlet / outlet angles and the integrated
        # relative curvature
        curv = s.curv
        dtan = np.zeros(npin + 1, f32)
        for n in range(2, npin + 1):
            dtan[n] = f32(dtan[n - 1] + f32(f32(f32(0.5) * f32(curv[n] + curv[n - 1])) * f32(fracx[n] - fracx[n - 1])))
        slope[1] = f32(np.tan(f32(slope[1] * DEGRAD)))
        slope[npin] = f32(np.tan(f32(slope[npin] * DEGRAD)))
        dslope = f32(slope[npin] - slope[1])
        slp1 = slope[1]
        for n in range(1, npin + 1):
            fcurv = f32(dtan[n] / dtan[npin])
            slope[n] = f32(slp1 + f32(fcurv * dslope))
    if s.nsmooth != 0:
        if intype in (1, 2, 4):
            smooth(npin, s.nsmooth, 0.25, fracx, slope)
        if intype == 2:
            smooth(npin, s.nsmooth, 0.25, fracx, tkh)
            smooth(npin, s.nsmooth, 0.25, fracx, tkl)
        if intype == 3:
            smooth(npin, s.nsmooth, 0.25, fracx, slpup)
            smooth(npin, s.nsmooth, 0.25, fracx, slplow)
    n1 = nxpts + 1
    xin = np.zeros(n1, f32)
    yin = np.zeros(n1, f32)
    dydx = np.zeros(n1, f32)
    tkhigh = np.zeros(n1, f32)
    tklow = np.zeros(n1, f32)
    dydxup = np.zeros(n1, f32)
    dydxlow = np.zeros(n1, f32)
    yupc = np.zeros(n1, f32)
    ylowc = np.zeros(n1, f32)
    tkin = np.zeros(n1, f32)
    dydx[1], dydxup[1], dydxlow[1] = slope[1], slpup[1], slplow[1]
    for n in range(2, nxpts + 1):
        theta = f32(f32(n - 1) * PI / f32(nxpts - 1))
        xin[n] = f32(f32(0.5) * f32(f32(1.0) - f32(np.cos(theta))))
        dx = f32(xin[n] - xin[n - 1])
        if intype in (1, 2, 4):
            dydx[n] = intp(npin, fracx, slope, xin[n])
        if intype == 2:
            tkhigh[n] = intp(npin, fracx, tkh, xin[n])
            tklow[n] = intp(npin, fracx, tkl, xin[n])
        if intype in (1, 2, 4):
            dy = f32(f32(f32(0.5) * f32(dydx[n] + dydx[n - 1])) * dx)
            yin[n] = f32(yin[n - 1] + dy)
        if intype == 2:
            yupc[n] = f32(yin[n] + tkhigh[n])
            ylowc[n] = f32(yin[n] - tklow[n])
            tkin[n] = f32(yupc[n] - ylowc[n])
        if intype == 3:
            dydxup[n] = intp(npin, fracx, slpup, xin[n])
            yupc[n] = f32(yupc[n - 1] + f32(f32(f32(0.5) * f32(dydxup[n] + dydxup[n - 1])) * dx))
            dydxlow[n] = intp(npin, fracx, slplow, xin[n])
            ylowc[n] = f32(ylowc[n - 1] + f32(f32(f32(0.5) * f32(dydxlow[n] + dydxlow[n - 1])) * dx))
    if intype == 2:
        for n in range(1, nxpts + 1):
            yin[n] = f32(f32(0.5) * f32(yupc[n] + ylowc[n]))
    if intype == 3:
        # close the trailing edge by rotating the two surfaces
        diff = f32(yupc[nxpts] - ylowc[nxpts])
        for n in range(1, nxpts + 1):
            drot = f32(diff * xin[n])
            yupc[n] = f32(yupc[n] - f32(f32(0.5) * drot))
            ylowc[n] = f32(ylowc[n] + f32(f32(0.5) * drot))
            yin[n] = f32(f32(0.5) * f32(yupc[n] + ylowc[n]))
            tkin[n] = f32(yupc[n] - ylowc[n])
        dydx = find_dydx(nxpts, xin, yin)
    stager = f32(f32(yin[nxpts] - yin[1]) / f32(xin[nxpts] - xin[1]))
    tru_chord = f32(np.sqrt(f32(f32(stager * stager) + f32(1.0))))
    tkle, tkte, tkmax, xtmax, xmodle, xmodte, tk_typ = (f32(v) for v in s.thick)
    if tk_typ < 0.001:
        tk_typ = f32(2.0)
    fchord, fperp, ftkscale = (f32(v) for v in s.fchord)
    one = f32(1.0)
    tkle = f32(f32(tkle * f32(one - fchord)) + f32(f32(tkle * tru_chord) * fchord))
    tkte = f32(f32(tkte * f32(one - fchord)) + f32(f32(tkte * tru_chord) * fchord))
    tkmax = f32(f32(tkmax * f32(one - fchord)) + f32(f32(tkmax * tru_chord) * fchord))
    le_exp = 3
    xup = np.zeros(n1, f32)
    xlow = np.zeros(n1, f32)
    fthick = np.ones(2 * nxpts + 2, f32)
    if intype in (1, 4):
        power = f32(f32(np.log(f32(0.5))) / f32(np.log(xtmax)))
        xmax = xin[nxpts]
        factk = f32(1.0)
        if fperp > 0.99 and f32(tkle + tkmax) > 0.2:
            raise StagenError(f"section '{s.label}': a thick blade with perpendicular thickness asks for FACTK")
        tkadd = f32(tkmax - f32(tkle + f32(xtmax * f32(tkte - tkle))))
        half_pow = f32(np.power(f32(0.5), tk_typ))
        for n in range(1, nxpts + 1):
            faxcrd = f32(xin[n] / xmax)
            xin[n] = faxcrd
            xtrans = f32(np.power(faxcrd, power))
            tklin = f32(tkle + f32(xin[n] * f32(tkte - tkle)))
            tkin[n] = f32(tklin + f32(tkadd * f32(one - f32(f32(np.power(f32(abs(f32(xtrans - f32(0.5)))), tk_typ))
                                                               / half_pow))))
        tklim = f32(tkmax * f32(1.0e-5))
        for n in range(1, nxpts + 1):
            fthick[n] = factk
            tkin[n] = f32(tkin[n] * fthick[n])
            tkin[n] = f32(tkin[n] / xmax)
            if tkin[n] < tklim:
                tkin[n] = tklim
            yin[n] = f32(yin[n] / xmax)
        fperp1 = f32(one - fperp)
        for n in range(1, nxpts + 1):
            sc = f32(np.arctan(dydx[n]))
            cs, sn = f32(np.cos(sc)), f32(np.sin(sc))
            dperp = f32(f32(f32(0.5) * tkin[n]) * cs)
            half = f32(f32(fperp1 * f32(0.5)) * tkin[n])
            yupc[n] = f32(f32(yin[n] + f32(f32(fperp * dperp) * cs)) + half)
            ylowc[n] = f32(f32(yin[n] - f32(f32(fperp * dperp) * cs)) - half)
            xup[n] = f32(f32(xin[n] - f32(f32(fperp * dperp) * sn)) + f32(0.00001))
            xlow[n] = f32(f32(xin[n] + f32(f32(fperp * dperp) * sn)) - f32(0.00001))
    if intype in (2, 3):
        tkmaxgen = f32(0.0)
        for n in range(1, nxpts + 1):
            fthick[n] = one
            tkin[n] = f32(f32(tkin[n] + tkle) + f32(xin[n] * f32(tkte - tkle)))
            if tkin[n] > tkmaxgen:
                tkmaxgen = tkin[n]
        tkrat = f32(tkmax / tkmaxgen)
        tkrat = f32(f32(one - ftkscale) + f32(ftkscale * tkrat))
        for n in range(1, nxpts + 1):
            tkin[n] = f32(tkin[n] * tkrat)
        for n in range(1, nxpts + 1):
            xup[n] = xin[n]
            xlow[n] = xin[n]
            yupc[n] = f32(yin[n] + f32(f32(0.5) * tkin[n]))
            ylowc[n] = f32(yin[n] - f32(f32(0.5) * tkin[n]))
    # leading / trailing edge rounding factors (6626)
    xmax = xin[nxpts]
    facl = np.ones(n1, f32)
    for n in range(1, nxpts + 1):
        faxcrd = f32(xin[n] / xmax)
        xin[n] = faxcrd
        facl[n] = one
        if not xmodle < 0.0001:
            xmle = f32(faxcrd / xmodle)
            if not xmle > 1.0:
                xmle = f32(abs(f32(xmle - one)))
                facl[n] = f32(np.sqrt(f32(one - f32(f32(xmle * xmle) * xmle))))
        if not xmodte < 0.001:
            xmte = f32(f32(one - faxcrd) / xmodte)
            if not xmte > 1.0:
                xmte = f32(xmte - one)
                facl[n] = f32(facl[n] * f32(np.sqrt(f32(one - f32(xmte * xmte)))))
    facl[1] = f32(f32(0.5) * facl[2])
    facl[nxpts] = f32(f32(0.5) * facl[nxpts - 1])
    assert le_exp == 3
    # the surface points nearly perpendicular to the centre line, thinned
    # towards the edges (3334)
    nin = 2 * nxpts
    xsurf = np.zeros(nin + 2, f32)
    ysurf = np.zeros(nin + 2, f32)
    for nc in range(1, nxpts + 1):
        nup = nc
        nlow = nxpts + (nxpts + 1 - nc)
        alpha = f32(f32(np.arctan(dydx[nc])) + f32(f32(0.5) * PI))
        x0, y0 = xin[nc], yin[nc]
        a = insect(nxpts, nc, xup, yupc, x0, y0, alpha)
        b = insect(nxpts, nc, xlow, ylowc, x0, y0, alpha)
        if a is None or b is None:
            raise StagenError(f"section '{s.label}': no surface point normal to the centre line at point {nc}")
        xsu, ysu = a
        xsl, ysl = b
        xmid = f32(f32(0.5) * f32(xsu + xsl))
        ymid = f32(f32(0.5) * f32(ysu + ysl))
        xspan = f32(xsu - xsl)
        yspan = f32(ysu - ysl)
        xsurf[nup] = f32(xmid + f32(f32(f32(0.5) * facl[nc]) * xspan))
        xsurf[nlow] = f32(xmid - f32(f32(f32(0.5) * facl[nc]) * xspan))
        ysurf[nup] = f32(ymid + f32(f32(f32(0.5) * facl[nc]) * yspan))
        ysurf[nlow] = f32(ymid - f32(f32(f32(0.5) * facl[nc]) * yspan))
    return nin, xsurf, ysurf, fthick


def _sample(xup, yup, nsuct, xlow, ylow, npres, xmin, xchord, fthick, nxpts, interp):
    """The suction surface and the thickness at NXPTS cosine-spaced points
    of the chord, scaled to unit axial chord (the loop of
    Stagen-18.1.f:1469-1490, commented out in the distributed source)."""
    xin = np.zeros(nxpts + 1, f32)
    ysin = np.zeros(nxpts + 1, f32)
    tkin = np.zeros(nxpts + 1, f32)
    for n in range(1, nxpts + 1):
        theta = f32(f32(n - 1) * PI / f32(nxpts - 1))
        xi = f32(f32(0.5) * f32(f32(1.0) - f32(np.cos(theta))))
        xarg = f32(xmin + f32(xi * xchord))
        ys = interp(nsuct, xup, yup, xarg)
        yp = interp(npres, xlow, ylow, xarg)
        yavg = f32(f32(0.5) * f32(ys + yp))
        ys = f32(f32(yavg + f32(f32(ys - yavg) / fthick[n])) / xchord)
        yp = f32(f32(yavg + f32(f32(yp - yavg) / fthick[n])) / xchord)
        ysin[n] = ys
        tkin[n] = f32(abs(f32(ys - yp)))
        xin[n] = f32(f32(xarg - xmin) / xchord)
    return xin, ysin, tkin


def _expansion(r, npts, up: bool):
    """The grid expansion ratio that makes NPTS growing spacings span R
    first spacings (Stagen-18.1.f:1644-1668: 50 fixed-point iterations; the
    downstream branch with R < NPTS takes the update without the average,
    as the reference does)."""
    rat = f32(1.2)
    if r < npts:
        rat = f32(0.9)
    for _ in range(50):
        rhs = f32(f32(rat - f32(1.0)) * r)
        if r >= npts:
            rat = f32(f32(0.5) * f32(rat + f32(np.power(f32(rhs + f32(1.0)), f32(f32(1.0) / f32(npts))))))
        elif up:
            rat = f32(f32(0.5) * f32(f32(rat + f32(f32(_powi(rat, npts) - f32(1.0)) / r)) + f32(1.0)))
        else:
            rat = f32(f32(f32(_powi(rat, npts) - f32(1.0)) / r) + f32(1.0))
    return rat


def _powi(x, n: int):
    """REAL**INTEGER by repeated squaring (libgfortran's pow_r4_i4)."""
    x = f32(x)
    pow_ = f32(1.0)
    u = n
    while True:
        if u & 1:
            pow_ = f32(pow_ * x)
        u >>= 1
        if u:
            x = f32(x * x)
        else:
            break
    return pow_


def generate_row(row: RowInput, km: int, if_cusp: int = 0, lcusp: int = 0,
                 interp=linint) -> RowGrid:
    """Every section of one blade row on the row's J grid (Stagen-18.1.f:
    469-530 and 1604-2105)."""
    npup, npon, npdn = row.nintup, row.ninton + 1, row.nintdn
    ninton = row.ninton
    jm = npup + npon + npdn
    jle = npup + 1
    jte = npup + npon
    # relative spacing of the grid on the blade, normalised (73-7)
    nfr = len(row.xfrac) - 1
    F = np.zeros(ninton + 1, f32)
    for jj in range(1, ninton + 1):
        xx = f32(f32(jj - 1) / f32(ninton - 1))
        F[jj] = intp(nfr, row.xfrac, row.relspce, xx)
    tot = f32(0.0)
    for i in range(1, ninton + 1):
        tot = f32(tot + F[i])
    for i in range(1, ninton + 1):
        F[i] = f32(F[i] / tot)
    xgridon = np.zeros(ninton + 2, f32)
    for i in range(1, ninton + 1):
        xgridon[i + 1] = f32(xgridon[i] + F[i])
    out = RowGrid(row.title, row.nblade, jm, jle, jte)
    xcent_hub = ycent_hub = None
    for nsect, s in enumerate(row.sections, start=1):
        xup, yup, nsuct, xlow, ylow, npres, xmin, xchord, fthick = _blade_xy(s)
        nxpts = s.nxpts
        xin, ysin, tkin = _sample(xup, yup, nsuct, xlow, ylow, npres, xmin, xchord, fthick, nxpts, interp)
        xg = np.zeros(jm + 2, f32)
        yg = np.zeros(jm + 2, f32)
        tg = np.zeros(jm + 2, f32)
        rg = np.zeros(jm + 2, f32)
        sg = np.zeros(jm + 2, f32)
        for i in range(2, npon + 1):
            xarg = xgridon[i]
            nf = npup + i
            xg[nf] = xarg
            yg[nf] = intp(nxpts, xin, ysin, xarg)
            tg[nf] = intp(nxpts, xin, tkin, xarg)
        xcup, xcdwn, betup, betdn = (f32(v) for v in s.ext)
        betup = f32(np.tan(f32(betup * DEGRAD)))
        betdn = f32(np.tan(f32(betdn * DEGRAD)))
        ratup = _expansion(f32(xcup / F[1]), npup, True)
        ratdn = _expansion(f32(xcdwn / F[ninton]), npdn, False)
        # upstream extension (80)
        dx = F[1]
        dy = f32(dx * betup)
        xg[npup + 1] = f32(0.0)
        yc1 = f32(yg[npup + 2] - f32(f32(0.5) * tg[npup + 2]))
        yc2 = f32(yg[npup + 3] - f32(f32(0.5) * tg[npup + 3]))
        yg[npup + 1] = f32(f32(f32(2.0) * yc1) - yc2)
        tg[npup + 1] = f32(0.0)
        for i in range(1, npup + 1):
            nf = npup + 1 - i
            xg[nf] = f32(xg[nf + 1] - dx)
            yg[nf] = f32(yg[nf + 1] - dy)
            tg[nf] = f32(0.0)
            dx = f32(dx * ratup)
            dy = f32(betup * dx)
        # downstream extension (90)
        dx = F[ninton]
        dy = f32(dx * betdn)
        for i in range(1, npdn + 1):
            nf = npup + npon + i
            xg[nf] = f32(xg[nf - 1] + dx)
            yg[nf] = f32(f32(yg[nf - 1] - f32(f32(0.5) * tg[nf - 1])) + dy)
            tg[nf] = f32(0.0)
            dx = f32(dx * ratdn)
            dy = f32(dx * betdn)
        tg[jte + 1] = f32(f32(0.5) * tg[jte])
        # the stream surface and the meridional chord (108-109)
        xrin, rin = s.xrin, s.rin
        nss = len(xrin) - 1
        xle, xte, rle, rte = (f32(v) for v in s.edges)
        smerid = np.zeros(nss + 1, f32)
        for n in range(2, nss + 1):
            ddx = f32(xrin[n] - xrin[n - 1])
            ddr = f32(rin[n] - rin[n - 1])
            smerid[n] = f32(smerid[n - 1] + f32(np.sqrt(f32(f32(ddx * ddx) + f32(ddr * ddr)))))
        smerle, smerte = smerid[1], smerid[nss]
        for n in range(2, nss + 1):
            ddx = f32(xrin[n] - xrin[n - 1])
            if ddx < 1.0e-5:
                ddx = f32(1.0e-5)
            drdx = f32(f32(rin[n] - rin[n - 1]) / ddx)
            for is_le in (True, False):
                xa, ra = (xle, rle) if is_le else (xte, rte)
                dxr = f32(xa - xrin[n - 1])
                dxf = f32(xa - xrin[n])
                drr = f32(ra - rin[n - 1])
                drf = f32(ra - rin[n])
                hit = f32(dxr * dxf) <= 0.0 if abs(drdx) <= 1.0 else f32(drr * drf) <= 0.0
                if hit:
                    add = f32(np.sqrt(f32(f32(dxr * dxr) + f32(drr * drr))))
                    if is_le:
                        smerle = f32(smerid[n - 1] + add)
                    else:
                        smerte = f32(smerid[n - 1] + add)
        schord = f32(smerte - smerle)
        scale = f32(schord / f32(1.0))          # the sampled section has unit axial chord
        for j in range(1, jm + 1):
            sg[j] = f32(smerle + f32(scale * xg[j]))
            yg[j] = f32(scale * yg[j])
            tg[j] = f32(scale * tg[j])
            xg[j] = intp(nss, smerid, xrin, sg[j])
            rg[j] = intp(nss, smerid, rin, sg[j])
        # centroid (44) and its J (46)
        tot = s1 = s2 = f32(0.0)
        for j in range(jle + 1, jte + 1):
            area = f32(f32(f32(0.5) * f32(tg[j] + tg[j - 1])) * f32(xg[j] - xg[j - 1]))
            tot = f32(tot + area)
            s1 = f32(s1 + f32(f32(area * f32(0.5)) * f32(xg[j] + xg[j - 1])))
            s2 = f32(s2 + f32(area * f32(f32(f32(0.5) * f32(yg[j] + yg[j - 1]))
                                         - f32(f32(0.25) * f32(tg[j] + tg[j - 1])))))
        with np.errstate(divide="ignore", invalid="ignore"):
            xcent = f32(s1 / tot)           # 0/0 on a purely radial section, as in the reference
        jcent = jm // 2
        dxjm1 = f32(0.0)
        for j in range(jle, jte + 1):
            dxj = f32(xcent - xg[j])
            with np.errstate(divide="ignore", invalid="ignore"):
                ratx = f32(dxjm1 / dxj)
            if ratx < 0.0:
                jcent = j
            dxjm1 = dxj
        # Y -> R*THETA (111-112)
        th = np.zeros(jm + 1, f32)
        for j in range(2, jm + 1):
            th[j] = f32(th[j - 1] + f32(f32(f32(2.0) * f32(yg[j] - yg[j - 1])) / f32(rg[j] + rg[j - 1])))
        for j in range(1, jm + 1):
            yg[j] = f32(rg[j] * f32(th[j] - th[jcent]))
        ycent = yg[jcent]
        if nsect == 1:
            xcent_hub, ycent_hub = xcent, ycent
        # stacking (120-127)
        fcentroid, ftang, flean, fsweep, faxial = (f32(v) for v in s.stack)
        fscale, fconst = (f32(v) for v in s.scale)
        if fscale < 0.00001:
            fscale, fconst = f32(1.0), f32(0.0)
        radial = fcentroid > 1.01 or abs(f32(rte - rle)) > f32(f32(0.5) * abs(f32(xte - xle)))
        if not radial:
            for j in range(1, jm + 1):
                xg[j] = f32(xg[j] + f32(fcentroid * f32(xcent_hub - xcent)))
                yg[j] = f32(yg[j] + f32(fcentroid * f32(ycent_hub - ycent)))
        xle2, xte2 = xg[jle], xg[jte]
        yte2, yle2 = yg[jte], yg[jle]
        rle2, rte2 = rg[jle], rg[jte]
        xdif = f32(xte2 - xle2)
        ydif = f32(yte2 - yle2)
        rdif = f32(rte2 - rle2)
        deltax = f32(f32(f32(-fsweep * xdif) - f32(flean * ydif)) + f32(faxial * xdif))
        deltay = f32(f32(f32(-fsweep * ydif) + f32(flean * xdif)) + f32(ftang * xdif))
        xconst = f32(xle2 + f32(fconst * xdif))
        for j in range(1, jm + 1):
            xg[j] = f32(xconst + f32(fscale * f32(f32(xg[j] - xconst) + deltax)))
            yg[j] = f32(fscale * f32(yg[j] + deltay))
            if not abs(rdif) > f32(f32(0.5) * abs(xdif)):
                rg[j] = intp(nss, xrin, rin, xg[j])
        ymid = np.zeros(jm + 2, f32)
        sg[1] = f32(0.0)
        for j in range(2, jm + 1):
            ddx = f32(xg[j] - xg[j - 1])
            ddr = f32(rg[j] - rg[j - 1])
            sg[j] = f32(sg[j - 1] + f32(np.sqrt(f32(f32(ddx * ddx) + f32(ddr * ddr)))))
            ymid[j] = f32(yg[j] - f32(f32(0.5) * tg[j]))
        if if_cusp > 0:
            _cusp(xg, yg, tg, sg, ymid, jle, jte, jm, lcusp)
        out.x.append(xg[1:jm + 1].copy())
        out.y.append(yg[1:jm + 1].copy())
        out.tk.append(tg[1:jm + 1].copy())
        out.r.append(rg[1:jm + 1].copy())
    return out


def _cusp(xg, yg, tg, sg, ymid, jle, jte, jm, lcusp):
    """IF_CUSP > 0: a cusp extrapolated from upstream of the trailing edge
    (Stagen-18.1.f:2032-2062)."""
    j = jte
    for jj in range(jte - 10, jte + 1):
        j = jj
        if f32(tg[jj] / tg[jj - 1]) < 0.9:
            break
    else:
        j = jte + 1
    jcs = j - 1
    if jcs <= jle + 2:
        jcs = jle + 2
    jce = jte + lcusp
    tkgrad = f32(f32(tg[jcs] - tg[jcs - 2]) / f32(sg[jcs] - sg[jcs - 2]))
    ygrad = f32(f32(ymid[jcs] - ymid[jcs - 2]) / f32(sg[jcs] - sg[jcs - 2]))
    for j in range(jcs, jte + 1):
        ymid[j] = f32(ymid[jcs] + f32(ygrad * f32(sg[j] - sg[jcs])))
        tg[j] = f32(tg[jcs] + f32(tkgrad * f32(sg[j] - sg[jcs])))
        if tg[j] < 0.0:
            tg[j] = f32(0.0)
        yg[j] = f32(ymid[j] + f32(f32(0.5) * tg[j]))
    tkgrad = f32(-tg[jte] / f32(sg[jce] - sg[jte]))
    for j in range(jte, jm + 1):
        ymid[j] = f32(ymid[jcs] + f32(ygrad * f32(sg[j] - sg[jcs])))
        tg[j] = f32(tg[jte] + f32(tkgrad * f32(sg[j] - sg[jte])))
        if tg[j] < 0.0:
            tg[j] = f32(0.0)
        yg[j] = f32(ymid[j] + f32(f32(0.5) * tg[j]))


# ---------------------------------------------------------------------------
# the new-format deck (Stagen-18.1.f:166-446, 576-640, 676-680, 2095-2103,
# 2186-2320)
# ---------------------------------------------------------------------------

# the control variables Stagen sets when IFDEF = 0 (166-274); those it
# never sets (cooling, bleed, roughness, exit smoothing, plate loss,
# throttle, repeating stage, F_PDOWN) are zero
DEFAULTS = dict(NMAX=9000, IN_VTAN=0, IN_PRESS=0, IN_VR=1, ITIMST=3, IPOUT=1, IN_FLOW=0, ILOS=10, NLOS=5,
                IF_RESTART=0, IBOUND=0, IR=3, JR=3, KR=3, IRBB=9, JRBB=9, KRBB=9, IFMIX=1, JTRANS=0,
                JTRANP=0, JTRANH=0, JTRANT=0, ISHIFT=2, NCHANGE=1000, IF_CUSP=0, IF_CUSP_OUT=1, ICUSP=0,
                LCUSP=3, LCUSPUP=0, IFANGLES=0, NEXTRAP_LE=10, NEXTRAP_TE=10, IF_DESIGN=0, IF_RESTAGGER=0,
                IF_LEAN=0, CFL=0.4, SFT=0.005, SFX=0.005, FAC_4TH=0.8, MACHLIM=2.0, DAMP=10.0, FBLK1=0.4,
                FBLK2=0.2, FBLK3=0.1, CLIM=0.001, RFIN=0.5, RFMIX=0.025, FSMTHB=1.0, FEXTRAP=0.8,
                FANGLE=0.8, FSTURB=1.0, TURBVIS_DAMP=0.5, TURBVIS_LIM=3000.0, REYNO=800000.0, PRANDTL=1.0,
                RF_VIS=0.5, FTRANS=0.0001, YPLUSWALL=0.0, YPLAM=5.0, YPTURB=25.0, FACMIXUP=2.0,
                NMIXUP=1000, FRACPB=0.05, FRACPW=0.05, FRACPUP=0.03, FRACPIN=0.02, FRACPLE=0.03,
                FRACPTE=0.03, FRACPDWN=0.04, FAC_STMIX=0.0, FAC_ST0=1.0, FAC_ST1=1.0, FAC_ST2=1.0,
                FAC_ST3=1.0, FAC_SFVIS=2.0, FAC_VORT=0.0, FAC_PGRAD=0.0, F_PDOWN=0.0, IFCOOL=0, IFBLEED=0,
                IF_ROUGH=0, IF_REPEAT=0, SFEXIT=0.0, NSFEXIT=0, PLATE_LOSS=0.0, THROTTLE_EXIT=0.0)


def _fortran(fmt, values) -> List[str]:
    """Formatted WRITE: fmt a list of (kind, width, decimals) edit
    descriptors; a new record starts when the list is used up (format
    reversion).  A value too wide for its field prints as asterisks."""
    lines, cur, k = [], "", 0
    for v in values:
        kind, w, dec = fmt[k]
        t = ("%*d" % (w, int(v))) if kind == "I" else ("%*.*f" % (w, dec, float(v)))
        cur += t if len(t) <= w else "*" * w
        k += 1
        if k == len(fmt):
            lines.append(cur)
            cur, k = "", 0
    if cur or not lines:
        lines.append(cur)
    return lines


def _F(n, w, d):
    return [("F", w, d)] * n


F1700, F1701, F1717 = _F(8, 10, 6), _F(8, 10, 1), _F(8, 10, 4)
I1703 = [("I", 10, 0)] * 8


def _ld(*items) -> str:
    """List-directed WRITE: strings as they are, integers in 12 columns,
    reals in gfortran's default REAL*4 form."""
    out = ""
    for it in items:
        if isinstance(it, str):
            out += it
        elif isinstance(it, (int, np.integer)):
            out += "%12d" % it
        else:
            out += "%16.8g" % float(it)
    return " " + out


def write_deck(inp: StagenInput, **overrides) -> str:
    """The MULTALL deck Stagen writes to stage_new.dat for this input
    (IFDEF = 0: the control variables take Stagen's defaults; IFDEF != 0:
    those of the input's control block, every variable it does not set
    zero as in the reference, which then skips its defaults; keyword
    overrides by Stagen name go on top)."""
    if inp.controls is None:
        d = dict(DEFAULTS)
    else:
        d = {k: 0 for k in DEFAULTS}
        d.update({k: v for k, v in inp.controls.items() if k in d or k in ("CP", "GA")})
    for k, v in overrides.items():
        if k not in d:
            raise StagenError(f"unknown control variable {k}")
        d[k] = v
    im, km = inp.im, inp.km
    gam = f32(d.get("GA", inp.gamma))
    cp = f32(d["CP"]) if "CP" in d else f32(f32(f32(inp.rgas) * gam) / f32(gam - f32(1.0)))
    fp = pitch_spacing(im, inp.fprat, inp.fpmax)
    fr = pitch_spacing(km, inp.frrat, inp.frmax)
    L: List[str] = []
    w = L.append
    w(' DATA SET FOR "multall" . GENERATED BY "stagen" .')
    w(_ld("   CP   and   GAMMA "))
    L += _fortran(_F(2, 10, 4), [cp, gam])
    w(_ld("      ITIMST "))
    L += _fortran(I1703, [d["ITIMST"]])
    w(_ld("    CFL,    DAMP,    MACHLIM,    F_PDOWN "))
    L += _fortran(F1700, [d["CFL"], d["DAMP"], d["MACHLIM"], d["F_PDOWN"]])
    w(_ld(" IF_RESTART "))
    L += _fortran(I1703, [d["IF_RESTART"]])
    w(_ld(" NSTEPS_MAX, CONLIM "))
    L += _fortran([("I", 10, 0), ("F", 10, 6)], [d["NMAX"], d["CLIM"]])
    w(_ld("  SFX,      SFT,      FAC_4TH,     NCHANGE "))
    L += _fortran(_F(3, 10, 6) + [("I", 10, 0)], [d["SFX"], d["SFT"], d["FAC_4TH"], d["NCHANGE"]])
    w(_ld("      NUMBER OF BLADE ROWS "))
    L += _fortran(I1703, [inp.nrows])
    w(_ld("       IM        KM "))
    L += _fortran(I1703, [im, km])
    w(_ld(" FP(I),I=1,IMM1 "))
    L += _fortran(F1700, fp)
    w(_ld(" FR(K),K=1,KMM1 "))
    L += _fortran(F1700, fr)
    w(_ld("       IR        JR        KR        IRBB      JRBB      KRBB "))
    L += _fortran(I1703, [d[k] for k in ("IR", "JR", "KR", "IRBB", "JRBB", "KRBB")])
    w(_ld("  FBLK1,     FBLK2,     FBLK3  "))
    L += _fortran(F1700, [d["FBLK1"], d["FBLK2"], d["FBLK3"]])
    w(_ld("      IFMIX "))
    L += _fortran(I1703, [d["IFMIX"]])
    w(_ld("  RFMIX,    FEXTRAP,   FSMTHB,    FANGLE "))
    L += _fortran(F1700, [d["RFMIX"], d["FEXTRAP"], d["FSMTHB"], d["FANGLE"]])
    w(_ld("     IFCOOL    IFBLEED    IF_ROUGH "))
    L += _fortran(I1703, [d["IFCOOL"], d["IFBLEED"], d["IF_ROUGH"]])
    w(_ld("      NSECS_IN "))
    L += _fortran(I1703, [inp.nosect])
    w(_ld("      IN_PRESS  IN_VTAN   IN_VR    IN_FLOW  IF_REPEAT  RFIN "))
    L += _fortran([("I", 10, 0)] * 5 + [("F", 10, 5)],
                  [d["IN_PRESS"], d["IN_VTAN"], d["IN_VR"], d["IN_FLOW"], d["IF_REPEAT"], d["RFIN"]])
    w(_ld(" IPOUT  SFEXIT  NSFEXIT "))
    L += _fortran([("I", 5, 0), ("F", 10, 6), ("I", 5, 0)], [d["IPOUT"], d["SFEXIT"], d["NSFEXIT"]])
    w(_ld(" PLATE_LOSS  THROTTLE_EXIT "))
    L += _fortran(F1700, [d["PLATE_LOSS"], d["THROTTLE_EXIT"]])
    if d["THROTTLE_EXIT"] > 0.001 or d["IN_FLOW"] != 0 or d["IF_REPEAT"] != 0:
        raise StagenError("throttle, IN_FLOW and repeating-stage cards are not written")
    w(_ld("       ILOS      NLOS      IBOUND "))
    L += _fortran(I1703, [d["ILOS"], d["NLOS"], d["IBOUND"]])
    if d["ILOS"] != 0:
        w(_ld("  REYNO,     RF_VIS,   FTRANS, TURBVIS_LIM, PRANDTL,   YPLUSWALL"))
        L += _fortran([("F", 10, 1)] + _F(3, 10, 3) + [("F", 10, 1)] + _F(2, 10, 3),
                      [d["REYNO"], d["RF_VIS"], d["FTRANS"], d["TURBVIS_LIM"], d["PRANDTL"], d["YPLUSWALL"]])
    if d["ILOS"] >= 200:
        w(_ld(" FAC_STMIX,FAC_ST0,FAC_ST1,FAC_ST2,FAC_ST3,FAC_SFVIS, FAC_VORT, FAC_PGRAD"))
        L += _fortran(F1700, [d[k] for k in ("FAC_STMIX", "FAC_ST0", "FAC_ST1", "FAC_ST2", "FAC_ST3",
                                            "FAC_SFVIS", "FAC_VORT", "FAC_PGRAD")])
    w(_ld("  YPLAM      YPTURB "))
    L += _fortran(F1700, [d["YPLAM"], d["YPTURB"]])
    w(_ld("     ISHIFT    NEXTRAP_LE  NEXTRAP_TE "))
    L += _fortran(I1703, [d["ISHIFT"], d["NEXTRAP_LE"], d["NEXTRAP_TE"]])
    w(_ld(" (NSTG(N),N=1,NROWS) "))
    L += _fortran(I1703, [(nr + 1) // 2 for nr in range(1, inp.nrows + 1)])
    w(_ld(" 5  TIME STEPS FOR PRINTOUT "))
    L += _fortran(I1703, [d["NMAX"]] * 5)
    w(_ld(" MARKER FOR VARIABLES TO BE SENT TO THE OUTPUT FILE."))
    L += _fortran([("I", 2, 0)] * 40, [0] * 20)
    w(_ld(" STREAM SURFACES ON WHICH RESULTS ARE TO BE SENT TO  THE OUTPUT FILE "))
    L += _fortran([("I", 2, 0)] * 40, [0] * km)
    nshroud = 0
    for nrow, row in enumerate(inp.rows, start=1):
        ktips, ktipe, jroths, jrothe, jrotts, jrotte = row.tip[:6]
        fractip, rpmhub = row.tip[6], row.tip[7]
        rpmrow, puprow, plerow, pterow, pdrow = row.rpm_p
        if ktips < 0:
            nshroud += 1
        g = generate_row(row, km, if_cusp=d["IF_CUSP"], lcusp=d["LCUSP"])
        w(_ld("***************************************************************"))
        w(_ld("************STARTING THE INPUT FOR EACH BLADE ROW**************"))
        w(row.title)
        w(_ld("   NUMBER OF BLADES IN ROW "))
        L += _fortran(I1703, [row.nblade])
        w(_ld("       JM        JLE       JTE "))
        L += _fortran(I1703, [g.jm, g.jle, g.jte])
        w(_ld("     KTIPSTART  KTIPEND "))
        L += _fortran(I1703, [ktips, ktipe])
        if ktips > 0:
            tkmult = np.ones(km + 1, f32)
            for k in range(1, km + 1):
                if ktips <= k <= ktipe:
                    tkmult[k] = 0.0
            if ktips != 1:
                tkmult[ktips - 1] = 0.5
            if ktipe != km:
                tkmult[ktipe + 1] = 0.5
            if ktips != 1:
                tkmult[ktips - 2] = 0.9
            if ktipe != km:
                tkmult[ktipe + 2] = 0.9
            w(_ld(" FRACTIP1, FRACTIP2"))
            L += _fortran(F1700, [fractip, fractip])
            w(_ld(" BLADE TIP THINNING FACTORS"))
            L += _fortran(F1700, tkmult[1:])
        w(_ld("      BOUNDARY LAYER TRANSITION POINTS "))
        L += _fortran(I1703, [d["JTRANS"], d["JTRANP"], d["JTRANH"], d["JTRANT"]])
        w(_ld(' SET NEWGRID= 1 TO GENERATE A NEW GRID WITH DIFFERENT "J" POINTS AND SPACINGS.'))
        L += _fortran(I1703, [0])
        w(_ld("  RPMROW,    RPMHUB "))
        L += _fortran(F1701, [rpmrow, rpmhub])
        w(_ld("      JROTHS    JROTHE    JROTTS    JROTTE "))
        L += _fortran(I1703, [jroths, jrothe, jrotts, jrotte])
        w(_ld("  PUPROW    PLEROW   PTEROW    PDROW "))
        L += _fortran(F1701, [puprow, plerow, pterow, pdrow])
        w(_ld("     NSECS_ROW   INSURF  "))
        L += _fortran(I1703, [inp.nosect, 0])
        w(_ld(" IF_CUSP_OUT   IFANGLES "))
        L += _fortran(I1703, [d["IF_CUSP_OUT"], d["IFANGLES"]])
        if d["IF_CUSP_OUT"] == 1:
            L += _fortran(I1703, [d["ICUSP"], d["LCUSP"], d["LCUSPUP"]])
        if d["IF_CUSP_OUT"] == 2:
            L += _fortran([("I", 5, 0)] * 3 + _F(2, 10, 5), [2, 2, 3, 0.01, 0.99])
        for nsect in range(1, inp.nosect + 1):
            w(_ld("***************************************************************"))
            w(_ld(" ROW NUMBER", nrow, " SECTION NUMBER ", nsect))
            w(_ld(d["IF_DESIGN"], d["IF_RESTAGGER"], d["IF_LEAN"], " IF_DESIGN etc "))
            fs = inp.fac_scale
            L += _fortran(_F(2, 10, 5) + [("I", 5, 0)], [fs, 0.0, 0])
            L += _fortran(F1700, g.x[nsect - 1])
            L += _fortran(F1700, [fs, 0.0])
            L += _fortran(F1700, g.y[nsect - 1])
            L += _fortran(F1700, [fs])
            L += _fortran(F1700, g.tk[nsect - 1])
            L += _fortran(F1700, [fs, 0.0])
            L += _fortran(F1700, g.r[nsect - 1])
    # inlet conditions on the spanwise grid (95) and the exit pressures
    sumfr = np.zeros(km + 1, f32)
    for k in range(2, km + 1):
        sumfr[k] = f32(sumfr[k - 1] + fr[k - 2])
    t = inp.inlet
    nin = len(t["FSPAN"]) - 1
    bc = {n: np.zeros(km, f32) for n in ("POIN", "TOIN", "VTIN", "VMIN", "B1IN", "BRIN")}
    for k in range(1, km + 1):
        arg = f32(sumfr[k] / sumfr[km])
        for n in bc:
            bc[n][k - 1] = intp(nin, t["FSPAN"], t[n], arg)
    w(_ld(" STARTING INLET BOUNDARY CONDITION DATA ."))
    w(_ld(" NUMBER OF POINTS FOR INLET BOUNDARY CONDITIONS "))
    L += _fortran(I1703, [km])
    w(_ld(" SPACING OF INLET BOUNDARY CONDITION POINTS "))
    L += _fortran(F1700, fr)
    for label, n, f in (("  INLET STAGNATION PRESSURES ", "POIN", F1701),
                        ("  INLET STAGNATION TEMPERATURES ", "TOIN", F1717),
                        ("  INLET ABSOLUTE TANGENTIAL VELOCITY ", "VTIN", F1717),
                        ("  INLET MERIDIONAL VELOCITY ", "VMIN", F1717),
                        ("  INLET MERIDIONAL YAW ANGLE  ", "B1IN", F1717),
                        ("  INLET PITCH ANGLE ", "BRIN", F1717)):
        w(_ld(label))
        L += _fortran(f, bc[n])
    w(_ld("  PDOWN_HUB   PDOWN_TIP "))
    L += _fortran(F1701, [inp.pressures[2], inp.pressures[3]])
    if d["ILOS"] != 0:
        w(_ld("MIXING LENGTH LIMITS ON ALL BLADE ROWS"))
        for _ in range(inp.nrows):
            if d["ILOS"] == 10:
                L += _fortran(F1700, [d["FRACPB"]] * 4 + [d["FRACPW"], d["FRACPUP"]])
            if d["ILOS"] > 10:
                L += _fortran(F1700, [d["FRACPIN"], d["FRACPLE"], d["FRACPTE"], d["FRACPDWN"], d["FSTURB"],
                                      d["TURBVIS_DAMP"]])
    w(_ld(" FACTOR TO INCREASE THE TURBULENT VISCOSITY OVER THE FIRST NMIXUP STEPS "))
    L += _fortran([("F", 10, 5), ("I", 5, 0)], [d["FACMIXUP"], d["NMIXUP"]])
    for _ in range(nshroud):
        w(_ld("INPUT SHROUD DATA HERE"))
    return "\n".join(L) + "\n"


def deck_sections(text: str, jms) -> dict:
    """The blade-section arrays of a new-format deck as printed, keyed by
    (row, section), 1-based: after each 'ROW NUMBER n SECTION NUMBER m'
    line and its IF_DESIGN line, four groups of a scale line followed by
    JM values (X, R*THETA, thickness, R).  jms: JM of each row."""
    lines = text.splitlines()
    out = {}
    i = 0
    while i < len(lines):
        t = lines[i].split()
        if len(t) >= 6 and t[0] == "ROW" and t[1] == "NUMBER" and t[3] == "SECTION":
            nr, ns = int(t[2]), int(t[5])
            jm = jms[nr - 1]
            i += 2
            arrs = []
            for _ in range(4):
                i += 1
                vals: List[float] = []
                while len(vals) < jm:
                    vals += [float(v) for v in lines[i].split()]
                    i += 1
                arrs.append(np.array(vals, f32))
            out[(nr, ns)] = arrs
            continue
        i += 1
    return out


def input_to_dict(inp: StagenInput) -> dict:
    """A JSON-ready form of the parsed input (tables as lists)."""
    def conv(v):
        if isinstance(v, np.ndarray):
            return [float(x) for x in v[1:]]
        if isinstance(v, (np.floating,)):
            return float(v)
        if isinstance(v, tuple):
            return [conv(x) for x in v]
        if isinstance(v, dict):
            return {k: conv(x) for k, x in v.items()}
        if isinstance(v, list):
            return [conv(x) for x in v]
        return v
    out = {k: conv(v) for k, v in inp.__dict__.items() if k != "rows"}
    out["rows"] = []
    for r in inp.rows:
        rd = {k: conv(v) for k, v in r.__dict__.items() if k != "sections"}
        rd["sections"] = [{k: conv(v) for k, v in s.__dict__.items()} for s in r.sections]
        out["rows"].append(rd)
    return out


def input_from_dict(d: dict) -> StagenInput:
    """The inverse of input_to_dict."""
    def tab(v):
        return None if v is None else _tab(v)
    inp = StagenInput(**{k: (f32(v) if isinstance(v, float) else v) for k, v in d.items()
                         if k not in ("rows", "pressures", "inlet")})
    inp.pressures = tuple(f32(v) for v in d["pressures"])
    inp.inlet = {k: _tab(v) for k, v in d["inlet"].items()}
    for rd in d["rows"]:
        row = RowInput(rd["title"], rd["nintup"], rd["ninton"], rd["nintdn"], _tab(rd["xfrac"]),
                       _tab(rd["relspce"]), rd["nblade"], tuple(f32(v) for v in rd["rpm_p"]),
                       tuple(rd["tip"][:6]) + tuple(f32(v) for v in rd["tip"][6:]))
        for sd in rd["sections"]:
            s = SectionInput(sd["label"], sd["intype"], sd["nxpts"], sd["nsmooth"])
            for k in ("fracx", "slope", "tkh", "tkl", "slpup", "slplow", "curv", "xrin", "rin"):
                setattr(s, k, tab(sd[k]))
            if sd["xyin"] is not None:
                x, y, c, r = sd["xyin"]
                s.xyin = (_tab(x), _tab(y), c, r)
            for k in ("thick", "fchord", "rot", "ext", "edges", "stack", "scale"):
                setattr(s, k, tuple(f32(v) for v in sd[k]))
            row.sections.append(s)
        inp.rows.append(row)
    return inp


def case_from_input(inp: StagenInput, **overrides):
    """(CaseSpec, CaseGeometry) of the machine: the deck Stagen writes for
    the input, read as MULTALL reads it (mgpu.deck)."""
    from . import deck as _deck
    return _deck.read_deck(write_deck(inp, **overrides))


def main(argv=None) -> int:
    """As the reference's program runs: read a Stagen input file and write
    the new-format deck (stage_new.dat by default)."""
    import argparse
    ap = argparse.ArgumentParser(description="Stagen: blade-design input -> MULTALL deck")
    ap.add_argument("input", help="Stagen input file (e.g. stagen.dat)")
    ap.add_argument("-o", "--output", default="stage_new.dat", help="deck to write")
    args = ap.parse_args(argv)
    with open(args.input) as f:
        inp = read_stagen(f.read())
    text = write_deck(inp)
    with open(args.output, "w") as f:
        f.write(text)
    jms = [r.nintup + r.ninton + 1 + r.nintdn for r in inp.rows]
    print(f"{args.output}: {inp.nrows} rows, IM = {inp.im}, JM = {sum(jms)}, KM = {inp.km}")
    return 0


if __name__ == "__main__":
    import sys
    sys.exit(main())
