"""Reader for Multall's new-format input decks: the part of NEW_READIN
(multall-open-18.3.f:148-2161) that the time-marching path accepts, with
the geometry steps the reference runs on what it reads before SETUP forms
the metrics:

  - the per-row and per-section cards (792-1540): blade sections given as
    X, R*THETA of the upper surface, tangential thickness and radius at
    every J point of the row, scaled and shifted by their FAC/SHIFT cards,
    too-small meridional spacings opened up (1440-1468), and re-interpolated
    onto NSECS_IN sections equally spaced from hub to casing (1655-1697);
  - the grid of the gaps between rows and upstream / downstream of the
    blading for ISHIFT = 1..4 (1553-1818), with GRID_UP (9433-9512),
    GRID_DOWN (9201-9432, including the trailing-edge cusp of IF_CUSP = 1)
    and SOLVE (9513-9540);
  - the inlet boundary cards and INPINT's interpolation onto the KM grid
    points (1855-1946, 9073-9199), the FP / FR / FR_IN geometric series
    (1948-2028), the mixing-length limits and FACMIXUP (2036-2081), the
    roughness cards (2091-2113);
  - NEW_INTPOL (7493-7613), called by SETUP (6435) after FR is normalised
    (6322-6327): the KM stream surfaces, with the tip-gap grid (FRMOD).

The result is a CaseSpec and a CaseGeometry, which common_setup.build_common
turns into the COMMON state, as for the generated cases.  This is test-side
input, like common_setup: it is not on the product path.

Arithmetic is float32 in the reference's order of operations (REAL*4).  One
value is undefined in the reference: GRID_DOWN's IF_CUSP = 0 branch starts
its running meridional distance from the local SNEW(J1-NEXTRAP-1), which no
statement sets; it is taken as 0 here.  Only differences of SNEW are used,
so this can change the rounding and nothing else.  `x ** n` with an integer
n is evaluated by binary powering, as gfortran's run time does.

Options outside the library's scope are refused with DeckError: real gas
(CP < 0), ITIMST 5/6, throughflow and Q3D (IM = 2, KM = 2), IF_REPEAT,
cooling and bleed, shrouds (KTIPS < 0), designed / restaggered / leaned
sections, INSURF != 0, NEW_GRID, IPOUT = 3.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List

import numpy as np

from .case import CaseGeometry, CaseSpec, RowSpec

f32 = np.float32
PI = f32(3.14159265)
DEGRAD = f32(PI / f32(180.0))


class DeckError(ValueError):
    """The deck uses an option this reader (and the library) does not cover,
    or it does not parse as the reader's cards."""


def _powi(x, n: int):
    """x**n for an integer n: binary powering in float32."""
    m = abs(n)
    y = x if m % 2 else f32(1.0)
    while True:
        m >>= 1
        if not m:
            break
        x = f32(x * x)
        if m % 2:
            y = f32(y * x)
    return f32(f32(1.0) / y) if n < 0 else y


class _Cards:
    """Fortran list-directed reads over the deck's lines: each READ starts
    on a new line, takes as many lines as its items need, and drops the
    rest of its last line."""

    def __init__(self, text: str):
        self.lines = text.splitlines()
        self.pos = 0

    def line(self) -> str:
        if self.pos >= len(self.lines):
            raise DeckError("the deck ends early")
        s = self.lines[self.pos]
        self.pos += 1
        return s

    def skip(self, n: int = 1):
        """READ(5,*) DUMMY_INPUT: one line of text."""
        for _ in range(n):
            self.line()

    def _tokens(self, n: int) -> List[str]:
        out: List[str] = []
        while len(out) < n:
            for t in self.line().replace(",", " ").split():
                if len(out) == n:
                    break
                if "*" in t:
                    rep, v = t.split("*", 1)
                    out.extend([v] * int(rep))
                else:
                    out.append(t)
        return out[:n]

    def reals(self, n: int) -> List[np.float32]:
        try:
            return [f32(t.replace("D", "E").replace("d", "e")) for t in self._tokens(n)]
        except ValueError as e:
            raise DeckError(f"line {self.pos}: {e}") from None

    def ints(self, n: int) -> List[int]:
        try:
            return [int(t) for t in self._tokens(n)]
        except ValueError as e:
            raise DeckError(f"line {self.pos}: {e}") from None

    def mixed(self, kinds: str) -> list:
        """One READ of items typed by kinds ('i' integer, 'r' real)."""
        toks = self._tokens(len(kinds))
        try:
            return [int(t) if k == "i" else f32(t.replace("D", "E")) for k, t in zip(kinds, toks)]
        except ValueError as e:
            raise DeckError(f"line {self.pos}: {e}") from None

    def optional(self, kinds: str, defaults: list) -> list:
        """READ(5,*,ERR=...): items are taken across lines, as for any
        list-directed read, until one does not parse; that item and the rest
        keep their defaults, and the read ends with the line it stopped on."""
        out = list(defaults)
        n = 0
        while n < len(kinds):
            for t in self.line().replace(",", " ").split():
                try:
                    v = int(t) if kinds[n] == "i" else f32(t.replace("D", "E"))
                    if kinds[n] == "i" and not -2 ** 31 <= v < 2 ** 31:
                        raise ValueError("integer overflow")
                    out[n] = v
                except ValueError:
                    return out
                n += 1
                if n == len(kinds):
                    break
        return out


def intp(n: int, xn, yn, x):
    """INTP (7801-7872): Lagrange interpolation through four neighbouring
    table points (all n points when n < 4).  xn, yn are 1-based."""
    span = f32(xn[n] - xn[1])
    y = f32(0.0)
    L = 1
    nm = n
    if n >= 4:
        nm = 4
        while True:
            if (span > 0.0 and x < xn[L]) or (span < 0.0 and x > xn[L]):
                # label 5
                if L > 2:
                    L = L - 2 if L != n else n - 3
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
            if l1 == l2:
                temp = f32(1.0)
            else:
                temp = f32(f32(x - xn[L + l2 - 1]) / f32(xn[L + l1 - 1] - xn[L + l2 - 1]))
            co = f32(co * temp)
        y = f32(y + f32(co * yn[L + l1 - 1]))
    return y


def solve(npup: int, xup, dx1):
    """SOLVE (9513-9540): the expansion ratio of a geometric progression of
    npup intervals with first interval dx1 covering xup."""
    rup = f32(xup / dx1)
    rat = f32(1.2)
    if rup < f32(npup):
        rat = f32(0.9)
    m = 1
    while True:
        rhs = f32(f32(rat - f32(1.0)) * rup)
        if rup >= f32(npup):
            rnew = f32(np.power(f32(rhs + f32(1.0)), f32(f32(1.0) / f32(npup))))
        else:
            rnew = f32(f32(f32(_powi(rat, npup) - f32(1.0)) / rup) + f32(1.0))
        diff = abs(f32(f32(rnew / rat) - f32(1.0)))
        rat = rnew
        m += 1
        if diff < f32(0.00001) or m > 250:
            return rat


@dataclasses.dataclass
class _RowCards:
    nblades: int
    jm: int
    jle: int
    jte: int
    ktips: int
    ktipe: int
    fractip: tuple
    fthick: np.ndarray
    jtran: tuple
    rpm: float
    rpm_hub: float
    jrot: tuple
    pguess: tuple
    nsecs_row: int
    if_cusp: int
    if_angles: int
    cusp: tuple          # ICUSP, LCUSP, LCUSPUP
    sep: tuple           # NUP_I1, NUP_IM, N_WAKE, SEP_THIK, SEP_DRAG
    angles: tuple        # BETAUP, BETADWN1, BETADWN2 per section (IF_ANGLES > 0)
    title: str


class _Geometry:
    """XSURF, RSURF, RT_UPP, RT_THICK (J, K) on the input sections, 1-based,
    and SMERID, as the reader's COMMON holds them."""

    def __init__(self, jd: int, kd: int):
        self.xs = np.zeros((jd + 2, kd + 2), f32)
        self.rs = np.zeros((jd + 2, kd + 2), f32)
        self.rtu = np.zeros((jd + 2, kd + 2), f32)
        self.rtt = np.zeros((jd + 2, kd + 2), f32)
        self.smerid = np.zeros((jd + 2, kd + 2), f32)

    def merid(self, k: int, jm: int):
        self.smerid[1, k] = f32(0.0)
        for j in range(2, jm + 1):
            xd = f32(self.xs[j, k] - self.xs[j - 1, k])
            rd = f32(self.rs[j, k] - self.rs[j - 1, k])
            self.smerid[j, k] = f32(self.smerid[j - 1, k] + np.sqrt(f32(f32(xd * xd) + f32(rd * rd))))


def _grid_down(g: _Geometry, k, j1, j2, s1, s2, ngap, sdist, xint, rint, nextrap, beta_dwn1, beta_dwn2,
               ifcusp, icusp, lcusp, lcuspup, ifangles):
    """GRID_DOWN (9201-9432): the grid from a trailing edge to the mixing
    plane or the exit, and the grid angles (and cusp) there."""
    n = g.xs.shape[0]
    snew = np.zeros(n, f32)
    ansx = np.zeros(n, f32)
    ansr = np.zeros(n, f32)
    th_upp = np.zeros(n, f32)
    th_thick = np.zeros(n, f32)
    th_mid = np.zeros(n, f32)
    snew[j1] = s1
    snew[j2] = s2
    sdiff = f32(s2 - s1)
    nint = j2 - j1
    r1 = f32(g.smerid[j1, k] - g.smerid[j1 - 1, k])
    rat = solve(nint, sdiff, r1)
    xd = r1
    for j in range(j1 + 1, j2):
        snew[j] = f32(snew[j - 1] + xd)
        xd = f32(xd * rat)
    for j in range(j1, j2 + 1):
        ansx[j] = intp(ngap, sdist, xint, snew[j])
        ansr[j] = intp(ngap, sdist, rint, snew[j])
    for j in range(j1, j2 + 1):
        g.xs[j, k] = ansx[j]
        g.rs[j, k] = ansr[j]
    if ifcusp == 0:
        if ifangles == 0:
            jstrt = j1 - nextrap
            # snew[jstrt - 1] is the undefined local of the reference, here 0
            snew[jstrt - 1] = f32(0.0)
            for j in range(jstrt, j2 + 1):
                xd = f32(g.xs[j, k] - g.xs[j - 1, k])
                rd = f32(g.rs[j, k] - g.rs[j - 1, k])
                snew[j] = f32(snew[j - 1] + np.sqrt(f32(f32(xd * xd) + f32(rd * rd))))
                th_upp[j] = f32(g.rtu[j, k] / g.rs[j, k])
                th_thick[j] = f32(g.rtt[j, k] / g.rs[j, k])
                th_mid[j] = f32(th_upp[j] - f32(f32(0.5) * th_thick[j]))
            dsmer = f32(snew[j1] - snew[jstrt])
            slopes = f32(f32(th_upp[j1] - th_upp[jstrt]) / dsmer)
            slopetk = f32(f32(th_thick[j1] - th_thick[jstrt]) / dsmer)
            slopep = f32(slopes - slopetk)
            slopecent = f32(f32(0.5) * f32(slopes + slopep))
            betadown1 = slopecent
            betadown2 = betadown1
        else:
            betadown1 = f32(f32(np.tan(f32(beta_dwn1 * DEGRAD))) / g.rs[j1, k])
            betadown2 = f32(f32(np.tan(f32(beta_dwn2 * DEGRAD))) / g.rs[j2, k])
        js = j1
        for j in range(j1, j2 + 1):
            if g.rtt[j, k] < f32(f32(1.0e-4) * sdiff):
                js = j
                break
        for j in range(js + 1, j2 + 1):
            fdown = f32(f32(snew[j] - snew[j1]) / f32(snew[j2] - snew[j1]))
            betadown = f32(betadown1 + f32(fdown * f32(betadown2 - betadown1)))
            dsdist = f32(snew[j] - snew[j - 1])
            g.rtu[j, k] = f32(g.rtu[j - 1, k] + f32(f32(g.rs[j, k] * betadown) * dsdist))
            g.rtt[j, k] = f32(0.0)
        return
    # a new cusp (IF_CUSP != 0)
    lup = 20
    jstrt = j1 - lup
    snew[jstrt - 1] = f32(0.0)
    for j in range(jstrt, j2 + 1):
        xd = f32(g.xs[j, k] - g.xs[j - 1, k])
        rd = f32(g.rs[j, k] - g.rs[j - 1, k])
        snew[j] = f32(snew[j - 1] + np.sqrt(f32(f32(xd * xd) + f32(rd * rd))))
        th_upp[j] = f32(g.rtu[j, k] / g.rs[j, k])
        th_thick[j] = f32(g.rtt[j, k] / g.rs[j, k])
        th_mid[j] = f32(th_upp[j] - f32(f32(0.5) * th_thick[j]))
    js = jstrt + 1
    if js > j1:
        js = j1
    j = js
    while j <= j1:
        rthik = f32(th_thick[j] / th_thick[j - 1])
        if rthik < f32(0.9):
            break
        j += 1
    jcs = j - 1
    tkgrad = f32(f32(th_thick[jcs] - th_thick[jcs - 2]) / f32(snew[jcs] - snew[jcs - 2]))
    ygrad = f32(f32(th_mid[jcs] - th_mid[jcs - 2]) / f32(snew[jcs] - snew[jcs - 2]))
    for j in range(jcs, j1 + 1):
        th_mid[j] = f32(th_mid[jcs] + f32(ygrad * f32(snew[j] - snew[jcs])))
        th_thick[j] = f32(th_thick[jcs] + f32(tkgrad * f32(snew[j] - snew[jcs])))
        if th_thick[j] < 0.0:
            th_thick[j] = f32(0.0)
        th_upp[j] = f32(th_mid[j] + f32(f32(0.5) * th_thick[j]))
        g.rtu[j, k] = f32(g.rs[j, k] * th_upp[j])
        g.rtt[j, k] = f32(g.rs[j, k] * th_thick[j])
    jstrt = j1 - lcuspup
    dsmer = f32(snew[jstrt] - snew[jstrt - 2])
    slopes = f32(f32(th_upp[jstrt] - th_upp[jstrt - 2]) / dsmer)
    slopetk = f32(f32(th_thick[jstrt] - th_thick[jstrt - 2]) / dsmer)
    slopep = f32(slopes - slopetk)
    slopecent = f32(f32(0.5) * f32(slopes + slopep))
    if ifangles == 0:
        betadown1 = betadown2 = slopecent
    else:
        betadown1 = f32(f32(np.tan(f32(beta_dwn1 * DEGRAD))) / g.rs[jstrt, k])
        betadown2 = f32(f32(np.tan(f32(beta_dwn2 * DEGRAD))) / g.rs[jstrt, k])
    ythickte = g.rtt[jstrt, k]
    if ythickte < 0.0:
        ythickte = f32(0.0)
    ymidte = f32(g.rtu[jstrt, k] - f32(f32(0.5) * ythickte))
    for j in range(jstrt + 1, j2 + 1):
        fdown = f32(f32(snew[j] - snew[jstrt]) / f32(snew[j2] - snew[jstrt]))
        betadown = f32(betadown1 + f32(fdown * f32(betadown2 - betadown1)))
        dsdist = f32(snew[j] - snew[j - 1])
        ymid = f32(ymidte + f32(f32(g.rs[j, k] * slopecent) * f32(snew[j] - snew[jstrt])))
        clength = f32(snew[jstrt + lcusp] - snew[jstrt])
        plength = f32(snew[j] - snew[jstrt])
        if plength > clength:
            plength = clength
        jcuspend = jstrt + lcusp
        if jcuspend - j >= 0:
            ytnew = f32(ythickte * f32(f32(1.0) - f32(plength / clength)))
            g.rtt[j, k] = ytnew
            if icusp == 0:
                g.rtu[j, k] = f32(ymid + f32(f32(0.5) * ytnew))
            if icusp == 1:
                g.rtu[j, k] = f32(g.rtu[j - 1, k] + f32(f32(g.rs[j, k] * slopes) * dsdist))
            if icusp == -1:
                g.rtu[j, k] = f32(f32(f32(g.rtu[j - 1, k] - g.rtt[j - 1, k])
                                      + f32(f32(g.rs[j, k] * slopep) * dsdist)) + ytnew)
        else:
            g.rtu[j, k] = f32(g.rtu[j - 1, k] + f32(f32(g.rs[j, k] * betadown) * dsdist))
            g.rtt[j, k] = f32(0.0)


def _grid_up(g: _Geometry, k, j1, j2, s1, s2, ngap, sdist, xint, rint, nextrap, beta_up, ifangles):
    """GRID_UP (9433-9512): the grid from the inlet or a mixing plane to a
    leading edge, with the grid angle of the blade's camber line there."""
    n = g.xs.shape[0]
    snew = np.zeros(n, f32)
    ansx = np.zeros(n, f32)
    ansr = np.zeros(n, f32)
    th_upp = np.zeros(n, f32)
    th_thick = np.zeros(n, f32)
    snew[j1] = s1
    snew[j2] = s2
    sdiff = f32(s2 - s1)
    nint = j2 - j1
    r1 = f32(g.smerid[j2 + 1, k] - g.smerid[j2, k])
    rat = solve(nint, sdiff, r1)
    xd = r1
    for j in range(j1 + 1, j2):
        jsub = j2 + j1 - j
        snew[jsub] = f32(snew[jsub + 1] - xd)
        xd = f32(xd * rat)
    if j1 != 1:
        snew[j1] = f32(snew[j1] + f32(f32(0.01) * f32(snew[j1 + 1] - snew[j1])))
    for j in range(j1, j2 + 1):
        ansx[j] = intp(ngap, sdist, xint, snew[j])
        ansr[j] = intp(ngap, sdist, rint, snew[j])
    for j in range(j1, j2 + 1):
        g.xs[j, k] = ansx[j]
        g.rs[j, k] = ansr[j]
    for j in range(j1, j2 + nextrap + 1):
        th_upp[j] = f32(g.rtu[j, k] / g.rs[j, k])
        th_thick[j] = f32(g.rtt[j, k] / g.rs[j, k])
    if ifangles == 0:
        num = f32(f32(f32(th_upp[j2] - f32(f32(0.5) * th_thick[j2])) - th_upp[j2 + nextrap])
                  + f32(f32(0.5) * th_thick[j2 + nextrap]))
        slopet = f32(num / f32(g.smerid[j2, k] - g.smerid[j2 + nextrap, k]))
    else:
        slopet = f32(f32(np.tan(f32(beta_up * DEGRAD))) / g.rs[j2, k])
    rtheta_le = f32(g.rtu[j2, k] - f32(f32(0.5) * g.rtt[j2, k]))
    for j in range(j1, j2):
        g.rtu[j, k] = f32(rtheta_le + f32(f32(g.rs[j, k] * slopet) * f32(snew[j] - snew[j2])))


def _geometric(f: np.ndarray, m: int):
    """The FP / FR / FR_IN geometric series (1960-2028) when entry 3 is 0:
    f is 1-based with m points (m-1 intervals)."""
    if f[3] > f32(0.00001):
        return
    rat, fmax = f[1], f[2]
    f[1] = f32(1.0)
    f[m] = f32(0.0)
    for k in range(2, m):
        f[k] = f32(f[k - 1] * rat)
    for k in range(1, m):
        frev = f[m - k]
        if frev < f[k]:
            f[k] = frev
        if f[k] > fmax:
            f[k] = fmax


def read_deck(text: str, name: str = "deck") -> tuple[CaseSpec, CaseGeometry]:
    """Reads a new-format deck; returns the CaseSpec (control cards, row
    cards, inlet data on the KM grid points) and the CaseGeometry that
    NEW_INTPOL leaves for SETUP."""
    c = _Cards(text)
    c.line()                                            # TITLE
    c.skip()
    cp, ga = c.optional("rr", [f32(1005.0), f32(1.4)])
    if cp < 0.0:
        raise DeckError("real-gas properties (CP < 0, IFGAS = 1) are not supported")
    c.skip()
    (itimst,) = c.optional("i", [3])
    if itimst in (5, 6, -5, -6):
        raise DeckError("ITIMST 5/6 (artificial compressibility) are not supported")
    if itimst in (4, -4):
        raise DeckError("ITIMST 4 (user F1/F2/F3) is not supported")
    c.skip()
    cfl, dampin, machlim, f_pdown = c.optional("rrrr", [f32(0.4), f32(10.0), f32(2.0), f32(0.0)])
    c.skip()
    (if_restart,) = c.optional("i", [0])
    c.skip()
    nsteps_max, conlim = c.optional("ir", [5000, f32(0.005)])
    c.skip()
    sfxin, sftin, fac_4th, nchange = c.optional("rrri", [f32(0.005), f32(0.005), f32(0.8), nsteps_max // 4])
    if if_restart:
        nchange = 100
    c.skip()
    (nrows,) = c.ints(1)
    c.skip()
    im, km = c.ints(2)
    if im <= 2 or km <= 2:
        raise DeckError("throughflow / Q3D grids (IM = 2 or KM = 2) are not supported")
    fp = np.zeros(im + 2, f32)
    fr = np.zeros(km + 2, f32)
    c.skip()
    fp[1:im] = c.reals(im - 1)
    c.skip()
    fr[1:km] = c.reals(km - 1)
    c.skip()
    ir, jr, kr, irbb, jrbb, krbb = c.optional("iiiiii", [3, 3, 3, 9, 9, 9])
    c.skip()
    fblk = c.optional("rrr", [f32(0.4), f32(0.2), f32(0.1)])
    c.skip()
    (ifmix,) = c.optional("i", [1])
    rfmix, fextrap, fsmthb, fangle = f32(0.025), f32(0.8), f32(1.0), f32(0.8)
    if ifmix != 0:
        c.skip()
        rfmix, fextrap, fsmthb, fangle = c.optional("rrrr", [rfmix, fextrap, fsmthb, fangle])
    c.skip()
    ifcool, ifbleed, if_rough = c.optional("iii", [0, 0, 0])
    if ifcool or ifbleed:
        raise DeckError("cooling and bleed flows are not supported")
    c.skip()
    (nsecs_in,) = c.ints(1)
    c.skip()
    in_press, in_vtan, in_vr, in_flow, if_repeat, rfin = c.optional("iiiiir", [0, 0, 1, 0, 0, f32(0.1)])
    if if_repeat:
        raise DeckError("IF_REPEAT is not supported")
    c.skip()
    ipout, sfexit, nsfexit = c.optional("iri", [1, f32(0.0), 0])
    if ipout == 3:
        raise DeckError("IPOUT = 3 (exit pressure given per K) is not supported")
    c.skip()
    plate_loss, throttle_exit = c.optional("rr", [f32(0.0), f32(0.0)])
    throttle_pres = throttle_mas = rfthrotl = f32(0.0)
    if throttle_exit > f32(0.001):
        throttle_pres, throttle_mas, rfthrotl = c.reals(3)
    flowin = rflow = f32(0.0)
    if in_flow != 0:
        c.skip()
        flowin, rflow = c.reals(2)
    c.skip()
    ilos, nlos, ibound = c.optional("iii", [100, 5, 0])
    reyno, rf_vis, ftrans, turbvis_lim, prandtl, ypluswall = (f32(500000.0), f32(0.5), f32(0.0001),
                                                              f32(3000.0), f32(1.0), f32(0.0))
    if ilos != 0:
        c.skip()
        reyno, rf_vis, ftrans, turbvis_lim, prandtl, ypluswall = c.optional(
            "rrrrrr", [reyno, rf_vis, ftrans, turbvis_lim, prandtl, ypluswall])
    sa = [f32(0.0), f32(1.0), f32(1.0), f32(1.0), f32(1.0), f32(2.0), f32(0.0), f32(0.0)]
    if ilos >= 200:
        c.skip()
        sa = c.optional("rrrrrrrr", sa)
    yplam, ypturb = f32(5.0), f32(25.0)
    if ilos != 0:
        c.skip()
        yplam, ypturb = c.optional("rr", [yplam, ypturb])
    c.skip()
    ishift, nextrap_le, nextrap_te = c.optional("iii", [2, 10, 10])
    nstage = [1 + (n - 1) // 2 for n in range(1, nrows + 1)]
    c.skip()
    got = c.optional("i" * nrows, nstage)
    nstage = [int(v) for v in got]
    c.skip()
    c.optional("iiiii", [0] * 5)                        # NOUT
    c.skip()
    c.optional("i" * 13, [0] * 13)                      # IOUT
    c.skip()
    c.optional("i" * km, [0] * km)                      # KOUT

    maxk = max(nsecs_in, km) + 2
    jd = 4000
    g = _Geometry(jd, maxk)
    rows: List[_RowCards] = []
    jstart, jmix, jle_, jte_ = [], [], [], []
    j1 = 1
    for nr in range(1, nrows + 1):
        c.skip(2)
        title = c.line().strip()
        c.skip()
        (nblades,) = c.ints(1)
        c.skip()
        jmrow, jlerow, jterow = c.ints(3)
        c.skip()
        ktips, ktipe = c.ints(2)
        if ktips <= 0:
            ktipe = 0
        if ktips < 0:
            raise DeckError("shroud leakage (KTIPS < 0) is not supported")
        fractip = (f32(0.0), f32(0.0))
        if ktips > 0:
            c.skip()
            fractip = tuple(c.reals(2))
        fthick = np.ones(km, f32)
        if ktips > 0 and ktipe > 0:
            c.skip()
            fthick[:] = c.reals(km)
        c.skip()
        jtran = tuple(c.ints(4))
        c.skip()
        (new_grid,) = c.ints(1)
        if new_grid != 0:
            raise DeckError("NEW_GRID (a regenerated streamwise grid) is not supported")
        c.skip()
        rpmrow, rpmhub = c.reals(2)
        c.skip()
        jr4 = c.ints(4)
        jr4 = [jmrow if (v == 0 or v > jmrow) else v for v in jr4]
        c.skip()
        pguess = tuple(c.reals(4))
        c.skip()
        nsecs_row, insurf = c.optional("ii", [nsecs_in, 0])
        if insurf != 0:
            raise DeckError("INSURF != 0 (new hub / casing curves) is not supported")
        if nsecs_in == 1:
            nsecs_row = 1
            nsecs_in = 2
        if nsecs_row == 1:
            nsecs_row = 2
        c.skip()
        if_cusp, if_angles = c.optional("ii", [0, 0])
        cusp = (0, 0, 0)
        sep = (0, 0, 0, f32(0.0), f32(1.0))
        if if_cusp == 1:
            cusp = tuple(c.ints(3))
        if if_cusp == 2:
            sep = tuple(c.mixed("iiirr"))
        j2 = j1 + jmrow - 1
        if j2 + 2 > jd:
            raise DeckError("JM too large")
        for k in range(1, nsecs_row + 1):
            c.skip(2)
            if_design, if_stagger, if_lean = c.optional("iii", [0, 0, 0])
            if if_design or if_stagger or if_lean:
                raise DeckError("designed, restaggered or leaned sections are not supported")
            fac1, xshift = c.reals(2)
            g.xs[j1:j2 + 1, k] = c.reals(jmrow)
            fac2, tshift = c.reals(2)
            g.rtu[j1:j2 + 1, k] = c.reals(jmrow)
            (fac3,) = c.reals(1)
            g.rtt[j1:j2 + 1, k] = c.reals(jmrow)
            fac4, rshift = c.reals(2)
            g.rs[j1:j2 + 1, k] = c.reals(jmrow)
            # meridional spacings too small for the grid, 1440-1468
            sd = np.zeros(jd + 2, f32)
            for j in range(j1 + 1, j2 + 1):
                xd = f32(g.xs[j, k] - g.xs[j - 1, k])
                rd = f32(g.rs[j, k] - g.rs[j - 1, k])
                sd[j] = f32(sd[j - 1] + np.sqrt(f32(f32(xd * xd) + f32(rd * rd))))
            srange = f32(sd[j2] - sd[j1])
            slim = f32(f32(0.0001) * srange)
            for j in range(j1 + 2, j2 + 1):
                if f32(sd[j] - sd[j - 1]) < slim:
                    den = f32(sd[j - 2] - sd[j - 1])
                    xd = f32(f32(slim * f32(g.xs[j - 2, k] - g.xs[j - 1, k])) / den)
                    rd = f32(f32(slim * f32(g.rs[j - 2, k] - g.rs[j - 1, k])) / den)
                    g.xs[j, k] = f32(g.xs[j - 1, k] + xd)
                    g.rs[j, k] = f32(g.rs[j - 1, k] + rd)
            # scale and shift, 1500
            for j in range(j1, j2 + 1):
                g.xs[j, k] = f32(fac1 * f32(xshift + g.xs[j, k]))
                g.rtt[j, k] = f32(fac3 * g.rtt[j, k])
                g.rs[j, k] = f32(fac4 * f32(rshift + g.rs[j, k]))
                g.rtu[j, k] = f32(fac2 * f32(tshift + g.rtu[j, k]))
        # NSECS_IN sections equally spaced between the hub and casing, 1655-1697
        xi1 = np.zeros(maxk, f32)
        xi2 = np.zeros(maxk, f32)
        xi3 = np.zeros(maxk, f32)
        xi4 = np.zeros(maxk, f32)
        for j in range(j1, j2 + 1):
            xnh, rnh = g.xs[j, 1], g.rs[j, 1]
            xnt, rnt = g.xs[j, nsecs_row], g.rs[j, nsecs_row]
            xspan = f32(xnt - xnh)
            rspan = f32(rnt - rnh)
            for k in range(1, nsecs_row + 1):
                xi1[k], xi2[k], xi3[k], xi4[k] = g.xs[j, k], g.rs[j, k], g.rtu[j, k], g.rtt[j, k]
            for k in range(1, nsecs_in + 1):
                fspan = f32(f32(k - 1) / f32(nsecs_in - 1))
                if abs(xspan) > abs(rspan):
                    xarg = f32(xnh + f32(fspan * f32(xnt - xnh)))
                    g.xs[j, k] = xarg
                    g.rs[j, k] = intp(nsecs_row, xi1, xi2, xarg)
                    g.rtu[j, k] = intp(nsecs_row, xi1, xi3, xarg)
                    g.rtt[j, k] = intp(nsecs_row, xi1, xi4, xarg)
                else:
                    rarg = f32(rnh + f32(fspan * f32(rnt - rnh)))
                    g.rs[j, k] = rarg
                    g.xs[j, k] = intp(nsecs_row, xi2, xi1, rarg)
                    g.rtu[j, k] = intp(nsecs_row, xi2, xi3, rarg)
                    g.rtt[j, k] = intp(nsecs_row, xi2, xi4, rarg)
        angles = ((), (), ())
        if if_angles > 0:
            c.skip()
            (n_angles,) = c.ints(1)
            fr_sp = np.zeros(n_angles + 1, f32)
            aup = np.zeros(n_angles + 1, f32)
            ad1 = np.zeros(n_angles + 1, f32)
            ad2 = np.zeros(n_angles + 1, f32)
            fr_sp[1:] = c.reals(n_angles)
            aup[1:] = c.reals(n_angles)
            ad1[1:] = c.reals(n_angles)
            ad2[1:] = c.reals(n_angles)
            qspan = np.zeros(maxk, f32)
            j_mid = j1 + (jlerow + jterow) // 2
            for k in range(2, nsecs_in + 1):
                xdif = f32(g.xs[j_mid, k] - g.xs[j_mid, k - 1])
                rdif = f32(g.rs[j_mid, k] - g.rs[j_mid, k - 1])
                qspan[k] = f32(qspan[k - 1] + np.sqrt(f32(f32(xdif * xdif) + f32(rdif * rdif))))
            for k in range(1, nsecs_in + 1):
                qspan[k] = f32(qspan[k] / qspan[nsecs_in])
            bu, b1, b2 = [f32(0)] * (nsecs_in + 1), [f32(0)] * (nsecs_in + 1), [f32(0)] * (nsecs_in + 1)
            for k in range(1, nsecs_in + 1):
                bu[k] = intp(n_angles, fr_sp, aup, qspan[k])
                b1[k] = intp(n_angles, fr_sp, ad1, qspan[k])
                b2[k] = intp(n_angles, fr_sp, ad2, qspan[k])
            angles = (tuple(bu), tuple(b1), tuple(b2))
        rows.append(_RowCards(nblades, jmrow, jlerow, jterow, ktips, ktipe, fractip, fthick, jtran,
                              float(rpmrow), float(rpmhub), tuple(jr4), pguess, nsecs_row, if_cusp, if_angles,
                              cusp, sep, angles, title))
        jle_.append(j1 + jlerow - 1)
        jte_.append(j1 + jterow - 1)
        jstart.append(j1)
        jmix.append(j2)
        j1 = j2 + 1
    jm = j2

    # ------------------ the grid between the rows, 1553-1818 ---------------
    if ishift == 1 or ishift > 2:
        # ISHIFT = 1 (and the first part of 3, 4): blades shifted axially so
        # that the hub spacing is continuous across each mixing plane
        xshift = f32(0.0)
        for j in range(2, jm + 1):
            if (j - 1) in jmix and (j - 1) != jm:
                diff1 = f32(g.xs[j - 1, 1] - g.xs[j - 2, 1])
                diff2 = f32(g.xs[j + 1, 1] - g.xs[j, 1])
                xshift = f32(f32(g.xs[j - 1, 1] + f32(f32(0.01) * f32(diff1 + diff2))) - g.xs[j, 1])
            for k in range(1, km + 1):
                g.xs[j, k] = f32(g.xs[j, k] + xshift)
    if ishift >= 2:
        xint = np.zeros(jd + 2, f32)
        rint = np.zeros(jd + 2, f32)
        sdist = np.zeros(jd + 2, f32)
        for nrow_gap in range(1, nrows + 2):
            if nrow_gap == 1:
                nrw, jst, jend = 1, 1, jle_[0]
                jmid = 0
            if 1 < nrow_gap != nrows + 1:
                nrw = nrow_gap
                jst, jend, jmid = jte_[nrw - 2], jle_[nrw - 1], jmix[nrw - 2]
            if nrow_gap == nrows + 1:
                nrw = nrows + 1
                jst, jend = jte_[nrows - 1], jm
            for k in range(1, nsecs_in + 1):
                g.merid(k, jm)
                dlast = f32(-1.0)
                npoints = 1
                xgap = f32(g.xs[jend, k] - g.xs[jst, k])
                rgap = f32(g.rs[jend, k] - g.rs[jst, k])
                gap = np.sqrt(f32(f32(xgap * xgap) + f32(rgap * rgap)))
                for j in range(jst, jend + 1):
                    xd = f32(g.xs[j, k] - g.xs[jst, k])
                    rd = f32(g.rs[j, k] - g.rs[jst, k])
                    proj = f32(f32(xd * xgap) + f32(rd * rgap))
                    if ishift >= 3:
                        proj = f32(proj / gap)
                    dist = np.sqrt(f32(f32(xd * xd) + f32(rd * rd)))
                    if proj < 0.0:
                        continue
                    if dist > f32(f32(1.00001) * gap):
                        xint[npoints] = g.xs[jend, k]
                        rint[npoints] = g.rs[jend, k]
                        npoints += 1
                        break
                    if dist < dlast:
                        continue
                    dlast = dist
                    lin = ishift == 3 or (ishift == 4 and not (k == 1 or k == nsecs_in))
                    if lin:
                        xint[npoints] = f32(g.xs[jst, k] + f32(f32(proj * xgap) / gap))
                        rint[npoints] = f32(g.rs[jst, k] + f32(f32(proj * rgap) / gap))
                    else:
                        xint[npoints] = g.xs[j, k]
                        rint[npoints] = g.rs[j, k]
                    npoints += 1
                ngaps = npoints - 1
                sfgap = f32(0.2)
                for _ in range(10):
                    for nn in range(2, ngaps):
                        xint[nn] = f32(f32(f32(f32(1.0) - sfgap) * xint[nn])
                                       + f32(f32(sfgap * f32(0.5)) * f32(xint[nn - 1] + xint[nn + 1])))
                        rint[nn] = f32(f32(f32(f32(1.0) - sfgap) * rint[nn])
                                       + f32(f32(sfgap * f32(0.5)) * f32(rint[nn - 1] + rint[nn + 1])))
                sdist[1] = g.smerid[jst, k]
                for nn in range(2, ngaps + 1):
                    xd = f32(xint[nn] - xint[nn - 1])
                    rd = f32(rint[nn] - rint[nn - 1])
                    sdist[nn] = f32(sdist[nn - 1] + np.sqrt(f32(f32(xd * xd) + f32(rd * rd))))
                smid = f32(f32(0.5) * f32(sdist[1] + sdist[ngaps]))
                ste = sdist[1]
                sle = sdist[ngaps]

                def ang(rw, which):
                    a = rows[rw - 1].angles[which]
                    return a[k] if a else f32(0.0)
                anglup = ang(nrw, 0) if nrw <= nrows else f32(0.0)
                if nrw == 1:
                    angd1, angd2 = ang(1, 1), ang(1, 2)
                else:
                    angd1, angd2 = ang(nrw - 1, 1), ang(nrw - 1, 2)
                if nrw == nrows + 1:
                    angd1, angd2 = ang(nrows, 1), ang(nrows, 2)
                if nrw == 1:
                    _grid_up(g, k, jst, jend, ste, sle, ngaps, sdist, xint, rint, nextrap_le, anglup,
                             rows[0].if_angles)
                if nrw == nrows + 1:
                    up = rows[nrows - 1]
                    _grid_down(g, k, jst, jend, ste, sle, ngaps, sdist, xint, rint, nextrap_te, angd1, angd2,
                               up.if_cusp, *up.cusp, up.if_angles)
                elif nrw != 1:
                    up = rows[nrw - 2]
                    _grid_down(g, k, jst, jmid, ste, smid, ngaps, sdist, xint, rint, nextrap_te, angd1, angd2,
                               up.if_cusp, *up.cusp, up.if_angles)
                    _grid_up(g, k, jmid + 1, jend, smid, sle, ngaps, sdist, xint, rint, nextrap_le, anglup,
                             rows[nrw - 1].if_angles)

    # ------------------ inlet boundary data, 1855-1946 ---------------------
    c.skip(2)
    (kin,) = c.ints(1)
    fr_in = np.zeros(max(kin, 3) + 2, f32)
    c.skip()
    fr_in[1:kin] = c.reals(kin - 1)
    inl = {}
    for nm in ("PO1", "TO1", "VTIN", "VM1", "BS", "BR"):
        c.skip()
        inl[nm] = np.zeros(max(kin, km) + 2, f32)
        inl[nm][1:kin + 1] = c.reals(kin)
    c.skip()
    pdown_hub, pdown_tip = c.reals(2)
    _geometric(fr, km)
    if kin == 2:
        fr_in[1], fr_in[2] = f32(1.0), f32(0.0)
    else:
        _geometric(fr_in, kin)
    _geometric(fp, im)
    # INPINT, 9073-9199: onto the KM points at the cumulative FR fractions
    sumfn = np.zeros(km + 2, f32)
    for k in range(2, km + 1):
        sumfn[k] = f32(sumfn[k - 1] + fr[k - 1])
    for k in range(2, km + 1):
        sumfn[k] = f32(sumfn[k] / sumfn[km])
    sumf_in = np.zeros(kin + 2, f32)
    for k in range(2, kin + 1):
        sumf_in[k] = f32(sumf_in[k - 1] + fr_in[k - 1])
    for k in range(2, kin + 1):
        sumf_in[k] = f32(sumf_in[k] / sumf_in[kin])
    inlet = {}
    for nm in ("PO1", "TO1", "VTIN", "VM1", "BR", "BS"):
        inlet[nm] = np.array([intp(kin, sumf_in, inl[nm], sumfn[k]) for k in range(1, km + 1)], f32)

    # ------------------ mixing-length limits, FACMIXUP, roughness ----------
    xllim = [(0.03, 0.03, 0.03, 0.03, 0.03, 0.02)] * nrows
    xllim_new = [(0.02, 0.03, 0.04, 0.05)] * nrows
    fsturb = [1.0] * nrows
    tdamp = [0.5] * nrows
    facmixup, nmixup = 2.0, 1000
    if ilos != 0:
        c.skip()
        for n in range(nrows):
            if ilos == 10:
                v = c.optional("rrrrrr", [f32(a) for a in xllim[n]])
                xllim[n] = tuple(float(a) for a in v)
            if ilos >= 100:
                v = c.optional("rrrrrr", [f32(a) for a in xllim_new[n]] + [f32(fsturb[n]), f32(tdamp[n])])
                xllim_new[n] = tuple(float(a) for a in v[:4])
                fsturb[n], tdamp[n] = float(v[4]), float(v[5])
        c.skip()
        fm, nmixup = c.optional("ri", [f32(2.0), 1000])
        facmixup = max(float(fm), 1.0)
        if if_restart:
            facmixup = 1.0
    rough = [(0.0, 0.0, 0.0, 0.0)] * nrows
    if if_rough > 0:
        c.skip()
        for n in range(nrows):
            rough[n] = tuple(float(f32(v * f32(1.0e-6))) for v in c.reals(4))

    # the sections NEW_INTPOL starts from (the device form of it takes these)
    sections = np.stack([g.xs[1:jm + 1, 1:nsecs_in + 1].T, g.rs[1:jm + 1, 1:nsecs_in + 1].T,
                         g.rtu[1:jm + 1, 1:nsecs_in + 1].T, g.rtt[1:jm + 1, 1:nsecs_in + 1].T]).astype(f32)
    fractip = np.array([[rw.fractip[0], rw.fractip[1]] for rw in rows], f32)

    # ------------------ NEW_INTPOL, 7493-7613 ------------------------------
    frn = fr.copy()
    s = f32(0.0)
    for k in range(1, km):
        s = f32(s + frn[k])
    for k in range(1, km):
        frn[k] = f32(frn[k] / s)
    for k in range(1, nsecs_in + 1):
        g.merid(k, jm)
    X = np.zeros((km, jm), f32)
    R = np.zeros((km, jm), f32)
    RTU = np.zeros((km, jm), f32)
    RTT = np.zeros((km, jm), f32)
    nrow_of = np.zeros(jm + 1, np.int32)
    for nr in range(1, nrows + 1):
        nrow_of[jstart[nr - 1]:jmix[nr - 1] + 1] = nr
    xi = np.zeros(maxk, f32)
    yi = np.zeros(maxk, f32)
    ru = np.zeros(maxk, f32)
    rt = np.zeros(maxk, f32)
    qod = np.zeros(maxk, f32)
    for j in range(1, jm + 1):
        nr = nrow_of[j]
        row = rows[nr - 1]
        jj1, jl, jt, je = jstart[nr - 1], jle_[nr - 1], jte_[nr - 1], jmix[nr - 1]
        frmod = frn.copy()
        if row.ktips > 0:
            ktip = 1 if row.ktips == 1 else nsecs_in
            ktipe = row.ktipe if row.ktips != 1 else row.ktipe
            if row.ktips > 1:
                ktipe = km
            ks1, ks2 = (ktipe, km - 1) if row.ktips == 1 else (1, row.ktips - 1)
            fac = 1.0
            tipgap = 0.0
            sm = g.smerid
            if jj1 <= j < jl:
                fac = float(f32(f32(sm[j, ktip] - sm[jj1, ktip]) / f32(sm[jl, ktip] - sm[jj1, ktip])))
                tipgap = float(row.fractip[0])
            if jl <= j <= jt:
                fac = 1.0
                frac = f32(f32(sm[j, ktip] - sm[jl, ktip]) / f32(sm[jt, ktip] - sm[jl, ktip]))
                tipgap = float(f32(row.fractip[0] + f32(frac * f32(row.fractip[1] - row.fractip[0]))))
            if jt < j <= je:
                fac = float(f32(f32(sm[je, ktip] - sm[j, ktip]) / f32(sm[je, ktip] - sm[jt, ktip])))
                tipgap = float(row.fractip[1])
            # FAC, TIPGAP, TIPSPACE and SUMFR are DOUBLE PRECISION here
            sumfr = 0.0
            ncell = ktipe - row.ktips
            tipspace = tipgap / ncell
            for k in range(row.ktips, ktipe):
                sumfr = sumfr + float(frn[k])
            for k in range(row.ktips, ktipe):
                frmod[k] = f32(tipspace * fac + (1.0 - fac) * float(frn[k]))
            for k in range(ks1, ks2 + 1):
                frmod[k] = f32(float(frn[k]) * ((1.0 - tipgap) / (1.0 - sumfr) * fac + (1.0 - fac)))
        qod[1] = f32(0.0)
        for k in range(1, nsecs_in + 1):
            xi[k], yi[k], ru[k], rt[k] = g.xs[j, k], g.rs[j, k], g.rtu[j, k], g.rtt[j, k]
            if k > 1:
                rd = f32(g.rs[j, k] - g.rs[j, k - 1])
                xd = f32(g.xs[j, k] - g.xs[j, k - 1])
                qod[k] = f32(qod[k - 1] + np.sqrt(f32(f32(xd * xd) + f32(rd * rd))))
        xarg = f32(0.0)
        qospan = qod[nsecs_in]
        for k in range(1, km + 1):
            X[k - 1, j - 1] = intp(nsecs_in, qod, xi, xarg)
            R[k - 1, j - 1] = intp(nsecs_in, qod, yi, xarg)
            RTU[k - 1, j - 1] = intp(nsecs_in, qod, ru, xarg)
            RTT[k - 1, j - 1] = intp(nsecs_in, qod, rt, xarg)
            xarg = f32(xarg + f32(frmod[k] * qospan))

    # ------------------ the spec and geometry for SETUP --------------------
    rowspecs = []
    for n, rw in enumerate(rows):
        rs = RowSpec(nblade=rw.nblades, jm=rw.jm, jle=rw.jle, jte=rw.jte, rpm=rw.rpm, rpm_hub=rw.rpm_hub,
                     pup=float(rw.pguess[0]), ple=float(rw.pguess[1]), pte=float(rw.pguess[2]),
                     pdn=float(rw.pguess[3]), stage=nstage[n], xllim=xllim[n], xllim_new=xllim_new[n],
                     fsturb=fsturb[n], turbvis_damp=tdamp[n], if_cusp=2 if rw.if_cusp == 2 else 0,
                     nup_i1=int(rw.sep[0]), nup_im=int(rw.sep[1]), n_wake=int(rw.sep[2]),
                     sep_thik=float(rw.sep[3]), sep_drag=float(rw.sep[4]), jrot=rw.jrot, jtran=rw.jtran,
                     rough=rough[n])
        rowspecs.append(rs)
    kmid = int(0.5 * km)
    spec = CaseSpec(name=name, im=im, km=km, rows=rowspecs, hub=None, casing=None,
                    po1=float(inlet["PO1"][kmid - 1]), to1=float(inlet["TO1"][kmid - 1]),
                    pdown_hub=float(pdown_hub), pdown_tip=float(pdown_tip), cp=float(cp), ga=float(ga),
                    cfl=float(cfl), itimst=itimst, nsteps_max=nsteps_max, conlim=float(conlim),
                    dampin=float(dampin), machlim=float(machlim), sfxin=float(sfxin), sftin=float(sftin),
                    fac_4th=float(fac_4th), nchange=nchange, ir=ir, jr=jr, kr=kr, irbb=irbb, jrbb=jrbb,
                    krbb=krbb, fblk=tuple(float(v) for v in fblk), ifmix=ifmix, rfmix=float(rfmix),
                    fextrap=float(fextrap), fsmthb=float(fsmthb), fangle=float(fangle), rfin=float(rfin),
                    ipout=ipout, reyno=float(reyno), rf_vis=float(rf_vis), ftrans=float(ftrans),
                    prandtl=float(prandtl), ypluswall=float(ypluswall), facmixup=facmixup, nmixup=nmixup,
                    nlos=nlos, ilos=ilos, fac_stmix=float(sa[0]), fac_st=tuple(float(v) for v in sa[1:5]),
                    fac_sfvis=float(sa[5]), fac_vort=float(sa[6]), fac_pgrad=float(sa[7]),
                    turbvis_lim=float(turbvis_lim), in_vr=in_vr, in_flow=in_flow, flowin=float(flowin),
                    rflow=float(rflow), plate_loss=float(plate_loss), throttle_exit=float(throttle_exit),
                    throttle_pres=float(throttle_pres), throttle_mas=float(throttle_mas),
                    rfthrotl=float(rfthrotl), inlet=inlet, ibound=ibound, in_vtan=in_vtan,
                    in_press=in_press, f_pdown=float(f_pdown), sfexit=float(sfexit), nsfexit=nsfexit,
                    yplam=float(yplam), ypturb=float(ypturb))
    geo = CaseGeometry(spec=spec, im=im, jm=jm, km=km, x=X, r=R, rt_upp=RTU, rt_thick=RTT,
                       fp=fp[1:im + 1].copy(), fr=fr[1:km + 1].copy(), row_first_j=list(jstart),
                       ktips=[rw.ktips for rw in rows], ktipe=[rw.ktipe for rw in rows],
                       fthick=np.stack([rw.fthick for rw in rows]).astype(f32), sections=sections, fractip=fractip)
    return spec, geo


def read_deck_file(path: str) -> tuple[CaseSpec, CaseGeometry]:
    import os
    with open(path, encoding="latin-1") as f:
        return read_deck(f.read(), os.path.basename(path))


# --------------------------------------------------------------------------
# Fixtures: what the reader leaves for SETUP, stored so that a machine
# without the reference's decks can rebuild the same COMMON state.
# --------------------------------------------------------------------------

_GEO_ARRAYS = ("x", "r", "rt_upp", "rt_thick", "fp", "fr", "fthick")


def save_fixture(path: str, spec: CaseSpec, geo: CaseGeometry, source: str = ""):
    """Writes spec and geometry to an .npz: the arrays as float32, the
    scalar and per-row cards as JSON."""
    import json
    sd = {f.name: getattr(spec, f.name) for f in dataclasses.fields(spec)
          if f.name not in ("rows", "hub", "casing", "inlet")}
    rows = [{f.name: getattr(r, f.name) for f in dataclasses.fields(r)} for r in spec.rows]
    meta = dict(spec=sd, rows=rows, im=geo.im, jm=geo.jm, km=geo.km, row_first_j=geo.row_first_j,
                ktips=geo.ktips, ktipe=geo.ktipe, source=source)
    arrays = {k: np.asarray(getattr(geo, k), f32) for k in _GEO_ARRAYS}
    if geo.sections is not None:
        arrays["sections"] = np.asarray(geo.sections, f32)
        arrays["fractip"] = np.asarray(geo.fractip, f32)
    for k, v in (spec.inlet or {}).items():
        arrays["inlet_" + k] = np.asarray(v, f32)
    np.savez_compressed(path, meta=np.array(json.dumps(meta, default=float)), **arrays)


def load_fixture(path: str) -> tuple[CaseSpec, CaseGeometry]:
    import json
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    rows = []
    for rd in meta["rows"]:
        rd = {k: (tuple(v) if isinstance(v, list) else v) for k, v in rd.items()}
        rows.append(RowSpec(**rd))
    sd = {k: (tuple(v) if isinstance(v, list) else v) for k, v in meta["spec"].items()}
    inlet = {k[len("inlet_"):]: z[k] for k in z.files if k.startswith("inlet_")} or None
    spec = CaseSpec(rows=rows, hub=None, casing=None, inlet=inlet, **sd)
    geo = CaseGeometry(spec=spec, im=meta["im"], jm=meta["jm"], km=meta["km"],
                       **{k: z[k] for k in _GEO_ARRAYS}, row_first_j=meta["row_first_j"],
                       ktips=meta["ktips"], ktipe=meta["ktipe"],
                       sections=z["sections"] if "sections" in z.files else None,
                       fractip=z["fractip"] if "fractip" in z.files else None)
    return spec, geo
