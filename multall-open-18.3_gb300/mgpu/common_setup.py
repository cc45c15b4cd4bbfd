"""Host-side stand-in for the part of Multall that stays outside the GPU
loop: the reader's per-row bookkeeping and SUBROUTINE SETUP.

In the reference, NEW_READIN (multall-open-18.3.f:148-2161) and SETUP
(6280-7487, with SET_XLENGTH 12194-12517) fill COMMON before `CALL LOOP`.
That Fortran is not compilable where this library is built, so this module
restates what those routines leave in COMMON for a generated case
(mgpu.case): face areas, volumes, the initial guess, the time steps and the
multigrid maps.  It produces the named COMMON data the mgpu C ABI binds
(include/mgpu_common_table.h).  It runs once per case, on the host, in
float32 like the reference.  The two calls SETUP makes into the hot path,
STEPUP(1.0) and the first LOSS, are left to the library
(mgpu_stepup / mgpu_loss_init), so that they run the GPU code.

Array layout: numpy C order with the Fortran indices reversed, i.e. A(I,J,K)
is stored as a[K-1, J-1, I-1]; a flat copy is the packed Fortran layout.
"""
from __future__ import annotations

import math
from typing import Dict

import numpy as np

from .case import CaseGeometry, CaseSpec, build_geometry

f32 = np.float32
PI = f32(3.14159265)            # multall-open-18.3.f:184
DEGRAD = f32(PI / f32(180.0))


class CommonData:
    """Named COMMON scalars and packed arrays for one case."""

    def __init__(self, im: int, jm: int, km: int, nrows: int):
        self.im, self.jm, self.km, self.nrows = im, jm, km, nrows
        self.ints: Dict[str, int] = {}
        self.reals: Dict[str, float] = {}
        self.arrays: Dict[str, np.ndarray] = {}

    def nodes(self) -> int:
        return self.im * self.jm * self.km


def _intp(n, xs, ys, x):
    return float(np.interp(x, xs[:n], ys[:n]))


def build_common(spec: CaseSpec, geo: CaseGeometry | None = None, metrics64: bool = False,
                 metrics_only: bool = False, theta_only: bool = False) -> CommonData:
    """The COMMON state SETUP leaves for the loop.  metrics64: also keep the
    face areas and volumes computed in double precision in cd.geom64;
    metrics_only: stop there (cd holds only geom64); theta_only: stop once
    the node angles THETA (KM, JM, IM) are formed (cd.theta)."""
    if geo is None:
        geo = build_geometry(spec, dtype=np.float64 if metrics64 else f32)
    IM, JM, KM = geo.im, geo.jm, geo.km
    NROWS = len(spec.rows)
    IMM1, JMM1, KMM1, IMM2, KMM2 = IM - 1, JM - 1, KM - 1, IM - 2, KM - 2
    IMID = int(0.5 * IM)
    KMID = int(0.5 * KM)
    cd = CommonData(IM, JM, KM, NROWS)

    # ---------------- reader bookkeeping per row / per J -----------------
    # (multall-open-18.3.f:1420-1535)
    JSTART = np.zeros(NROWS, np.int32)
    JMIX = np.zeros(NROWS, np.int32)
    JLE = np.zeros(NROWS, np.int32)
    JTE = np.zeros(NROWS, np.int32)
    JLED = np.zeros(NROWS, np.int32)
    KTIPS = np.zeros(NROWS, np.int32)
    KTIPE = np.zeros(NROWS, np.int32)
    KS1 = np.zeros(NROWS, np.int32)
    KS2 = np.zeros(NROWS, np.int32)
    IND = np.zeros(JM + 1, np.int32)       # 1-based scratch
    INDLE = np.zeros(JM + 1, np.int32)
    INDTE = np.zeros(JM + 1, np.int32)
    INDMIX = np.zeros(JM + 3, np.int32)
    INDMID = np.zeros(JM + 1, np.int32)
    NBLADE = np.zeros(JM + 1, np.int32)
    NROW = np.zeros(JM + 1, np.int32)
    WRAD = np.zeros(JM + 1, f32)
    WHUB = np.zeros(JM + 1, f32)
    WTIP = np.zeros(JM + 1, f32)
    PGUESS = np.zeros(JM + 1, f32)
    J1 = 1
    for nr, row in enumerate(spec.rows, start=1):
        JMROW, JLEROW, JTEROW = row.jm, row.jle, row.jte
        JLE[nr - 1] = J1 + JLEROW - 1
        JTE[nr - 1] = J1 + JTEROW - 1
        J2 = J1 - 1 + JMROW
        kt, ke = geo.ktips[nr - 1], geo.ktipe[nr - 1]
        if kt <= 0:
            ke = 0
        KTIPS[nr - 1], KTIPE[nr - 1] = kt, ke
        if kt <= 0:
            KS1[nr - 1], KS2[nr - 1] = 1, KMM1
        elif kt == 1:
            KS1[nr - 1], KS2[nr - 1] = ke, KMM1
        else:
            KS1[nr - 1], KS2[nr - 1] = 1, kt - 1
            KTIPE[nr - 1] = KM
        # the rotating parts of the hub and casing (reader 940-960); by
        # default the hub rotates over the whole row, the casing not
        JROTHS, JROTHE, JROTTS, JROTTE = row.jrot if row.jrot is not None else (1, JMROW, JMROW, JMROW)
        JMIDRW = int(0.5 * (JLEROW + JTEROW))
        JROW = 0
        for J in range(J1, J2 + 1):
            JROW += 1
            WRAD[J] = f32(f32(row.rpm) * PI / f32(30.0))
            WHUB[J] = f32(f32(row.rpm_hub) * PI / f32(30.0)) if (JROTHS < JROW < JROTHE) else f32(0)
            WTIP[J] = WRAD[J] if (JROTTS < JROW < JROTTE) else f32(0)
            NBLADE[J] = row.nblade
            NROW[J] = nr
            if JLEROW < JROW <= JTEROW:
                IND[J] = 1
            if JROW == JLEROW:
                INDLE[J] = 1
                JLED[nr - 1] = J
                INDLE[J - 1] = -1
                INDLE[J - 2] = -2
            if JROW == JTEROW:
                INDTE[J] = 1
            if JROW == JMIDRW:
                INDMID[J] = 1
            pu, pl, pt, pd = f32(row.pup), f32(row.ple), f32(row.pte), f32(row.pdn)
            if JROW <= JLEROW:
                PGUESS[J] = pu + (pl - pu) * f32(JROW - 1) / f32(JLEROW - 1)
            if JLEROW < JROW <= JTEROW:
                PGUESS[J] = pl + (pt - pl) * f32(JROW - JLEROW) / f32(JTEROW - JLEROW)
            if JROW > JTEROW:
                PGUESS[J] = pt + (pd - pt) * f32(JROW - JTEROW) / f32(JMROW - JTEROW)
        INDMIX[J2] = 1
        JMIX[nr - 1] = J2
        JSTART[nr - 1] = J1
        J1 = J2 + 1
    INDMIX[JM] = 0
    NSTAGES = spec.rows[-1].stage

    # ---------------- inlet boundary data on the KM grid points ----------
    if spec.inlet is not None:
        # a deck's inlet cards as INPINT interpolated them (9073-9199)
        PO1, TO1, VTIN, VM1, BS, BR = (np.asarray(spec.inlet[n], f32).copy()
                                       for n in ("PO1", "TO1", "VTIN", "VM1", "BS", "BR"))
    else:
        PO1 = np.full(KM, f32(spec.po1), f32)
        TO1 = np.full(KM, f32(spec.to1), f32)
        VTIN = np.zeros(KM, f32)
        BS = np.zeros(KM, f32)
        BR = np.zeros(KM, f32)
        # VM1: the inlet meridional speed of the initial guess, isentropic from
        # P0 to the first row's upstream pressure guess
        pr = spec.rows[0].pup / spec.po1
        vm1 = math.sqrt(max(2.0 * spec.cp * spec.to1 * (1.0 - pr ** ((spec.ga - 1) / spec.ga)), 1.0))
        VM1 = np.full(KM, f32(vm1), f32)

    # ---------------- SETUP (multall-open-18.3.f:6280-7487) ---------------
    BSSIN = np.sin(BS * DEGRAD).astype(f32)
    BSCOS = np.cos(BS * DEGRAD).astype(f32)
    BRSIN = np.sin(BR * DEGRAD).astype(f32)
    BRCOS = np.cos(BR * DEGRAD).astype(f32)
    FR = geo.fr.astype(f32).copy()            # length KM, FR(KM)=0
    s = f32(0.0)
    for k in range(KMM1):
        s = f32(s + FR[k])
    FR[:KMM1] = (FR[:KMM1] / s).astype(f32)
    FP = geo.fp.astype(f32).copy()
    s = f32(0.0)
    for i in range(IMM1):
        s = f32(s + FP[i])
    FP[:IMM1] = (FP[:IMM1] / s).astype(f32)
    FU = np.zeros(IM, f32)
    FD = np.zeros(IM, f32)
    for i in range(2, IMM1 + 1):
        FU[i - 1] = FP[i - 1] / (FP[i - 1] + FP[i - 2])
        FD[i - 1] = FP[i - 2] / (FP[i - 1] + FP[i - 2])
    FU[0] = FP[0] / FP[1]
    FU[IM - 1] = FP[IMM1 - 1] / FP[IMM2 - 1]
    FKU = np.zeros(KM, f32)
    FKD = np.zeros(KM, f32)
    for k in range(2, KMM1 + 1):
        FKU[k - 1] = FR[k - 1] / (FR[k - 1] + FR[k - 2])
        FKD[k - 1] = FR[k - 2] / (FR[k - 1] + FR[k - 2])
    FKU[0] = FR[0] / FR[1]
    FKU[KM - 1] = FR[KMM1 - 1] / FR[KMM2 - 1]
    # corner distribution weights, 2006-2008
    FTL = np.zeros((KM, IM), f32)
    FBL = np.zeros((KM, IM), f32)
    FTR = np.zeros((KM, IM), f32)
    FBR = np.zeros((KM, IM), f32)
    for a in (FTL, FBL, FTR, FBR):
        a[:KMM1, :IMM1] = 0.125
    FTL[:KMM1, 0] = 0.25
    FBL[:KMM1, 0] = 0.25
    FTR[:KMM1, IMM1 - 1] = 0.25
    FBR[:KMM1, IMM1 - 1] = 0.25
    FBL[0, :IMM1] = 0.25
    FBR[0, :IMM1] = 0.25
    FTL[KMM1 - 1, :IMM1] = 0.25
    FTR[KMM1 - 1, :IMM1] = 0.25
    FTL[KMM1 - 1, 0] = 0.5
    FBL[0, 0] = 0.5
    FTR[KMM1 - 1, IMM1 - 1] = 0.5
    FBR[0, IMM1 - 1] = 0.5
    FACUP = np.zeros(JM, f32)
    FACDWN = np.zeros(JM, f32)
    FACUP[1:] = 1.0
    FACDWN[1:] = 1.0
    FACUP[1] = 2.0
    FACDWN[JM - 1] = 2.0

    dt = np.float64 if metrics64 else f32
    X = geo.x.astype(dt)            # (KM, JM)
    R = geo.r.astype(dt)
    RT_UPP = geo.rt_upp.astype(dt).copy()
    RT_THICK = geo.rt_thick.astype(dt).copy()
    # align the blades circumferentially across mixing planes, 3022
    SHIFT = dt(0.0)
    for J in range(3, JM + 1):
        if INDMIX[J - 1] == 1:
            SHIFT = dt((RT_UPP[KMID - 1, J - 2] - RT_UPP[KMID - 1, J - 1]) / R[KMID - 1, J - 1])
        RT_UPP[:, J - 1] = (RT_UPP[:, J - 1] + SHIFT * R[:, J - 1]).astype(dt)
    # pinched-tip thickness scaling, 2506
    for J in range(1, JM + 1):
        nr = NROW[J]
        rtmid = RT_UPP[:, J - 1] - dt(0.5) * RT_THICK[:, J - 1]
        thick = geo.fthick[nr - 1] * RT_THICK[:, J - 1]
        RT_UPP[:, J - 1] = (rtmid + dt(0.5) * thick).astype(dt)
        RT_THICK[:, J - 1] = thick.astype(dt)
    CP, GA = dt(spec.cp), dt(spec.ga)
    GA1 = dt(GA - dt(1.0))
    FGA = dt(GA1 / GA)
    RFGA = dt(dt(1.0) / FGA)
    CV = dt(CP / GA)
    RGAS = dt(CP - CV)

    # theta / r*theta of the grid nodes, 3000
    NB = NBLADE[1:JM + 1].astype(dt)                     # per J
    PITCH = (dt(2.0) * dt(PI) / NB).astype(dt)              # (JM,)
    GAP = (PITCH[None, :] * R - RT_THICK).astype(dt)     # (KM, JM)
    RTHETA = np.zeros((KM, JM, IM), dt)
    RTHETA[:, :, 0] = RT_UPP
    for i in range(2, IM + 1):
        RTHETA[:, :, i - 1] = RTHETA[:, :, i - 2] + dt(FP[i - 2]) * GAP
    THETA = (RTHETA / R[:, :, None]).astype(dt)
    if theta_only:
        # the node angles alone (design sensitivities through dJ/dTHETA)
        cd.theta = THETA
        return cd
    # meridional distances 3530
    SMERID = np.zeros((KM, JM), dt)
    DR = np.zeros((KM, JM), dt)
    DX = np.zeros((KM, JM), dt)
    DS = np.zeros((KM, JM), dt)
    DR[:, 1:] = R[:, 1:] - R[:, :-1]
    DX[:, 1:] = X[:, 1:] - X[:, :-1]
    DS[:, 1:] = np.sqrt(DR[:, 1:] * DR[:, 1:] + DX[:, 1:] * DX[:, 1:])
    for J in range(2, JM + 1):
        SMERID[:, J - 1] = SMERID[:, J - 2] + DS[:, J - 1]
    DSMIN = dt(DS[:, 1:].min())
    DX[:, 0] = DX[:, 1]
    DS[:, 0] = DS[:, 1]
    DR[:, 0] = DR[:, 1]
    CHORD = np.zeros(NROWS, dt)
    for nr in range(1, NROWS + 1):
        jl, jt = JLE[nr - 1], JTE[nr - 1]
        sch = SMERID[KMID - 1, jt - 1] - SMERID[KMID - 1, jl - 1]
        tch = RTHETA[KMID - 1, jl - 1, 0] - RTHETA[KMID - 1, jt - 1, 0]
        CHORD[nr - 1] = np.sqrt(sch * sch + tch * tch)
    RAVG_CELL = np.zeros((KM, JM), dt)
    RAVG_CELL[:KMM1, 1:] = dt(0.25) * (R[:KMM1, 1:] + R[:KMM1, :-1] + R[1:, :-1] + R[1:, 1:])
    UBLADE = (WRAD[1:JM + 1][None, :].astype(dt) * R).astype(dt)
    # theta extrapolated onto the upstream side of each mixing plane, 3025
    TEMP1 = np.zeros((KM, JM, IM), dt)
    TEMP2 = np.zeros((KM, JM, IM), dt)
    for J in range(1, JM + 1):
        if INDMIX[J] != 1:
            continue
        fac = (DS[:, J] / DS[:, J + 1]).astype(dt)          # DS(J+1)/DS(J+2)
        TEMP1[:, J - 1, :] = THETA[:, J, :] + fac[:, None] * (THETA[:, J, :] - THETA[:, J + 1, :])
        TEMP2[:, J - 1, :] = R[:, J - 1][:, None] * TEMP1[:, J - 1, :]

    # ---------------- face areas and volumes, 3030-4045 -------------------
    AQX = np.zeros((KM, JM, IM), dt)
    AQR = np.zeros((KM, JM, IM), dt)
    X1 = (X[1:, :] - X[:-1, :])[:, :, None]
    R1 = (R[1:, :] - R[:-1, :])[:, :, None]
    Rk = R[:-1, :][:, :, None]
    Rkp = R[1:, :][:, :, None]
    T1 = Rkp * (THETA[1:, :, 1:] - THETA[:-1, :, :-1])
    T2 = Rkp * (THETA[1:, :, :-1] - THETA[:-1, :, :-1]) - Rk * (THETA[:-1, :, 1:] - THETA[:-1, :, :-1])
    AQX[:KMM1, :, :IMM1] = dt(-0.5) * (R1 * T1 - R1 * T2)
    AQR[:KMM1, :, :IMM1] = dt(-0.5) * (X1 * T2 - X1 * T1)
    AQTOT = np.sqrt(AQX * AQX + AQR * AQR).astype(dt)
    AQX[KM - 1, :, :IMM1] = AQX[KMM1 - 1, :, :IMM1]
    AQR[KM - 1, :, :IMM1] = AQR[KMM1 - 1, :, :IMM1]
    AQX[:, :, IM - 1] = AQX[:, :, IMM1 - 1]
    AQR[:, :, IM - 1] = AQR[:, :, IMM1 - 1]

    ABT = np.zeros((KM, JM), dt)
    WRABT = np.zeros((KM, JM), dt)
    ABX = np.zeros((KM, JM, IM), dt)
    ABR = np.zeros((KM, JM, IM), dt)
    ABTOT = np.zeros((KM, JM, IM), dt)
    VOL = np.zeros((KM, JM, IM), dt)
    bx1 = X[1:, :-1] - X[:-1, 1:]          # X(J-1,K+1)-X(J,K), (KMM1, JMM1) over J=2..JM
    bx2 = X[1:, 1:] - X[:-1, :-1]          # X(J,K+1)-X(J-1,K)
    br1 = R[1:, :-1] - R[:-1, 1:]
    br2 = R[1:, 1:] - R[:-1, :-1]
    ABT[:KMM1, 1:] = dt(-0.5) * (bx1 * br2 - bx2 * br1)
    WRABT[:KMM1, 1:] = (WRAD[2:JM + 1][None, :].astype(dt) * dt(0.25) *
                        (R[:-1, 1:] + R[:-1, :-1] + R[1:, :-1] + R[1:, 1:]) * ABT[:KMM1, 1:])
    mixprev = np.array([INDMIX[J - 1] == 1 for J in range(2, JM + 1)])      # INDMIX(J-1), J=2..JM
    THm = np.where(mixprev[None, :, None], TEMP1[:, :-1, :], THETA[:, :-1, :])   # theta at J-1 (KM, JMM1, IM)
    RTm = np.where(mixprev[None, :, None], TEMP2[:, :-1, :], RTHETA[:, :-1, :])
    Rjm1_kp = R[1:, :-1][:, :, None]
    Rj_kp = R[1:, 1:][:, :, None]
    Rjm1_k = R[:-1, :-1][:, :, None]
    th_jk = THETA[:-1, 1:, :]
    T1 = Rjm1_kp * (THm[1:, :, :] - th_jk)
    T2 = Rj_kp * (THETA[1:, 1:, :] - th_jk) - Rjm1_k * (THm[:-1, :, :] - th_jk)
    ABX[:KMM1, 1:, :] = dt(-0.5) * (br1[:, :, None] * T2 - br2[:, :, None] * T1)
    ABR[:KMM1, 1:, :] = dt(-0.5) * (bx2[:, :, None] * T1 - bx1[:, :, None] * T2)
    ABTOT[:KMM1, 1:, :] = np.sqrt(ABX[:KMM1, 1:, :] ** 2 + ABR[:KMM1, 1:, :] ** 2 +
                                  ABT[:KMM1, 1:, None] ** 2)
    VOL[:KMM1, 1:, :IMM1] = ABT[:KMM1, 1:, None] * dt(0.25) * (
        RTHETA[:-1, 1:, 1:] + RTm[:-1, :, 1:] + RTm[1:, :, 1:] + RTHETA[1:, 1:, 1:]
        - RTHETA[:-1, 1:, :-1] - RTm[:-1, :, :-1] - RTm[1:, :, :-1] - RTHETA[1:, 1:, :-1])

    ASX = np.zeros((KM, JM, IM), dt)
    ASR = np.zeros((KM, JM, IM), dt)
    sx1 = (X[:, :-1] - X[:, 1:])[:, :, None]           # X(J-1,K)-X(J,K)
    sr1 = (R[:, :-1] - R[:, 1:])[:, :, None]
    Rjm1 = R[:, :-1][:, :, None]
    Rj = R[:, 1:][:, :, None]
    th = THETA[:, 1:, :-1]                              # THETA(I,J,K)
    T1 = Rjm1 * (THm[:, :, :-1] - th) - Rj * (THETA[:, 1:, 1:] - th)
    T2 = Rjm1 * (THm[:, :, 1:] - th)
    ASX[:, 1:, :IMM1] = dt(0.5) * (sr1 * T2 - sr1 * T1)
    ASR[:, 1:, :IMM1] = dt(0.5) * (sx1 * T1 - sx1 * T2)

    VOLOR = np.zeros((KM, JM, IM), dt)
    RAREA = (ABR[:KMM1, 1:, :IMM1] - ABR[:KMM1, 1:, 1:] + AQR[:KMM1, 1:, :IMM1] - AQR[:KMM1, :-1, :IMM1]
             + ASR[:KMM1, 1:, :IMM1] - ASR[1:, 1:, :IMM1])
    VOLOR[:KMM1, 1:, :IMM1] = dt(-0.125) * RAREA
    if metrics64:
        # the face areas and volumes in double precision (geometry
        # sensitivities); the deck itself continues in REAL*4
        cd.geom64 = dict(X=X.copy(), R=R.copy(), RTHETA=RTHETA.copy(), WRABT=WRABT.copy(),
                         AQX=AQX.copy(), AQR=AQR.copy(), ABX=ABX.copy(), ABR=ABR.copy(), ABT=ABT.copy(),
                         ASX=ASX.copy(), ASR=ASR.copy(), VOLOR=VOLOR.copy(), VOL=VOL.copy())
        if metrics_only:
            return cd
        (X, R, RT_UPP, RT_THICK, RTHETA, THETA, SMERID, DR, DX, DS, RAVG_CELL, UBLADE, AQX, AQR, AQTOT, ABT, WRABT,
         ABX, ABR, ABTOT, VOL, ASX, ASR, VOLOR, CHORD, GA1, FGA, RFGA, CV, RGAS, CP, GA, DSMIN) = (
            np.asarray(v).astype(f32) if isinstance(v, np.ndarray) else f32(v)
            for v in (X, R, RT_UPP, RT_THICK, RTHETA, THETA, SMERID, DR, DX, DS, RAVG_CELL, UBLADE, AQX, AQR,
                      AQTOT, ABT, WRABT, ABX, ABR, ABTOT, VOL, ASX, ASR, VOLOR, CHORD, GA1, FGA, RFGA, CV, RGAS,
                      CP, GA, DSMIN))

    # ---------------- initial guess, 3211-3500 -----------------------------
    PD = np.zeros(KM, f32)
    PD[0] = f32(spec.pdown_hub)
    for k in range(2, KM + 1):
        PD[k - 1] = PD[k - 2] + FR[k - 2] * f32(spec.pdown_tip - spec.pdown_hub)
    RPO1 = (f32(1.0) / PO1).astype(f32)
    P = np.zeros((KM, JM, IM), f32)
    RO = np.zeros((KM, JM, IM), f32)
    T_STATIC = np.zeros((KM, JM, IM), f32)
    PS = PGUESS[1:JM + 1][None, :]
    PRAT = (PS / PO1[:, None]).astype(f32)
    TS = (PRAT ** FGA * TO1[:, None]).astype(f32)
    ROS = (PS / TS / RGAS).astype(f32)
    P[:] = np.broadcast_to(PS[:, :, None], P.shape)
    RO[:] = ROS[:, :, None]
    T_STATIC[:] = TS[:, :, None]
    KAVG = int(0.75 * KM)
    VT = np.zeros((KM, JM, IM), f32)
    WT = np.zeros((KM, JM, IM), f32)
    VX = np.zeros((KM, JM, IM), f32)
    VR = np.zeros((KM, JM, IM), f32)
    HO = np.zeros((KM, JM, IM), f32)
    VT[:, 0, :] = VTIN[:, None]
    WT[:, 0, :] = (VTIN - UBLADE[:, 0])[:, None]
    HO[:, 0, :] = (CP * TO1)[:, None]
    FACJ = f32(0.9)
    AIN = f32(0)
    for J in range(2, JM + 1):
        if J > 2 and INDTE[J - 2] == 1:
            FACJ = f32(1.0)
        a = AQX[KAVG - 1, J - 1, IMID - 1]
        b = AQR[KAVG - 1, J - 1, IMID - 1]
        AREA = f32(np.sqrt(a * a + b * b) * f32(NBLADE[J]))
        if J == 2:
            AIN = AREA
        VS = f32(VM1[KAVG - 1] * AIN * RO[KAVG - 1, 0, IMID - 1] / (AREA * RO[KAVG - 1, J - 1, IMID - 1]))
        Rj = R[:, J - 1][:, None]
        Rjm = R[:, J - 2][:, None]
        VTGRID = VS * Rj * (THETA[:, J - 1, :] - THETA[:, J - 2, :]) / DS[:, J - 1][:, None] + UBLADE[:, J - 1][:, None]
        vt = (f32(1.0) - FACJ) * VTGRID + FACJ * VT[:, J - 2, :] * Rjm / Rj
        if INDMIX[J - 1] == 1:
            vt = VT[:, J - 2, :].copy()
        if J < JLE[0]:
            vt = np.broadcast_to((VTIN * R[:, 0] / R[:, J - 1])[:, None], vt.shape).copy()
        VT[:, J - 1, :] = vt
        WT[:, J - 1, :] = vt - UBLADE[:, J - 1][:, None]
        VX[:, J - 1, :] = (VS * DX[:, J - 1] / DS[:, J - 1])[:, None]
        VR[:, J - 1, :] = (VS * DR[:, J - 1] / DS[:, J - 1])[:, None]
        HO[:, J - 1, :] = HO[:, J - 2, :] + WRAD[J] * (Rj * VT[:, J - 1, :] - Rjm * VT[:, J - 2, :])
        if INDLE[J] == 1:
            FACJ = f32(0.9)
    VR[:, 0, :] = VR[:, 1, :]
    VX[:, 0, :] = VX[:, 1, :]
    WT[:, 0, :] = WT[:, 1, :]
    PREFF = f32(0.5) * (P[KMID - 1, 0, IMID - 1] + P[KMID - 1, JM - 1, IMID - 1])
    EKE = f32(0.5) * (VX ** 2 + VT ** 2 + VR ** 2)
    ROE = (P / (GA - f32(1)) + EKE * RO).astype(f32)
    ROVR = (RO * VR).astype(f32)
    ROVT = (RO * VT).astype(f32)
    ROWT = (RO * WT).astype(f32)
    RORVT = (ROVT * R[:, :, None]).astype(f32)
    ROVX = (RO * VX).astype(f32)
    PEFF = (P - PREFF).astype(f32)
    zeros3 = np.zeros((KM, JM, IM), f32)

    # ---------------- time steps, 7012-7052 --------------------------------
    VSOUND = f32(np.sqrt(RGAS * GA * TO1[KMID - 1]))
    with np.errstate(divide="ignore", invalid="ignore"):
        ATTOT = np.sqrt(ABT[:KMM1, 1:, None] ** 2 + ABX[:KMM1, 1:, :IMM1] ** 2 + ABR[:KMM1, 1:, :IMM1] ** 2)
        vol = VOL[:KMM1, 1:, :IMM1]
        PERPT = vol / ATTOT
        PERPQ = vol / AQTOT[:KMM1, 1:, :IMM1]
        ASTOT = np.sqrt(ASX[:KMM1, 1:, :IMM1] ** 2 + ASR[:KMM1, 1:, :IMM1] ** 2)
        PERPS = vol / ASTOT
        SMIN = np.minimum(np.minimum(PERPT, PERPQ), PERPS)
        STEP = np.zeros((KM, JM, IM), f32)
        STEP[:KMM1, 1:, :IMM1] = SMIN * f32(spec.cfl) / vol / VSOUND
    BSTEP = STEP.copy()
    RSTEP = np.zeros((KM, JM, IM), f32)
    RSTEP[:KMM1, 1:, :IMM1] = 1.0
    for nr in range(1, NROWS):
        J = JMIX[nr - 1]
        STEP[:KMM1, J, :IMM1] = f32(0.5) * (STEP[:KMM1, J - 1, :IMM1] + STEP[:KMM1, J + 1, :IMM1])
        BSTEP[:KMM1, J, :IMM1] = STEP[:KMM1, J, :IMM1]
        RSTEP[:KMM1, J, :IMM1] = 0.0

    # ---------------- multigrid maps and block time steps, 7067-7279 ------
    IR, JR, KR = spec.ir, spec.jr, spec.kr
    IRBB, JRBB, KRBB = spec.irbb, spec.jrbb, spec.krbb
    KB1 = np.array([1 + (k - 1) // KR for k in range(1, KM + 1)], np.int32)
    KB2 = np.array([1 + (k - 1) // KRBB for k in range(1, KM + 1)], np.int32)
    IB1 = np.array([1 + (i - 1) // IR for i in range(1, IM + 1)], np.int32)
    IB2 = np.array([1 + (i - 1) // IRBB for i in range(1, IM + 1)], np.int32)
    NKB1, NKB2 = int(KB1[KMM1 - 1]), int(KB2[KMM1 - 1])
    NIB1, NIB2 = int(IB1[IMM1 - 1]), int(IB2[IMM1 - 1])
    JB1 = np.zeros(JM + 1, np.int32)
    JB2 = np.zeros(JM + 1, np.int32)
    JSTT = 2
    JB1[1] = JB1[2] = 1
    for J in range(3, JM + 1):
        mark = INDMIX[J] == 1 or J == JM
        JB1[J] = JB1[J - 1] + 1 if ((J - JSTT) % JR == 0 and not mark) else JB1[J - 1]
        if INDMIX[J - 1] == 1:
            JB1[J] = 0
        if INDMIX[J - 2] == 1:
            JB1[J] = JB1[J - 2] + 1
            JSTT = J
    JSTT = 2
    JB2[1] = JB2[2] = 1
    for J in range(3, JM + 1):
        JP1 = JM if J == JM else J + 1
        mark = INDMIX[J] == 1 or J == JM or INDMIX[JP1] == 1 or (J + 1) == JM
        JB2[J] = JB2[J - 1] + 1 if ((J - JSTT) % JRBB == 0 and not mark) else JB2[J - 1]
        if INDMIX[J - 1] == 1:
            JB2[J] = 0
        if INDMIX[J - 2] == 1:
            JB2[J] = JB2[J - 2] + 1
            JSTT = J
    NJB1, NJB2 = int(JB1[JM]), int(JB2[JM])
    JSTART1 = np.zeros(max(NJB1, JM) + 3, np.int32)
    JEND1 = np.zeros_like(JSTART1)
    JSTART2 = np.zeros(max(NJB2, JM) + 3, np.int32)
    JEND2 = np.zeros_like(JSTART2)
    JSTART1[1] = JSTART2[1] = 2
    for J in range(2, JM + 1):
        if JB1[J] == 0:
            JB1[J] = NJB1 + 1
        if JB2[J] == 0:
            JB2[J] = NJB2 + 1
        if JB1[J] != JB1[J - 1]:
            JSTART1[JB1[J]] = J
        JEND1[JB1[J]] = J
        if JB2[J] != JB2[J - 1]:
            JSTART2[JB2[J]] = J
        JEND2[JB2[J]] = J
    JSTART1[NJB1 + 1] = JEND1[NJB1 + 1] = JM
    JSTART2[NJB2 + 1] = JEND2[NJB2 + 1] = JM
    JSBLK = np.zeros(JM + 1, np.int32)
    nsb = 1
    for J in range(1, JM + 1):
        JSBLK[J] = nsb
        if INDLE[J] == 1:
            nsb += 1
        if INDMID[J] == 1:
            nsb += 1
        if INDTE[J] == 1:
            nsb += 1
    NSBLK = int(JSBLK[JM])

    with np.errstate(divide="ignore", invalid="ignore"):
        ATT = np.sqrt(ABT[:, :, None] ** 2 + ABX ** 2 + ABR ** 2)      # (KM,JM,IM)
        AST = np.sqrt(ASX ** 2 + ASR ** 2)
        pT = (VOL / ATT).astype(f32)
        pQ = (VOL / AQTOT).astype(f32)
        pS = (VOL / AST).astype(f32)

    def block_steps(NIB, NJB, NKB, ir_, jr_, kr_, JSTARTb, JENDb, fblk):
        out = np.zeros((NKB, NJB + 1, NIB), f32)         # STEPn(I,J,K) packed
        for i1 in range(1, NIB + 1):
            ist = (i1 - 1) * ir_ + 1
            ien = min(ist + ir_ - 1, IMM1)
            for j1 in range(1, NJB + 1):
                jst, jen = JSTARTb[j1], JENDb[j1]
                for k1 in range(1, NKB + 1):
                    kst = (k1 - 1) * kr_ + 1
                    ken = min(kst + kr_ - 1, KMM1)
                    sl = (slice(kst - 1, ken), slice(jst - 1, jen), slice(ist - 1, ien))
                    perpt = f32(pT[sl].astype(np.float64).sum())
                    perpq = f32(pQ[sl].astype(np.float64).sum())
                    perps = f32(pS[sl].astype(np.float64).sum())
                    volb = f32(VOL[sl].astype(np.float64).sum())
                    perps = perps / f32(ir_ * jr_)
                    perpt = perpt / f32(jr_ * kr_)
                    perpq = perpq / f32(ir_ * kr_)
                    pmin = min(perps, perpt, perpq)
                    out[k1 - 1, j1 - 1, i1 - 1] = f32(spec.cfl) * f32(fblk) * pmin / VSOUND / volb
                    out[k1 - 1, NJB, i1 - 1] = 0.0
        return out

    STEP1 = block_steps(NIB1, NJB1, NKB1, IR, JR, KR, JSTART1, JEND1, spec.fblk[0])
    STEP2 = block_steps(NIB2, NJB2, NKB2, IRBB, JRBB, KRBB, JSTART2, JEND2, spec.fblk[1])
    STEPSBK = np.zeros(NSBLK, f32)
    perpq = 0.0
    volb = 0.0
    for J in range(2, JM + 1):
        jsb = JSBLK[J]
        perpq += float(pQ[:KMM1, J - 1, :IMM1].astype(np.float64).sum())
        volb += float(VOL[:KMM1, J - 1, :IMM1].astype(np.float64).sum())
        if J == JM or JSBLK[J + 1] != jsb:
            pav = f32(perpq) / f32(IMM1 * KMM1)
            STEPSBK[jsb - 1] = f32(spec.cfl) * f32(spec.fblk[2]) * pav / VSOUND / f32(volb)
            perpq = 0.0
            volb = 0.0

    # ---------------- wall distance (SET_XLENGTH, 12194-12517) -------------
    DWALLSQ, DIST = wall_distance_sq(IM, JM, KM, X, R, THETA, ASX, ASR, ABX, ABR, ABT, JSTART, JMIX, JLE, JTE,
                                     NROW, NBLADE, IMID, spec, with_dist=True)
    new_loss = {}
    if spec.ilos >= 100:
        new_loss = mixing_lengths(spec, IM, JM, KM, DIST, SMERID, JSTART, JMIX, JLE, JTE, NROW, IMID, KMID)
        # cell-average density: the initial guess's node values (6796) until
        # the first step forms it (4255-4267)
        new_loss["ROAVG_CELL"] = RO.copy()
        # vorticity limit (7322-7328)
        DR1, DX1 = R[KM - 1, 0] - R[0, 0], X[KM - 1, 0] - X[0, 0]
        DRM, DXM = R[KM - 1, JM - 1] - R[0, JM - 1], X[KM - 1, JM - 1] - X[0, JM - 1]
        AVGSPAN = f32(0.5) * (np.sqrt(f32(DX1 * DX1 + DR1 * DR1)) + np.sqrt(f32(DXM * DXM + DRM * DRM)))
        new_loss_vort = float(f32(5000.0) * VM1[KMID - 1] / AVGSPAN)

    # ---------------- publish --------------------------------------------
    # the wall shear stress of the YPLUSWALL model (reader 2083-2088)
    cfwall = float(f32(1.0) / (f32(spec.ypluswall) * f32(spec.ypluswall))) if spec.ypluswall > 5.0 else 0.0
    ints = dict(ITIMST=3, ILOS=spec.ilos, NLOS=spec.nlos, IBOUND=spec.ibound, IFMIX=spec.ifmix, IPOUT=spec.ipout,
                IN_PRESS=spec.in_press, IN_VTAN=spec.in_vtan, IN_VR=spec.in_vr, IN_FLOW=spec.in_flow, IF_REPEAT=0,
                NRSMTH=0, NSFEXIT=spec.nsfexit,
                NSTEPS_MAX=spec.nsteps_max, NCHANGE=spec.nchange, NMIXUP=spec.nmixup, IF_RESTART=0,
                IR=IR, JR=JR, KR=KR, NIB1=NIB1, NJB1=NJB1, NKB1=NKB1, NIB2=NIB2, NJB2=NJB2,
                NKB2=NKB2, NSBLK=NSBLK, NSTAGES=NSTAGES, IFGAS=0, IFCOOL=0, IFBLEED=0, IFSHROUD=0)
    if spec.itimst == -3:
        ints["NRSMTH"] = 1
    reals = dict(CP=spec.cp, GA=spec.ga, CFL=spec.cfl, DAMPIN=spec.dampin, MACHLIM=spec.machlim,
                 F_PDOWN=spec.f_pdown, SFXIN=spec.sfxin, SFTIN=spec.sftin, FAC_4TH=spec.fac_4th, RFIN=spec.rfin,
                 FEXTRAP=spec.fextrap, RFMIX=spec.rfmix, FSMTHB=spec.fsmthb, FANGLE=spec.fangle,
                 SFEXIT=spec.sfexit, RSMTH=0.4, F1=2.0, F2=-1.0, F3=0.0, REYNO=spec.reyno, RF_VIS=spec.rf_vis,
                 FTRANS=spec.ftrans, PRANDTL=spec.prandtl, YPLUSWALL=spec.ypluswall, YPLAM=spec.yplam,
                 YPTURB=spec.ypturb, CFWALL=cfwall, FACMIXUP=spec.facmixup, PDOWN_HUB=spec.pdown_hub,
                 PDOWN_TIP=spec.pdown_tip, PLATE_LOSS=spec.plate_loss, THROTTLE_EXIT=spec.throttle_exit,
                 THROTTLE_PRES=spec.throttle_pres, THROTTLE_MAS=spec.throttle_mas, RFTHROTL=spec.rfthrotl,
                 FLOWIN=spec.flowin, RFLOW=spec.rflow, VSOUND=float(VSOUND),
                 CONLIM=spec.conlim, VISLAM=0.0, FTCOND=0.0)
    if spec.itimst == -3:
        reals.update(F2=-1.65, F3=-0.65)
    reals["TURBVIS_LIM"] = spec.turbvis_lim
    if new_loss:
        reals["VORT_MAX"] = new_loss_vort
    if spec.ilos >= 200:
        # the Spalart-Allmaras cards (reader 631-652, 2070-2073)
        reals.update(FAC_STMIX=spec.fac_stmix, FAC_ST0=spec.fac_st[0], FAC_ST1=spec.fac_st[1],
                     FAC_ST2=spec.fac_st[2], FAC_ST3=spec.fac_st[3], FAC_SFVIS=spec.fac_sfvis,
                     FAC_VORT=spec.fac_vort, FAC_PGRAD=spec.fac_pgrad)
        new_loss["FSTURB"] = np.array([r.fsturb for r in spec.rows], f32)
        new_loss["TURBVIS_DAMP"] = np.array([r.turbvis_damp for r in spec.rows], f32)
    xl = np.array([r.xllim for r in spec.rows], np.float32)
    arr = dict(
        JSTART=JSTART, JMIX=JMIX, JLE=JLE, JTE=JTE, JLED=JLED, KTIPS=KTIPS, KTIPE=KTIPE, KS1=KS1, KS2=KS2,
        JTRAN_I1=np.array([r.jtran[0] for r in spec.rows], np.int32),
        JTRAN_IM=np.array([r.jtran[1] for r in spec.rows], np.int32),
        JTRAN_K1=np.array([r.jtran[2] for r in spec.rows], np.int32),
        JTRAN_KM=np.array([r.jtran[3] for r in spec.rows], np.int32),
        IF_CUSP=np.array([r.if_cusp for r in spec.rows], np.int32),
        NUP_I1=np.array([r.nup_i1 for r in spec.rows], np.int32),
        NUP_IM=np.array([r.nup_im for r in spec.rows], np.int32),
        N_WAKE=np.array([r.n_wake for r in spec.rows], np.int32),
        NSTAGE=np.array([r.stage for r in spec.rows], np.int32),
        SEP_THIK=np.array([r.sep_thik for r in spec.rows], f32),
        SEP_DRAG=np.array([r.sep_drag for r in spec.rows], f32),
        RT_THICK=RT_THICK, RTHETA=RTHETA,
        XLLIM_I1=xl[:, 0], XLLIM_IM=xl[:, 1], XLLIM_K1=xl[:, 2], XLLIM_KM=xl[:, 3], XLLIM_DWN=xl[:, 4],
        XLLIM_UP=xl[:, 5], ROUGH_H=np.array([r.rough[0] for r in spec.rows], f32),
        ROUGH_T=np.array([r.rough[1] for r in spec.rows], f32), ROUGH_L=np.array([r.rough[2] for r in spec.rows], f32),
        ROUGH_U=np.array([r.rough[3] for r in spec.rows], f32), CHORD=CHORD,
        NBLADE=NBLADE[1:], IND=IND[1:], INDLE=INDLE[1:], INDMIX=INDMIX[1:JM + 1], NROW=NROW[1:],
        JB1=JB1[1:], JB2=JB2[1:], JSBLK=JSBLK[1:], WRAD=WRAD[1:], WHUB=WHUB[1:], WTIP=WTIP[1:],
        FACUP=FACUP, FACDWN=FACDWN, FP=FP, FU=FU, FD=FD, IB1=IB1, IB2=IB2, FR=FR, FKU=FKU, FKD=FKD,
        KB1=KB1, KB2=KB2, PO1=PO1, TO1=TO1, RPO1=RPO1, BSSIN=BSSIN, BSCOS=BSCOS, BRSIN=BRSIN,
        BRCOS=BRCOS, VTIN=VTIN, VM1=VM1, PD=PD, FBL=FBL, FBR=FBR, FTL=FTL, FTR=FTR,
        X=X, R=R, ABT=ABT, WRABT=WRABT, UBLADE=UBLADE, RAVG_CELL=RAVG_CELL, DX=DX, DR=DR, DS=DS,
        SMERID=SMERID, YPLUS_I1=np.full((KM, JM), 25.0, f32), YPLUS_IM=np.full((KM, JM), 25.0, f32),
        YPLUS_K1=np.full((JM, IM), 25.0, f32), YPLUS_KM=np.full((JM, IM), 25.0, f32),
        AQX=AQX, AQR=AQR, ABX=ABX, ABR=ABR, ASX=ASX, ASR=ASR, VOL=VOL, VOLOR=VOLOR, BSTEP=BSTEP,
        DWALLSQ=DWALLSQ, STEP1=STEP1, STEP2=STEP2, STEPSBK=STEPSBK,
        RO=RO, ROVX=ROVX, ROVR=ROVR, RORVT=RORVT, ROE=ROE, ROVT=ROVT, ROWT=ROWT, VX=VX, VR=VR, VT=VT,
        WT=WT, P=P, HO=HO, T_STATIC=T_STATIC, PEFF=PEFF, DRO=zeros3.copy(), DROE=zeros3.copy(),
        DROVX=zeros3.copy(), DROVR=zeros3.copy(), DRORVT=zeros3.copy(), XFORCE=zeros3.copy(),
        RFORCE=zeros3.copy(), TFORCE=zeros3.copy(), QSOURCE=zeros3.copy(), STEP=STEP, RSTEP=RSTEP,
        Y_PLUS=np.full((KM, JM, IM), 25.0, f32), DPDS_CELL=zeros3.copy(),
    )
    arr.update(new_loss)
    cd.ints = ints
    cd.reals = reals
    for k, v in arr.items():
        a = np.ascontiguousarray(v)
        cd.arrays[k] = a.astype(np.int32 if a.dtype.kind in "iu" else np.float32, copy=False)
    cd.extra = dict(JSTART1=JSTART1, JEND1=JEND1, JSTART2=JSTART2, JEND2=JEND2, THETA=THETA,
                    PREFF=float(PREFF), KMID=KMID, IMID=IMID)
    return cd


def wall_distance_sq(IM, JM, KM, X, R, THETA, ASX, ASR, ABX, ABR, ABT, JSTART, JMIX, JLE, JTE, NROW,
                     NBLADE, IMID, spec, ibound=0, with_dist=False):
    """DWALLSQ(I,J,K): the squared cell-average distance to the nearest
    solid wall, as SET_XLENGTH computes it (multall-open-18.3.f:12194-12517)."""
    JRANGE, KRANGE = 20, 5
    KMM1, IMM1 = KM - 1, IM - 1
    DIST = np.zeros((KM, JM, IM), f32)
    for J in range(1, JM + 1):
        nr = NROW[J]
        PITCH = f32(6.283185) * R[:, J - 1] / f32(NBLADE[J])           # (KM,)
        DIST_REF = f32(0.5) * PITCH
        j1 = max(J - JRANGE, 2)
        j2 = min(J + JRANGE, JM)
        js = np.arange(j1, j2 + 1)
        # hub / casing: independent of I
        dh = (X[:, J - 1][:, None] - X[0, js - 1][None, :]) ** 2 + (R[:, J - 1][:, None] - R[0, js - 1][None, :]) ** 2
        jmin_h = js[np.argmin(dh, axis=1)]
        dc = (X[:, J - 1][:, None] - X[KM - 1, js - 1][None, :]) ** 2 + (R[:, J - 1][:, None] - R[KM - 1, js - 1][None, :]) ** 2
        jmin_c = js[np.argmin(dc, axis=1)]

        def perp(jmin, kw):
            ax = ASX[kw, jmin - 1, IMID - 1]
            ar = ASR[kw, jmin - 1, IMID - 1]
            at = np.sqrt(ax * ax + ar * ar)
            return np.abs((X[:, J - 1] - X[kw, jmin - 1]) * (ax / at) + (R[:, J - 1] - R[kw, jmin - 1]) * (ar / at))

        hub = perp(jmin_h, 0)
        tip = perp(jmin_c, KM - 1)
        if ibound == 1 or ibound > 2:
            hub = DIST_REF
        if ibound >= 2:
            tip = DIST_REF
        endwall = (hub * tip / (hub + tip)).astype(f32)                   # (KM,)
        # blades
        b1 = max(J - JRANGE, 2)
        b1 = max(b1, JSTART[nr - 1])
        if b1 >= JTE[nr - 1]:
            b1 = JTE[nr - 1] - 1
        b2 = min(J + JRANGE, JM)
        b2 = min(b2, JMIX[nr - 1])
        if b2 <= JLE[nr - 1]:
            b2 = JLE[nr - 1] + 1
        jsb = np.arange(b1, b2 + 1)
        for K in range(1, KM + 1):
            k1 = max(K - KRANGE, 1)
            k2 = min(K + KRANGE, KM)
            ks = np.arange(k1, k2 + 1)
            xs = X[ks[None, :] - 1, jsb[:, None] - 1]                     # (nj, nk)
            rs = R[ks[None, :] - 1, jsb[:, None] - 1]
            xd = X[K - 1, J - 1] - xs
            rd = R[K - 1, J - 1] - rs
            th = THETA[K - 1, J - 1, :]                                   # (IM,)

            def side(isurf):
                ths = THETA[ks[None, :] - 1, jsb[:, None] - 1, isurf]   # (nj,nk)
                tsq = f32(4.0) * R[K - 1, J - 1] * rs * np.sin((th[:, None, None] - ths[None]) / f32(2.0)) ** 2
                dsq = (xd * xd + rd * rd)[None] + tsq                     # (IM,nj,nk)
                flat = dsq.reshape(IM, -1)
                idx = np.argmin(flat, axis=1)
                jmin = jsb[idx // ks.size]
                kmin = ks[idx % ks.size]
                knorm = np.where(kmin == KM, KM - 1, kmin)
                bx = ABX[knorm - 1, jmin - 1, isurf]
                br = ABR[knorm - 1, jmin - 1, isurf]
                bt = ABT[knorm - 1, jmin - 1]
                at = np.sqrt(bx * bx + br * br + bt * bt)
                xdif = X[K - 1, J - 1] - X[kmin - 1, jmin - 1]
                rdif = R[K - 1, J - 1] - R[kmin - 1, jmin - 1]
                tdif = f32(2.0) * np.sqrt(R[K - 1, J - 1] * R[kmin - 1, jmin - 1]) * np.sin(
                    (th - THETA[kmin - 1, jmin - 1, isurf]) / f32(2.0))
                d = np.abs(xdif * (bx / at) + rdif * (br / at) + tdif * (bt / at))
                le_te = (jmin <= JLE[nr - 1]) | (jmin >= JTE[nr - 1])
                d = np.where(le_te, np.sqrt(xdif * xdif + rdif * rdif + tdif * tdif), d)
                return d.astype(f32)

            ss = side(0)
            ps = side(IM - 1)
            blade = ss * ps / (ss + ps)
            if 1 < K < KM:
                ds_ = np.sqrt(endwall[K - 1] ** 2 + blade ** 2)
                ds_ = np.maximum(ds_, f32(1.0e-10))
                DIST[K - 1, J - 1, :] = blade * endwall[K - 1] / ds_
            else:
                DIST[K - 1, J - 1, :] = 0.0
    DW = np.zeros((KM, JM, IM), f32)
    avg = f32(0.125) * (DIST[:-1, 1:, :-1] + DIST[1:, 1:, :-1] + DIST[:-1, :-1, :-1] + DIST[1:, :-1, :-1]
                        + DIST[:-1, 1:, 1:] + DIST[1:, 1:, 1:] + DIST[:-1, :-1, 1:] + DIST[1:, :-1, 1:])
    DW[:KMM1, 1:, :IMM1] = avg * avg
    return (DW, DIST) if with_dist else DW


def mixing_lengths(spec, IM, JM, KM, DIST, SMERID, JSTART, JMIX, JLE, JTE, NROW, IMID, KMID):
    """XLENGTH and FST_RAT of NEW_LOSS from the node wall distances DIST_MIN
    (SET_XLENGTH, multall-open-18.3.f:12423-12492): the mixing-length limit
    XLIMIT(J) interpolated along the meridional distance from XLLIM_IN, _LE,
    _TE and _DN of the row, the blend of the linear and constant regions, and
    the cell averages, 0.41**2 times the squared mean length."""
    KMM1, IMM1 = KM - 1, IM - 1
    XLIMIT = np.zeros(JM + 1, f32)
    for J in range(1, JM + 1):
        nr = NROW[J]
        xin, xle, xte, xdn = (f32(v) for v in spec.rows[nr - 1].xllim_new)
        sm = lambda jj: SMERID[KMID - 1, jj - 1]
        js, jl, jt, jx = JSTART[nr - 1], JLE[nr - 1], JTE[nr - 1], JMIX[nr - 1]
        if J <= jl:
            XLLIM = xin + (sm(J) - sm(js)) / (sm(jl) - sm(js)) * (xle - xin)
        if jl < J <= jt:
            XLLIM = xle + (sm(J) - sm(jl)) / (sm(jt) - sm(jl)) * (xte - xle)
        if J > jt:
            XLLIM = xte + (sm(J) - sm(jt)) / (sm(jx) - sm(jt)) * (xdn - xte)
        XLIMIT[J] = f32(2.0) * DIST[KMID - 1, J - 1, IMID - 1] * f32(XLLIM)
    DBLEND = f32(0.6666666)
    EXPON = DBLEND / (f32(1.0) - DBLEND)
    FBLEND = (f32(1.0) - DBLEND) * DBLEND ** EXPON
    XL = XLIMIT[1:][None, :, None]
    RATIO = DIST / XL
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        STORE = np.where(RATIO > DBLEND, XL * (f32(1.0) - FBLEND * RATIO ** (-EXPON)), DIST).astype(f32)
    TEMP3 = ((STORE / XL) ** 4).astype(f32)

    def avg8(A):
        return f32(0.125) * (A[:-1, 1:, :-1] + A[1:, 1:, :-1] + A[:-1, :-1, :-1] + A[1:, :-1, :-1]
                             + A[:-1, 1:, 1:] + A[1:, 1:, 1:] + A[:-1, :-1, 1:] + A[1:, :-1, 1:])
    XLENGTH = np.zeros((KM, JM, IM), f32)
    FST_RAT = np.zeros((KM, JM, IM), f32)
    ax = avg8(STORE)
    XLENGTH[:KMM1, 1:, :IMM1] = f32(0.41) * f32(0.41) * ax * ax
    fs = np.array([f32(spec.rows[NROW[J] - 1].fsturb) for J in range(2, JM + 1)], f32)
    FST_RAT[:KMM1, 1:, :IMM1] = avg8(TEMP3) * fs[None, :, None]
    first = np.array([J == JSTART[NROW[J] - 1] for J in range(2, JM + 1)])
    XLENGTH[:KMM1, 1:, :IMM1][:, first, :] = 0.0
    FST_RAT[:KMM1, 1:, :IMM1][:, first, :] = 0.0
    return dict(XLENGTH=XLENGTH, FST_RAT=FST_RAT)
