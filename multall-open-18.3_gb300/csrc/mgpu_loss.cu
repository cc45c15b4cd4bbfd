// mgpu_loss.cu -- the viscous body forces of SUBROUTINE LOSS (ILOS=10,
// multall-open-18.3.f:8058-9066) with the Shih wall functions WALLFUN
// (15980-16047, YPLUSWALL in (-10,-0.001)); the every-5-step tail of LOOP
// (monitors 5264-5317 and STEPUP 7916-8002); and the EFICOOL/SUMFLX mass
// averages (10662-10849, 7873-7912).
//
// LOSS is two passes over the grid.  The streamwise-face pass takes one
// thread per (I,J) column of cells and walks K (the transition test needs
// the maximum of mu_t/mu over half the span before any stress is formed);
// the bladewise-face pass takes one thread per (J,K) line and walks I.
#include "mgpu_internal.cuh"

namespace mgpu {

static inline unsigned grid_for(size_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

constexpr int LMAX = 164;   // IM, KM <= 160 plus the 1-based end slots

// viscosity set on entry to LOSS (8088-8112); one thread
__global__ void k_loss_prologue(Dev d, int init_call) {
    DevCtl *c = d.ctl;
    if (!init_call && !c->do_loss) return;
    int nstep = init_call ? 1 : c->nstep;
    float VISLAM = c->VISLAM;
    if (nstep == 1 || nstep < d.NSTEPS_MAX / 4) {
        if (d.REYNO > 100.0f) {
            int J1 = A1(d.JLE, 1), J2 = A1(d.JTE, 1);
            if (A1(d.JLE, 1) > d.JM) J1 = 1;
            if (A1(d.JTE, 1) > d.JM) J2 = d.JM;
            float XCHORD = A2(d.SMERID, J2, d.KMID) - A2(d.SMERID, J1, d.KMID);
            float a = A3(d.ROVX, d.IMID, J2, d.KMID), b = A3(d.ROVR, d.IMID, J2, d.KMID), cc = A3(d.ROWT, d.IMID, J2, d.KMID);
            float ROW2 = sqrtf(a * a + b * b + cc * cc);
            VISLAM = XCHORD * ROW2 / d.REYNO;
        }
        if (d.REYNO > 0.0f && d.REYNO < 99.99f) VISLAM = d.REYNO / 100000.0f;
        if (d.REYNO < 0.0f) VISLAM = -d.REYNO * 1.0E-5f;
        float TCOND = d.CP * VISLAM / d.PRANDTL;
        c->FTCOND = TCOND / VISLAM;
        c->VISLAM = VISLAM;
    }
}

// Shih et al. wall function without the pressure-gradient term
__device__ inline void wallfun(float PERP, float DENSITY, float &TWALL, float YPLUS_OLD, float WREL_WALL,
                               float &YPLUS_NEW, float VISLAM) {
    float YP1 = YPLUS_OLD, YP2 = YP1 * YP1, YP3 = YP2 * YP1, YP4 = YP2 * YP2;
    float FYPLUS = 0.0f;
    if (YP1 <= 5.0f) FYPLUS = YP1 + 1.0E-2f * YP2 - 2.9E-03f * YP3;
    if (YP1 > 5.0f && YP1 <= 30.0f) FYPLUS = -0.872f + 1.465f * YP1 - 7.02E-2f * YP2 + 1.66E-03f * YP3 - 1.495E-5f * YP4;
    if (YP1 > 30.0f && YP1 <= 140.0f) FYPLUS = 8.6f + 0.1864f * YP1 - 2.006E-3f * YP2 + 1.144E-5f * YP3 - 2.551E-8f * YP4;
    if (YP1 > 140.0f) FYPLUS = 2.439f * logf(YP1) + 5.0f;
    float FRACP = 0.0f;
    float VPLUS = FYPLUS * (1.0f + FRACP);
    float VSTAR = WREL_WALL / VPLUS;
    TWALL = DENSITY * VSTAR * VSTAR;
    YPLUS_NEW = DENSITY * VSTAR * PERP / VISLAM;
}

// log-law skin friction with roughness (8285-8331 and its three copies)
__device__ inline float skin_friction(float RE, float PERP, float ROUGH, float dens, float wb, float VISLAM) {
    float RELOG = 1.0f / logf(RE);
    float CF;
    if (ROUGH > 1.0E-7f) {
        if (ROUGH > PERP) ROUGH = PERP;
        float REK = RE * ROUGH / PERP;
        REK = REK - 80.0f;
        if (REK < 0.0f) REK = 0.0f;
        float REKSQ = REK * REK;
        float A1c = -.00178493f + .0000814923f * REK + .000000150445f * REKSQ;
        float A2c = .029072f - .001584f * REK - .00000225194f * REKSQ;
        float A3c = .270313f + .0091409f * REK + .00000451537f * REKSQ + .00000000464767f * REKSQ * REK;
        CF = A1c + A2c * RELOG + A3c * RELOG * RELOG;
    } else {
        CF = -0.00178493f + 0.029072f * RELOG + 0.270313f * RELOG * RELOG;
    }
    float CFLAM = 2.0f / RE;
    CF = fmaxf(CF, CFLAM);
    if (RE < 125.0f) CF = CFLAM;
    if (ROUGH > 1.0E-7f) {
        float TW = 0.5f * CF * dens * wb * wb;
        float VSTAR = sqrtf(TW / dens);
        float PLUSK = ROUGH * VSTAR * dens / VISLAM;
        float RELOG10 = log10f(PERP / ROUGH);
        float FUNCN = 5.75f * RELOG10 + 8.5f;
        float CF_FULL_ROUGH = 2.0f / (FUNCN * FUNCN);
        if (PLUSK > 45.0f && CF > CF_FULL_ROUGH) CF = CF_FULL_ROUGH;
    }
    return 0.5f * CF * dens * wb * wb;
}

__device__ inline float fyplus_of(float yp, float yplam, float ypturb, float prev) {
    float f = prev;
    if (yp <= yplam) f = 0.0f;
    if (yp > yplam) {
        float XFAC = (yp - yplam) / (ypturb - yplam);
        if (XFAC > 1.0f) XFAC = 1.0f;
        f = XFAC * XFAC * (3.0f - 2.0f * XFAC);
    }
    return f;
}

// ---------------------------------------------------------------------
// stresses on the streamwise (K = const) faces, LOSS DO 50
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_loss_kfaces(Dev d, int init_call) {
    const DevCtl *c = d.ctl;
    if (!init_call && !c->do_loss) return;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.IMM1 * (d.JM - 1)) return;
    int i = t % d.IMM1 + 1, j = t / d.IMM1 + 2;
    const float RF_VIS = init_call ? 1.0f : d.RF_VIS;
    const float FMIXUP = init_call ? 1.0f : c->FMIXUP;
    float VISLAM = c->VISLAM, FTCOND = c->FTCOND;
    const int KM = d.KM, KMM1 = d.KMM1, KMID = d.KMID;
    float VXAVG[LMAX], VRAVG[LMAX], VTAVG[LMAX], ROAVG[LMAX], TAVG[LMAX], RAVG[LMAX], WABS[LMAX], WTB[LMAX],
        WBOUND[LMAX], AREA[LMAX], VLAM[LMAX], VTURB[LMAX];
    int NRW = A1(d.NROW, j);
    int JROW = j - A1(d.JSTART, NRW) + 1;
    int JTRHUB = A1(d.JTRAN_K1, NRW), JTRTIP = A1(d.JTRAN_KM, NRW);
    float WREL = A1(d.WRAD, j), WHUB = A1(d.WHUB, j), WTIP = A1(d.WTIP, j);
    for (int k = 1; k <= KM; ++k) {
        float asx = A3(d.ASX, i, j, k), asr = A3(d.ASR, i, j, k);
        AREA[k] = sqrtf(asx * asx + asr * asr);
        VXAVG[k] = 0.25f * (A3(d.VX, i, j, k) + A3(d.VX, i, j - 1, k) + A3(d.VX, i + 1, j, k) + A3(d.VX, i + 1, j - 1, k));
        VRAVG[k] = 0.25f * (A3(d.VR, i, j, k) + A3(d.VR, i, j - 1, k) + A3(d.VR, i + 1, j, k) + A3(d.VR, i + 1, j - 1, k));
        VTAVG[k] = 0.25f * (A3(d.VT, i, j, k) + A3(d.VT, i, j - 1, k) + A3(d.VT, i + 1, j, k) + A3(d.VT, i + 1, j - 1, k));
        ROAVG[k] = 0.25f * (A3(d.RO, i, j, k) + A3(d.RO, i, j - 1, k) + A3(d.RO, i + 1, j, k) + A3(d.RO, i + 1, j - 1, k));
        TAVG[k] = 0.25f * (A3(d.T_STATIC, i, j, k) + A3(d.T_STATIC, i, j - 1, k) + A3(d.T_STATIC, i + 1, j, k) +
                           A3(d.T_STATIC, i + 1, j - 1, k));
        RAVG[k] = 0.5f * (A2(d.R, j, k) + A2(d.R, j - 1, k));
        float WTAVG = VTAVG[k] - WREL * RAVG[k];
        float WABSQ = VXAVG[k] * VXAVG[k] + VRAVG[k] * VRAVG[k] + WTAVG * WTAVG;
        WABS[k] = sqrtf(WABSQ);
        WTB[k] = VTAVG[k] - WHUB * RAVG[k];
        if (k > KMID) WTB[k] = VTAVG[k] - WTIP * RAVG[k];
        WBOUND[k] = sqrtf(VXAVG[k] * VXAVG[k] + VRAVG[k] * VRAVG[k] + WTB[k] * WTB[k]);
    }
    if (d.REYNO < 0.0001f) {
        VISLAM = (fabsf(d.REYNO) / 100000.0f) * powf(TAVG[KMID] / 288.0f, 0.62f);
        float TCOND = d.CP * VISLAM / d.PRANDTL;
        FTCOND = TCOND / VISLAM;
    }
    float TWALLK1, TWALLKM;
    if (d.YPLUSWALL < -0.001f) {
        float PERPK1 = A3(d.VOL, i, j, 1) / AREA[1];
        float ynew;
        wallfun(PERPK1, ROAVG[1], TWALLK1, AIJ(d.YPLUS_K1, i, j), WBOUND[1], ynew, VISLAM);
        AIJ(d.YPLUS_K1, i, j) = fminf(1000.0f, ynew);
    } else if (d.YPLUSWALL < 5.0f) {
        float PERP = A3(d.VOL, i, j, 1) / AREA[1];
        float RE = PERP * ROAVG[2] * WBOUND[2] / VISLAM;
        TWALLK1 = skin_friction(RE, PERP, A1(d.ROUGH_H, NRW), ROAVG[2], WBOUND[2], VISLAM);
    } else {
        TWALLK1 = d.CFWALL * ROAVG[1] * WBOUND[1] * WBOUND[1];
    }
    if (d.YPLUSWALL < -0.001f) {
        float PERPKM = A3(d.VOL, i, j, KMM1) / AREA[KM];
        float ynew;
        wallfun(PERPKM, ROAVG[KMM1], TWALLKM, AIJ(d.YPLUS_KM, i, j), WBOUND[KMM1], ynew, VISLAM);
        AIJ(d.YPLUS_KM, i, j) = fminf(1000.0f, ynew);
    } else if (d.YPLUSWALL < 5.0f) {
        float PERP = A3(d.VOL, i, j, KMM1) / AREA[KM];
        float RE = PERP * ROAVG[KMM1] * WBOUND[KMM1] / VISLAM;
        TWALLKM = skin_friction(RE, PERP, A1(d.ROUGH_T, NRW), ROAVG[KMM1], WBOUND[KMM1], VISLAM);
    } else {
        TWALLKM = d.CFWALL * ROAVG[KM] * WBOUND[KM] * WBOUND[KM];
    }
    float VSTAR = sqrtf(TWALLK1 / ROAVG[1]);
    for (int k = 1; k <= KMID; ++k) {
        float PERP = sqrtf(A3(d.DWALLSQ, i, j, k));
        float YPLSK1 = VSTAR * PERP * ROAVG[1] / VISLAM;
        A3(d.Y_PLUS, i, j, k) = fminf(YPLSK1, 1000.0f);
    }
    VSTAR = sqrtf(TWALLKM / ROAVG[KM]);
    for (int k = KMID + 1; k <= KMM1; ++k) {
        float PERP = sqrtf(A3(d.DWALLSQ, i, j, k));
        float YPLS = VSTAR * PERP * ROAVG[KM] / VISLAM;
        A3(d.Y_PLUS, i, j, k) = fminf(YPLS, 1000.0f);
    }
    float FYPLUS = 0.0f;
    for (int k = 2; k <= KMM1; ++k) {
        FYPLUS = fyplus_of(A3(d.Y_PLUS, i, j, k), d.YPLAM, d.YPTURB, FYPLUS);
        float DPERP = A3(d.VOL, i, j, k) / AREA[k];
        VLAM[k] = d.FKLAM[(size_t)(NRW - 1) * KM + k - 1] * VISLAM / DPERP;
        VTURB[k] = d.FKTURB[(size_t)(NRW - 1) * KM + k - 1] * ROAVG[k] * fabsf(WABS[k + 1] - WABS[k - 1]) * FMIXUP;
        VTURB[k] = VTURB[k] * FYPLUS;
    }
    bool turb = false;
    if (!(JROW < JTRHUB)) {
        float RMAX = 0.0f;
        for (int k = 2; k <= KMID; ++k) {
            float RATVIS = VTURB[k] / VLAM[k];
            if (RATVIS < RMAX) continue;
            RMAX = RATVIS;
        }
        turb = RMAX > d.FTRANS;
    }
    if (!turb)
        for (int k = 2; k <= KMID; ++k) VTURB[k] = 0.0f;
    turb = false;
    if (!(JROW < JTRTIP)) {
        float RMAX = 0.0f;
        for (int k = KMID; k <= KMM1; ++k) {
            float RATVIS = VTURB[k] / VLAM[k];
            if (RATVIS < RMAX) continue;
            RMAX = RATVIS;
        }
        turb = RMAX > d.FTRANS;
    }
    if (!turb)
        for (int k = KMID; k <= KMM1; ++k) VTURB[k] = 0.0f;
    // stresses at the faces K, streamed from K=1 upwards
    float FMULT = TWALLK1 * AREA[1] / WBOUND[1];
    if (d.IBOUND == 1 || d.IBOUND > 2) FMULT = 0.0f;
    float xs_lo = FMULT * VXAVG[1], rs_lo = FMULT * VRAVG[1], ts_lo = FMULT * WTB[1];
    float qf_lo = 0.0f, wv_lo = ts_lo * WHUB * RAVG[1];
    float FMULTM = -TWALLKM * AREA[KM] / WBOUND[KM];
    if (d.IBOUND >= 2) FMULTM = 0.0f;
    float RF_VIS1 = 1.0f - RF_VIS;
    for (int k = 1; k <= KMM1; ++k) {
        int kp = k + 1;
        float xs_hi, rs_hi, ts_hi, qf_hi, wv_hi;
        if (kp == KM) {
            xs_hi = FMULTM * VXAVG[KM];
            rs_hi = FMULTM * VRAVG[KM];
            ts_hi = FMULTM * WTB[KM];
            qf_hi = 0.0f;
            wv_hi = ts_hi * WTIP * RAVG[KM];
        } else {
            float FM = AREA[kp] * (VLAM[kp] + VTURB[kp]);
            xs_hi = FM * (VXAVG[kp + 1] - VXAVG[kp - 1]);
            rs_hi = FM * (VRAVG[kp + 1] - VRAVG[kp - 1]);
            float VISTOT = VISLAM * (1.0f + VTURB[kp] / VLAM[kp]);
            ts_hi = FM * (VTAVG[kp + 1] - VTAVG[kp - 1]) - VISTOT * AREA[kp] * VTAVG[kp] / RAVG[kp];
            qf_hi = FM * FTCOND * (TAVG[kp + 1] - TAVG[kp - 1]);
            wv_hi = xs_hi * VXAVG[kp] + ts_hi * VTAVG[kp] + rs_hi * VRAVG[kp];
        }
        size_t n = ix3(d, i, j, k);
        d.XFORCE[n] = RF_VIS1 * d.XFORCE[n] + RF_VIS * (xs_lo - xs_hi);
        d.RFORCE[n] = RF_VIS1 * d.RFORCE[n] + RF_VIS * (rs_lo - rs_hi);
        d.TFORCE[n] = RF_VIS1 * d.TFORCE[n] + RF_VIS * (ts_lo * RAVG[k] - ts_hi * RAVG[kp]);
        d.QSOURCE[n] = RF_VIS1 * d.QSOURCE[n] + RF_VIS * (qf_lo - qf_hi + wv_lo - wv_hi);
        xs_lo = xs_hi; rs_lo = rs_hi; ts_lo = ts_hi; qf_lo = qf_hi; wv_lo = wv_hi;
    }
}

// ---------------------------------------------------------------------
// stresses on the bladewise (I = const) faces and the blade surfaces,
// LOSS DO 100
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_loss_ifaces(Dev d, int init_call) {
    const DevCtl *c = d.ctl;
    if (!init_call && !c->do_loss) return;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (d.JM - 1) * d.KMM1) return;
    int k = t % d.KMM1 + 1, j = t / d.KMM1 + 2;
    const float RF_VIS = init_call ? 1.0f : d.RF_VIS;
    const float FMIXUP = init_call ? 1.0f : c->FMIXUP;
    float VISLAM = c->VISLAM, FTCOND = c->FTCOND;
    const int IM = d.IM, IMM1 = d.IMM1, IMID = d.IMID;
    float VXAVG[LMAX], VRAVG[LMAX], VTAVG[LMAX], WTAVG[LMAX], ROAVG[LMAX], TAVG[LMAX], WABS[LMAX], AREA[LMAX];
    float XSTRES[LMAX], RSTRES[LMAX], TSTRES[LMAX], QFLOW[LMAX], WVISC[LMAX], VLAM[LMAX], VTURB[LMAX];
    int NRW = A1(d.NROW, j);
    int JROW = j - A1(d.JSTART, NRW) + 1;
    int JTRLOW = A1(d.JTRAN_I1, NRW), JTRUP = A1(d.JTRAN_IM, NRW);
    int JLEDGE = A1(d.JLE, NRW), JTEDGE = A1(d.JTE, NRW);
    float WREL = A1(d.WRAD, j);
    float RAVGK = A2(d.RAVG_CELL, j, k);
    float abt = A2(d.ABT, j, k);
    for (int i = 1; i <= IM; ++i) {
        float abx = A3(d.ABX, i, j, k), abr = A3(d.ABR, i, j, k);
        AREA[i] = sqrtf(abx * abx + abr * abr + abt * abt);
        VXAVG[i] = 0.25f * (A3(d.VX, i, j, k) + A3(d.VX, i, j - 1, k) + A3(d.VX, i, j - 1, k + 1) + A3(d.VX, i, j, k + 1));
        VRAVG[i] = 0.25f * (A3(d.VR, i, j, k) + A3(d.VR, i, j - 1, k) + A3(d.VR, i, j - 1, k + 1) + A3(d.VR, i, j, k + 1));
        VTAVG[i] = 0.25f * (A3(d.VT, i, j, k) + A3(d.VT, i, j - 1, k) + A3(d.VT, i, j - 1, k + 1) + A3(d.VT, i, j, k + 1));
        WTAVG[i] = 0.25f * (A3(d.WT, i, j, k) + A3(d.WT, i, j - 1, k) + A3(d.WT, i, j - 1, k + 1) + A3(d.WT, i, j, k + 1));
        ROAVG[i] = 0.25f * (A3(d.RO, i, j, k) + A3(d.RO, i, j - 1, k) + A3(d.RO, i, j - 1, k + 1) + A3(d.RO, i, j, k + 1));
        TAVG[i] = 0.25f * (A3(d.T_STATIC, i, j, k) + A3(d.T_STATIC, i, j - 1, k) + A3(d.T_STATIC, i, j - 1, k + 1) +
                           A3(d.T_STATIC, i, j, k + 1));
        float WABSQ = VXAVG[i] * VXAVG[i] + VRAVG[i] * VRAVG[i] + WTAVG[i] * WTAVG[i];
        WABS[i] = sqrtf(WABSQ);
    }
    if (d.REYNO < 0.0001f) {
        VISLAM = (fabsf(d.REYNO) / 100000.0f) * powf(TAVG[IMID] / 288.0f, 0.62f);
        float TCOND = d.CP * VISLAM / d.PRANDTL;
        FTCOND = TCOND / VISLAM;
    }
    const float *FIL = d.FILAM + (size_t)(NRW - 1) * IM;
    const float *FIT = d.FITURB + (size_t)(NRW - 1) * IM;
    const float *FIW = d.FIWAKE + (size_t)(NRW - 1) * IM;
    const float *FIU = d.FIUP + (size_t)(NRW - 1) * IM;
    bool in_blade = !(j <= JLEDGE || j > JTEDGE);
    bool in_gap = (A1(d.KTIPS, NRW) > 0) && (k >= A1(d.KTIPS, NRW)) && (k < A1(d.KTIPE, NRW));
    if (in_blade) {
        if (!in_gap) {
            float TWALLI1, TWALLIM;
            if (d.YPLUSWALL < -0.001f) {
                float PERPI1 = A3(d.VOL, 1, j, k) / AREA[1];
                float ynew;
                wallfun(PERPI1, ROAVG[1], TWALLI1, A2(d.YPLUS_I1, j, k), WABS[2], ynew, VISLAM);
                A2(d.YPLUS_I1, j, k) = fminf(1000.0f, ynew);
            } else if (d.YPLUSWALL < 5.0f) {
                float PERP = A3(d.VOL, 1, j, k) / AREA[1];
                float RE = ROAVG[2] * WABS[2] * PERP / VISLAM;
                TWALLI1 = skin_friction(RE, PERP, A1(d.ROUGH_L, NRW), ROAVG[2], WABS[2], VISLAM);
            } else {
                TWALLI1 = d.CFWALL * ROAVG[1] * WABS[1] * WABS[1];
            }
            if (d.YPLUSWALL < -0.001f) {
                float PERPIM = A3(d.VOL, IMM1, j, k) / AREA[IM];
                float ynew;
                wallfun(PERPIM, ROAVG[IMM1], TWALLIM, A2(d.YPLUS_IM, j, k), WABS[IMM1], ynew, VISLAM);
                A2(d.YPLUS_IM, j, k) = fminf(1000.0f, ynew);
            } else if (d.YPLUSWALL < 5.0f) {
                float PERP = A3(d.VOL, IMM1, j, k) / AREA[IM];
                float RE = ROAVG[IMM1] * WABS[IMM1] * PERP / VISLAM;
                TWALLIM = skin_friction(RE, PERP, A1(d.ROUGH_U, NRW), ROAVG[IMM1], WABS[IMM1], VISLAM);
            } else {
                TWALLIM = d.CFWALL * ROAVG[IM] * WABS[IM] * WABS[IM];
            }
            float VSTAR = sqrtf(TWALLI1 / ROAVG[1]);
            for (int i = 1; i <= IMID; ++i) {
                float YPLS = VSTAR * sqrtf(A3(d.DWALLSQ, i, j, k)) * ROAVG[1] / VISLAM;
                float YPLSP = A3(d.Y_PLUS, i, j, k);
                A3(d.Y_PLUS, i, j, k) = fminf(YPLS, YPLSP);
            }
            VSTAR = sqrtf(TWALLIM / ROAVG[IM]);
            for (int i = IMID + 1; i <= IMM1; ++i) {
                float YPLS = VSTAR * sqrtf(A3(d.DWALLSQ, i, j, k)) * ROAVG[IM] / VISLAM;
                float YPLSP = A3(d.Y_PLUS, i, j, k);
                A3(d.Y_PLUS, i, j, k) = fminf(YPLS, YPLSP);
            }
            float FMULT = TWALLI1 * AREA[1] / WABS[1];
            XSTRES[1] = FMULT * VXAVG[1];
            RSTRES[1] = FMULT * VRAVG[1];
            TSTRES[1] = FMULT * WTAVG[1];
            FMULT = -TWALLIM * AREA[IM] / WABS[IM];
            XSTRES[IM] = FMULT * VXAVG[IM];
            RSTRES[IM] = FMULT * VRAVG[IM];
            TSTRES[IM] = FMULT * WTAVG[IM];
            QFLOW[1] = 0.0f;
            WVISC[1] = TSTRES[1] * WREL * RAVGK;
            QFLOW[IM] = 0.0f;
            WVISC[IM] = TSTRES[IM] * WREL * RAVGK;
        }
        float FYPLUS = 0.0f;
        for (int i = 2; i <= IMM1; ++i) {
            FYPLUS = fyplus_of(A3(d.Y_PLUS, i, j, k), d.YPLAM, d.YPTURB, FYPLUS);
            float DPERP = A3(d.VOL, i, j, k) / AREA[i];
            VLAM[i] = FIL[i - 1] * VISLAM / DPERP;
            VTURB[i] = FIT[i - 1] * ROAVG[i] * fabsf(WABS[i + 1] - WABS[i - 1]) * FMIXUP;
            VTURB[i] = VTURB[i] * FYPLUS;
        }
        bool turb = false;
        if (!(JROW < JTRLOW)) {
            float RMAX = 0.0f;
            for (int i = 2; i <= IMID; ++i) {
                float RATVIS = VTURB[i] / VLAM[i];
                if (RATVIS < RMAX) continue;
                RMAX = RATVIS;
            }
            turb = RMAX > d.FTRANS;
        }
        if (!turb)
            for (int i = 2; i <= IMID; ++i) VTURB[i] = 0.0f;
        turb = false;
        if (!(JROW < JTRUP)) {
            float RMAX = 0.0f;
            for (int i = IMID; i <= IMM1; ++i) {
                float RATVIS = VTURB[i] / VLAM[i];
                if (RATVIS < RMAX) continue;
                RMAX = RATVIS;
            }
            turb = RMAX > d.FTRANS;
        }
        if (!turb)
            for (int i = IMID; i <= IMM1; ++i) VTURB[i] = 0.0f;
        for (int i = 2; i <= IMM1; ++i) {
            float FM = (VLAM[i] + VTURB[i]) * AREA[i];
            XSTRES[i] = FM * (VXAVG[i + 1] - VXAVG[i - 1]);
            RSTRES[i] = FM * (VRAVG[i + 1] - VRAVG[i - 1]);
            TSTRES[i] = FM * (WTAVG[i + 1] - WTAVG[i - 1]);
            A3(d.VISC_RAT, i, j, k) = VTURB[i] / VLAM[i];
            QFLOW[i] = FM * FTCOND * (TAVG[i + 1] - TAVG[i - 1]);
            WVISC[i] = XSTRES[i] * VXAVG[i] + RSTRES[i] * VRAVG[i] + TSTRES[i] * VTAVG[i];
        }
        if (in_gap) {
            XSTRES[1] = 0.5f * (XSTRES[2] + XSTRES[IMM1]);
            RSTRES[1] = 0.5f * (RSTRES[2] + RSTRES[IMM1]);
            TSTRES[1] = 0.5f * (TSTRES[2] + TSTRES[IMM1]);
            XSTRES[IM] = XSTRES[1];
            TSTRES[IM] = TSTRES[1];
            RSTRES[IM] = RSTRES[1];
            QFLOW[1] = 0.5f * (QFLOW[2] + QFLOW[IMM1]);
            WVISC[1] = 0.5f * (WVISC[2] + WVISC[IMM1]);
            QFLOW[IM] = QFLOW[1];
            WVISC[IM] = WVISC[1];
        }
    } else {
        float FACJ = 0.0f;
        bool wake = j > JTEDGE;
        if (wake) {
            FACJ = 0.1f * (float)(j - JTEDGE);
            if (FACJ > 1.0f) FACJ = 1.0f;
        }
        for (int i = 1; i <= IM; ++i) {
            int ISUB = (i == IM) ? IMM1 : i;
            int IM1 = (i == 1) ? IMM1 : i - 1;
            int IP1 = (i == IM) ? 2 : i + 1;
            float DPERP = A3(d.VOL, ISUB, j, k) / AREA[i];
            VLAM[i] = FIL[i - 1] * VISLAM / DPERP;
            if (wake) {
                float FBLEND = (FACJ * FIW[i - 1] + (1.0f - FACJ) * FIT[i - 1]) * FMIXUP;
                VTURB[i] = FBLEND * ROAVG[i] * fabsf(WABS[IP1] - WABS[IM1]);
            } else {
                VTURB[i] = FMIXUP * FIU[i - 1] * ROAVG[i] * fabsf(WABS[IP1] - WABS[IM1]);
            }
            A3(d.VISC_RAT, i, j, k) = VTURB[i] / VLAM[i];
            float FM = AREA[i] * (VLAM[i] + VTURB[i]);
            XSTRES[i] = FM * (VXAVG[IP1] - VXAVG[IM1]);
            RSTRES[i] = FM * (VRAVG[IP1] - VRAVG[IM1]);
            TSTRES[i] = FM * (WTAVG[IP1] - WTAVG[IM1]);
            QFLOW[i] = FM * FTCOND * (TAVG[IP1] - TAVG[IM1]);
            WVISC[i] = XSTRES[i] * VXAVG[i] + TSTRES[i] * VTAVG[i] + RSTRES[i] * VRAVG[i];
        }
        XSTRES[1] = 0.5f * (XSTRES[IM] + XSTRES[1]);
        RSTRES[1] = 0.5f * (RSTRES[IM] + RSTRES[1]);
        TSTRES[1] = 0.5f * (TSTRES[IM] + TSTRES[1]);
        XSTRES[IM] = XSTRES[1];
        RSTRES[IM] = RSTRES[1];
        TSTRES[IM] = TSTRES[1];
        QFLOW[1] = 0.5f * (QFLOW[IM] + QFLOW[1]);
        WVISC[1] = 0.5f * (WVISC[IM] + WVISC[1]);
        QFLOW[IM] = QFLOW[1];
        WVISC[IM] = WVISC[1];
    }
    for (int i = 1; i <= IMM1; ++i) {
        size_t n = ix3(d, i, j, k);
        d.XFORCE[n] = d.XFORCE[n] + RF_VIS * (XSTRES[i] - XSTRES[i + 1]);
        d.RFORCE[n] = d.RFORCE[n] + RF_VIS * (RSTRES[i] - RSTRES[i + 1]);
        d.TFORCE[n] = d.TFORCE[n] + RF_VIS * (TSTRES[i] - TSTRES[i + 1]) * RAVGK;
        d.QSOURCE[n] = d.QSOURCE[n] + RF_VIS * (QFLOW[i] - QFLOW[i + 1] + WVISC[i] - WVISC[i + 1]);
    }
}

void launch_loss(const Dev &d, Launch L, bool init_call) {
    k_loss_prologue<<<1, 1, 0, L.s>>>(d, init_call ? 1 : 0);
    mark(L, "k_loss_prologue");
    int nk = d.IMM1 * (d.JM - 1);
    k_loss_kfaces<<<grid_for(nk, 128), 128, 0, L.s>>>(d, init_call ? 1 : 0);
    mark(L, "k_loss_kfaces");
    int ni = (d.JM - 1) * d.KMM1;
    k_loss_ifaces<<<grid_for(ni, 128), 128, 0, L.s>>>(d, init_call ? 1 : 0);
    mark(L, "k_loss_ifaces");
}

// ---------------------------------------------------------------------
// every-5-step tail: mass flow per J (5665-5677), % change of Vm
// (8500-8520) with EMAX/EAVG, VREF/VMAX, and a health count
// ---------------------------------------------------------------------
constexpr int TAIL_BS = 256;

__global__ void __launch_bounds__(TAIL_BS) k_tail_flow(Dev d) {
    if (!d.ctl->do_tail) return;
    int j = blockIdx.x + 1;
    int ncell = d.IMM1 * d.KMM1;
    double s = 0.0;
    for (int c = threadIdx.x; c < ncell; c += TAIL_BS) {
        int i = c % d.IMM1 + 1, k = c / d.IMM1 + 1;
        s -= (double)A3(d.FLOWX, i, j, k);
    }
    __shared__ double sh[TAIL_BS / 32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < TAIL_BS / 32; ++w) t += sh[w];
        d.BLADE_FLOW[j - 1] = t * (double)A1(d.NBLADE, j);
    }
}

// finishes the |W|^2 reduction of k_prim: VREF and VMAX
__global__ void k_tail_vref(Dev d, int nparts) {
    DevCtl *c = d.ctl;
    if (!c->do_tail) return;
    double s = 0.0;
    unsigned long long key = 0ull;
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) {
        s += d.part_sum[p];
        unsigned long long k2 = d.part_key[p];
        key = k2 > key ? k2 : key;
    }
    __shared__ double ss[32];
    __shared__ unsigned long long sk[32];
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        unsigned long long ok = __shfl_down_sync(0xffffffffu, key, o);
        key = ok > key ? ok : key;
    }
    if ((threadIdx.x & 31) == 0) {
        ss[threadIdx.x >> 5] = s;
        sk[threadIdx.x >> 5] = key;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        unsigned long long kk = 0ull;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            t += ss[w];
            kk = sk[w] > kk ? sk[w] : kk;
        }
        c->mon.vrms = t;
        float vrms = (float)t;
        c->VREF = sqrtf(vrms * d.RIJKM);
        if (kk) {
            unsigned lin = 0xFFFFFFFFu - (unsigned)(kk & 0xFFFFFFFFull);
            float v = __uint_as_float((unsigned)(kk >> 32));
            c->VMAX = sqrtf(v);
            c->IVMAX = (int)(lin % d.IM) + 1;
            c->JVMAX = (int)((lin / d.IM) % d.JM) + 1;
            c->KVMAX = (int)(lin / ((unsigned)d.IM * d.JM)) + 1;
        } else {
            c->VMAX = 0.0f;
        }
    }
}

__global__ void __launch_bounds__(TAIL_BS) k_tail_dvm(Dev d) {
    const DevCtl *c = d.ctl;
    if (!c->do_tail) return;
    size_t n = (size_t)blockIdx.x * TAIL_BS + threadIdx.x;
    size_t N = (size_t)d.IM * d.JM * d.KM;
    double s = 0.0;
    unsigned long long key = 0ull;
    int bad = 0;
    if (n < N) {
        int i, j, k;
        node_ijk(d, n, i, j, k);
        float ro = d.RO[n];
        if (!isfinite(ro) || !(ro > 0.0f) || !isfinite(d.ROE[n]) || !isfinite(d.ROVX[n]) || !isfinite(d.ROVR[n]) ||
            !isfinite(d.RORVT[n]))
            bad = 1;
        if (j >= 2) {
            float RVEF = 100.0f / c->VREF;
            float XD = A2(d.DX, j, k), RD = A2(d.DR, j, k), SD = A2(d.DS, j, k);
            float VM_START = (XD * d.VX[n] + RD * d.VR[n]) / SD;
            float VM_END = (XD * d.ROVX[n] + RD * d.ROVR[n]) / SD / ro;
            float DVMER = (VM_END - VM_START) * RVEF;
            d.STORE[n] = DVMER;
            s = (double)fabsf(DVMER);
            key = max_key(fabsf(DVMER), n);
        }
    }
    __shared__ double ss[TAIL_BS / 32];
    __shared__ unsigned long long sk[TAIL_BS / 32];
    __shared__ int sc[TAIL_BS / 32];
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        unsigned long long ok = __shfl_down_sync(0xffffffffu, key, o);
        key = ok > key ? ok : key;
        bad += __shfl_down_sync(0xffffffffu, bad, o);
    }
    int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        ss[w] = s;
        sk[w] = key;
        sc[w] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        unsigned long long kk = 0ull;
        int cnt = 0;
        for (int q = 0; q < TAIL_BS / 32; ++q) {
            t += ss[q];
            kk = sk[q] > kk ? sk[q] : kk;
            cnt += sc[q];
        }
        d.part_sum[blockIdx.x] = t;
        d.part_key[blockIdx.x] = kk;
        d.part_cnt[blockIdx.x] = cnt;
    }
}

__global__ void k_tail_final(Dev d, int nparts) {
    DevCtl *c = d.ctl;
    if (!c->do_tail) return;
    double s = 0.0;
    unsigned long long key = 0ull;
    int bad = 0;
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) {
        s += d.part_sum[p];
        unsigned long long k2 = d.part_key[p];
        key = k2 > key ? k2 : key;
        bad += d.part_cnt[p];
    }
    __shared__ double ss[32];
    __shared__ unsigned long long sk[32];
    __shared__ int sc[32];
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        unsigned long long ok = __shfl_down_sync(0xffffffffu, key, o);
        key = ok > key ? ok : key;
        bad += __shfl_down_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
        ss[threadIdx.x >> 5] = s;
        sk[threadIdx.x >> 5] = key;
        sc[threadIdx.x >> 5] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        unsigned long long kk = 0ull;
        int cnt = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            t += ss[w];
            kk = sk[w] > kk ? sk[w] : kk;
            cnt += sc[w];
        }
        c->mon.eavg_sum = t;
        c->EAVG = (float)t / (float)(d.IM * d.JMM1 * d.KM);
        if (kk) {
            unsigned lin = 0xFFFFFFFFu - (unsigned)(kk & 0xFFFFFFFFull);
            c->EMAX = d.STORE[lin];
            c->IMAXE = (int)(lin % d.IM) + 1;
            c->JMAXE = (int)((lin / d.IM) % d.JM) + 1;
            c->KMAXE = (int)(lin / ((unsigned)d.IM * d.JM)) + 1;
        } else {
            c->EMAX = 0.0f;
        }
        c->health = cnt;
        // continuity error ECONT and its station
        double cf1 = d.BLADE_FLOW[0];
        float econt = 0.0f;
        int jc = c->JCONT;
        for (int j = 1; j <= d.JM; ++j) {
            float RATIO = (float)d.BLADE_FLOW[j - 1] / (float)cf1;
            float EMASS = fabsf(1.0f - RATIO);
            if (EMASS > econt) {
                econt = EMASS;
                jc = j;
            }
        }
        c->ECONT = econt;
        c->JCONT = jc;
        c->flow_in = d.BLADE_FLOW[0];
        c->flow_out = d.BLADE_FLOW[d.JM - 1];
        if ((c->EAVG < d.CONLIM && c->ECONT < 0.01f) || (fabsf(c->EMAX) < 4.0f * d.CONLIM && c->ECONT < 0.01f))
            c->converged = 1;
    }
}

void launch_tail(const Dev &d, Launch L) {
    k_tail_flow<<<d.JM, TAIL_BS, 0, L.s>>>(d);
    mark(L, "k_tail_flow");
    size_t N = (size_t)d.IM * d.JM * d.KM;
    int prim_parts = (int)grid_for(N, 256);
    k_tail_vref<<<1, 1024, 0, L.s>>>(d, prim_parts);
    mark(L, "k_tail_vref");
    int parts = (int)grid_for(N, TAIL_BS);
    k_tail_dvm<<<parts, TAIL_BS, 0, L.s>>>(d);
    mark(L, "k_tail_dvm");
    k_tail_final<<<1, 1024, 0, L.s>>>(d, parts);
    mark(L, "k_tail_final");
}

// ---------------------------------------------------------------------
// STEPUP(RELAX) (7916-8002): local time step ~ c/(|W|+c), relaxed
// ---------------------------------------------------------------------
__global__ void k_stepup_node(Dev d, int gated) {
    if (gated && !d.ctl->do_tail) return;
    size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t N = (size_t)d.IM * d.JM * d.KM;
    if (n >= N) return;
    float TLIM = 0.1f * A1(d.TO1, d.KMID);
    float VLIM = 0.01f * A1(d.VM1, d.KMID) * A1(d.VM1, d.KMID);
    float vx = d.VX[n], vt = d.VT[n], vr = d.VR[n];
    float VSQ = vx * vx + vt * vt + vr * vr;
    float HSTAT = d.HO[n] - 0.5f * VSQ;
    float TSTATIC = HSTAT * d.RCP;
    if (TSTATIC < TLIM) TSTATIC = TLIM;
    float WTREL = d.WT[n];
    float WSQ = VSQ - (vt * vt - WTREL * WTREL);
    if (WSQ < VLIM) WSQ = VLIM;
    float V_SONIC = sqrtf(d.GA * d.RGAS * TSTATIC);
    float VPLUSC = sqrtf(WSQ) + V_SONIC;
    d.TEMP1[n] = d.VSOUND / VPLUSC;
}

__device__ inline float stepup_cell(const Dev &d, int i, int j, int k, float RELAX) {
    const float *T = d.TEMP1;
    int ip1 = i + 1, kp1 = k + 1;
    float AMACHP;
    if (j == 2)
        AMACHP = A3(T, i, 1, k) + A3(T, ip1, 1, k) + A3(T, i, 1, kp1) + A3(T, ip1, 1, kp1);
    else
        AMACHP = A3(T, i, j - 1, k) + A3(T, i, j - 1, kp1) + A3(T, ip1, j - 1, k) + A3(T, ip1, j - 1, kp1);
    float AMACHL = A3(T, i, j, k) + A3(T, i, j, kp1) + A3(T, ip1, j, k) + A3(T, ip1, j, kp1);
    float AVMACH = 0.125f * (AMACHL + AMACHP);
    float STEPNEW = A3(d.BSTEP, i, j, k) * AVMACH;
    return RELAX * STEPNEW + (1.0f - RELAX) * A3(d.STEP, i, j, k);
}

__global__ void k_stepup_cell(Dev d, float RELAX, int gated) {
    if (gated && !d.ctl->do_tail) return;
    size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t N = (size_t)d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, n, i, j, k);
    if (i >= d.IM || j < 2 || k >= d.KM) return;
    float step = stepup_cell(d, i, j, k, RELAX);
    float rstep = step / d.BSTEP[n];
    if (A1(d.INDMIX, j - 1) == 1 && j < d.JM) {     // J = JMIX+1: take the step of JMIX+2
        step = stepup_cell(d, i, j + 1, k, RELAX);
        rstep = 0.0f;
    }
    // the JMIX+2 cell reads its own old STEP in stepup_cell, so write after
    // every reader of this cell's old value: STEP(I,J,K) is only read by
    // this cell and by the JMIX+1 cell below it, which recomputes it.
    d.TMP[n] = step;
    d.STORE[n] = rstep;
}

__global__ void k_stepup_store(Dev d, int gated) {
    if (gated && !d.ctl->do_tail) return;
    size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t N = (size_t)d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, n, i, j, k);
    if (i >= d.IM || j < 2 || k >= d.KM) return;
    d.STEP[n] = d.TMP[n];
    d.RSTEP[n] = d.STORE[n];
}

void launch_stepup(const Dev &d, Launch L, float relax, bool gated) {
    size_t N = (size_t)d.IM * d.JM * d.KM;
    unsigned g = grid_for(N, 256);
    k_stepup_node<<<g, 256, 0, L.s>>>(d, gated ? 1 : 0);
    mark(L, "k_stepup_node");
    k_stepup_cell<<<g, 256, 0, L.s>>>(d, relax, gated ? 1 : 0);
    mark(L, "k_stepup_cell");
    k_stepup_store<<<g, 256, 0, L.s>>>(d, gated ? 1 : 0);
    mark(L, "k_stepup_store");
}

// ---------------------------------------------------------------------
// EFICOOL node quantities (5610) and SUMFLX mass averages per J, FP64
// ---------------------------------------------------------------------
__global__ void k_int_node(Dev d) {
    size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t N = (size_t)d.IM * d.JM * d.KM;
    if (n >= N) return;
    float TO1M = A1(d.TO1, d.KMID), PO1M = A1(d.PO1, d.KMID);
    float vx = d.VX[n], vt = d.VT[n], vr = d.VR[n];
    float EKE = 0.5f * (vx * vx + vt * vt + vr * vr);
    float TS = (d.HO[n] - EKE) * d.RCP;
    float TSTAG = d.HO[n] * d.RCP;
    if (TSTAG < 0.1f * TO1M) TSTAG = 0.1f * TO1M;
    if (TS < 0.1f * TO1M) TS = 0.1f * TO1M;
    float PSTAT = d.P[n];
    if (PSTAT < 0.02f * PO1M) PSTAT = 0.02f * PO1M;
    float PSTAG = PSTAT * powf(TSTAG / TS, d.RFGA);
    d.TEMP1[n] = TSTAG;       // TEMP1: stagnation temperature
    d.TMP[n] = PSTAG / PO1M;  // TEMP2: stagnation pressure ratio
}

__global__ void __launch_bounds__(TAIL_BS) k_int_sum(Dev d, double *out) {
    int j = blockIdx.x + 1;
    int ncell = d.IMM1 * d.KMM1;
    double bf = 0, spo = 0, sto = 0, sps = 0;
    double nb = (double)A1(d.NBLADE, j);
    for (int c = threadIdx.x; c < ncell; c += TAIL_BS) {
        int i = c % d.IMM1 + 1, k = c / d.IMM1 + 1;
        double DFLOW = -(double)A3(d.FLOWX, i, j, k) * nb;
        double DFLOW4 = 0.25 * DFLOW;
        bf += DFLOW;
        spo += DFLOW4 * ((double)A3(d.TMP, i, j, k) + A3(d.TMP, i + 1, j, k) + A3(d.TMP, i + 1, j, k + 1) + A3(d.TMP, i, j, k + 1));
        sto += DFLOW4 * ((double)A3(d.TEMP1, i, j, k) + A3(d.TEMP1, i + 1, j, k) + A3(d.TEMP1, i + 1, j, k + 1) +
                         A3(d.TEMP1, i, j, k + 1));
        sps += DFLOW4 * ((double)A3(d.P, i, j, k) + A3(d.P, i + 1, j, k) + A3(d.P, i + 1, j, k + 1) + A3(d.P, i, j, k + 1));
    }
    __shared__ double sh[4][TAIL_BS / 32];
    double v[4] = {bf, spo, sto, sps};
    for (int q = 0; q < 4; ++q) {
        double x = v[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) sh[q][threadIdx.x >> 5] = x;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0.0;
        for (int w = 0; w < TAIL_BS / 32; ++w) t += sh[threadIdx.x][w];
        out[(size_t)threadIdx.x * d.JM + (j - 1)] = t;
    }
}

void launch_integrals(const Dev &d, Launch L, double *out) {
    size_t N = (size_t)d.IM * d.JM * d.KM;
    k_int_node<<<grid_for(N, 256), 256, 0, L.s>>>(d);
    mark(L, "k_int_node");
    k_int_sum<<<d.JM, TAIL_BS, 0, L.s>>>(d, out);
    mark(L, "k_int_sum");
}

}  // namespace mgpu
