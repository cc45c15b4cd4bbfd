// mgpu_loss.cu -- the viscous body forces of SUBROUTINE LOSS (ILOS=10,
// multall-open-18.3.f:8058-9066) with the Shih wall functions WALLFUN
// (15980-16047) and, for YPLUSWALL < -10, the pressure gradients of
// SET_PWALLGRAD (16052-16114); the every-5-step tail of LOOP (monitors
// 5264-5317 and STEPUP 7916-8002); and the EFICOOL/SUMFLX mass averages
// (10662-10849, 7873-7912).
//
// LOSS is two passes over the grid: the streamwise (K) faces for every
// (I,J) column, then the bladewise (I) faces for every (J,K) line.
#include "mgpu_internal.cuh"

namespace mgpu {

static inline unsigned grid_for(size_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }


// viscosity set on entry to LOSS (8088-8112); one thread
__global__ void k_loss_prologue(Dev d, int init_call) {
    pdl_wait();
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

// Shih et al. wall function (WALLFUN).  DPDS is the caller's DPDS_CELL
// element: with YPLUSWALL <= -10 the pressure-gradient term is added and,
// as the Fortran argument does, |DPDS| < 1 is raised to 1.0 in place.
__device__ inline void wallfun(float PERP, float &DPDS, float DENSITY, float &TWALL, float YPLUS_OLD, float WREL_WALL,
                               float &YPLUS_NEW, float VISLAM, float YPLUSWALL) {
    float SGN_DPDS = 0.0f, VPRES = 0.0f, VSTAR_P = 0.0f, FYPLUSP = 0.0f;
    const bool pres = !(YPLUSWALL > -10.0f);
    if (pres) {
        if (fabsf(DPDS) < 1.0f) DPDS = 1.0f;
        SGN_DPDS = fabsf(DPDS) / DPDS;
        VPRES = powf(VISLAM / DENSITY / DENSITY * fabsf(DPDS), 0.33333f);
        VSTAR_P = YPLUS_OLD * VISLAM / (DENSITY * PERP);
        if (SGN_DPDS < 0.0f && VPRES > 0.33f * VSTAR_P) VPRES = 0.33f * VSTAR_P;
        if (SGN_DPDS > 0.0f && VPRES > 2.0f * VSTAR_P) VPRES = 2.0f * VSTAR_P;
        float YPLUS_PRES = VPRES * PERP * DENSITY / VISLAM;
        float P1 = YPLUS_PRES, P2 = P1 * P1, P3 = P2 * P1, P4 = P2 * P2;
        if (P1 <= 4.0f) FYPLUSP = 0.5f * P2 - 7.31E-3f * P3;
        if (P1 > 4.0f && P1 <= 15.0f) FYPLUSP = -15.138f + 8.4688f * P1 - 0.81976f * P2 + 3.7292E-2f * P3 - 6.3866E-4f * P4;
        if (P1 > 15.0f && P1 <= 30.0f) FYPLUSP = 11.925f + 0.934f * P1 - 2.7805E-2f * P2 + 4.6262E-4f * P3 - 3.1442E-6f * P4;
        if (P1 > 30.0f) FYPLUSP = 5.0f * logf(P1) + 8.0f;
    }
    float YP1 = YPLUS_OLD, YP2 = YP1 * YP1, YP3 = YP2 * YP1, YP4 = YP2 * YP2;
    float FYPLUS = 0.0f;
    if (YP1 <= 5.0f) FYPLUS = YP1 + 1.0E-2f * YP2 - 2.9E-03f * YP3;
    if (YP1 > 5.0f && YP1 <= 30.0f) FYPLUS = -0.872f + 1.465f * YP1 - 7.02E-2f * YP2 + 1.66E-03f * YP3 - 1.495E-5f * YP4;
    if (YP1 > 30.0f && YP1 <= 140.0f) FYPLUS = 8.6f + 0.1864f * YP1 - 2.006E-3f * YP2 + 1.144E-5f * YP3 - 2.551E-8f * YP4;
    if (YP1 > 140.0f) FYPLUS = 2.439f * logf(YP1) + 5.0f;
    float FRACP = pres ? SGN_DPDS * (VPRES / VSTAR_P) * FYPLUSP / FYPLUS : 0.0f;
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
// SET_PWALLGRAD (16052-16114), run at the start of LOSS when YPLUSWALL <
// -10.  k_pwallgrad_cells: one thread per cell, the streamwise pressure
// gradient from GRADVEL (13468-13508) of PEFF along the cell's relative
// velocity, limited by DPDS_LIM.  k_pwallgrad_smooth: the smoothing along J
// within each row, sequential in J and across rows as the reference runs it;
// one warp takes 32 (I,K) columns staged in shared memory.  The last row
// reaches J = JM+1 .. JM+4, storage the reference never writes otherwise:
// those reads give 0 and the writes are dropped.
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_pwallgrad_cells(const __grid_constant__ Dev d, int init_call) {
    pdl_wait();
    if (!init_call && !d.ctl->do_loss) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int IMM1 = d.IMM1, KMM1 = d.KMM1;
    if (t >= IMM1 * KMM1 * (d.JM - 1)) return;
    const int i = t % IMM1 + 1, q = t / IMM1, k = q % KMM1 + 1, j = q / KMM1 + 2;
    float PDIV = 0.5f * (d.ctl->PDOWN_HUB + d.ctl->PDOWN_TIP);
    PDIV = PDIV / (float)d.NROWS;
    PDIV = PDIV / (A1(d.CHORD, 1) + A1(d.CHORD, d.NROWS));
    const float DPDS_LIM = fabsf(20.0f * (A1(d.PO1, d.KMID) - PDIV));
    const int sJ = d.IM, sK = d.IM * d.JM;
    const int n = ix3(d, i, j, k);
    // node offsets of the cell's corners: (i | i+1, j-1 | j, k | k+1)
    const int o000 = n, o100 = n + 1, o0m0 = n - sJ, o1m0 = n + 1 - sJ;
    const int o001 = n + sK, o101 = n + 1 + sK, o0m1 = n - sJ + sK, o1m1 = n + 1 - sJ + sK;
    const float *V = d.PEFF;
    const float RVOL = 0.25f / d.VOL[n];
    const float VAVGJ1 = V[o0m0] + V[o1m0] + V[o1m1] + V[o0m1];
    const float VAVGJ2 = V[o000] + V[o100] + V[o101] + V[o001];
    const float VAVGI1 = V[o000] + V[o0m0] + V[o0m1] + V[o001];
    const float VAVGI2 = V[o100] + V[o1m0] + V[o1m1] + V[o101];
    const float VAVGK1 = V[o000] + V[o100] + V[o1m0] + V[o0m0];
    const float VAVGK2 = V[o001] + V[o101] + V[o1m1] + V[o0m1];
    const float VAVGCELL = 0.125f * (VAVGJ1 + VAVGJ2);
    const float DPDX = -((VAVGJ2 * d.AQX[n] - VAVGJ1 * d.AQX[n - sJ] + VAVGI1 * d.ABX[n] - VAVGI2 * d.ABX[n + 1] +
                          VAVGK1 * d.ASX[n] - VAVGK2 * d.ASX[n + sK]) *
                         RVOL);
    const float DPDR = -((VAVGJ2 * d.AQR[n] - VAVGJ1 * d.AQR[n - sJ] + VAVGI1 * d.ABR[n] - VAVGI2 * d.ABR[n + 1] +
                          VAVGK1 * d.ASR[n] - VAVGK2 * d.ASR[n + sK]) *
                         RVOL) -
                       VAVGCELL / A2(d.RAVG_CELL, j, k);
    const float DPDT = -((VAVGI1 - VAVGI2) * A2(d.ABT, j, k) * RVOL);
    auto c8 = [&](const float *A) {
        return A[o000] + A[o0m0] + A[o100] + A[o1m0] + A[o001] + A[o0m1] + A[o101] + A[o1m1];
    };
    const float VXCELL = c8(d.VX), VRCELL = c8(d.VR), WTCELL = c8(d.WT);
    const float WREL_CELL = sqrtf(VXCELL * VXCELL + VRCELL * VRCELL + WTCELL * WTCELL);
    float DPDS = (DPDX * VXCELL + DPDR * VRCELL + DPDT * WTCELL) / WREL_CELL;
    if (fabsf(DPDS) > DPDS_LIM) DPDS = DPDS_LIM * DPDS / fabsf(DPDS);
    d.DPDS_CELL[n] = DPDS;
}

__global__ void __launch_bounds__(32) k_pwallgrad_smooth(const __grid_constant__ Dev d, int init_call) {
    pdl_wait();
    if (!init_call && !d.ctl->do_loss) return;
    extern __shared__ float col[];                 // [JM + 4][32], plane J at row J-1
    const int lane = threadIdx.x;
    const int i = blockIdx.x * 32 + lane + 1, k = blockIdx.y + 1;
    const bool act = i <= d.IMM1;
    const int JM = d.JM;
    const int sK = d.IM * JM;
    float *base = d.DPDS_CELL + (i - 1) + sK * (k - 1);
#define CJ(jj) col[((jj) - 1) * 32 + lane]
    for (int jj = 1; jj <= JM + 4; ++jj) CJ(jj) = (act && jj <= JM) ? base[(jj - 1) * d.IM] : 0.0f;
    if (act) {
        for (int nr = 1; nr <= d.NROWS; ++nr) {
            const int J1 = A1(d.JSTART, nr), J2 = A1(d.JMIX, nr);
            auto ends = [&]() {
                CJ(J2 + 1) = 0.0f;
                CJ(J2 + 2) = 2.0f * CJ(J2 + 3) - CJ(J2 + 4);
                CJ(J2) = 2.0f * CJ(J2 - 1) - CJ(J2 - 2);
            };
            ends();
            // TEMPP(J) = 0.5 D(J) + 0.25 (D(J-1) + D(J+1)) for J1+2..J2-1 from the
            // unsmoothed values, then D(J) = 0.5 T(J) + 0.25 (T(J-1) + T(J+1)) for
            // J1+3..J2-2: one pass with TEMPP in three registers, each D(J)
            // overwritten only after TEMPP(J+1) has read it
            if (J2 - 2 >= J1 + 3) {
                float tm = 0.5f * CJ(J1 + 2) + 0.25f * (CJ(J1 + 1) + CJ(J1 + 3));
                float tc = 0.5f * CJ(J1 + 3) + 0.25f * (CJ(J1 + 2) + CJ(J1 + 4));
                for (int jj = J1 + 3; jj <= J2 - 2; ++jj) {
                    float tp = 0.5f * CJ(jj + 1) + 0.25f * (CJ(jj) + CJ(jj + 2));
                    CJ(jj) = 0.5f * tc + 0.25f * (tm + tp);
                    tm = tc;
                    tc = tp;
                }
            }
            ends();
        }
    }
    __syncwarp();
    if (act)
        for (int jj = 1; jj <= JM; ++jj) base[(jj - 1) * d.IM] = CJ(jj);
#undef CJ
}

// ---------------------------------------------------------------------
// stresses on the streamwise (K = const) faces, LOSS DO 50 (8208-8556).
// One CTA = 32 consecutive I-columns of one J-plane (threadIdx.x = I,
// threadIdx.y = a K stride of LK_W), every column's K-line staged in shared
// memory ([K][32] arrays, K rows 1..KM), so each load instruction reads 32
// consecutive pitchwise points.  The per-column wall functions and the
// transition scans run one thread per column in the reference's order.
// ---------------------------------------------------------------------
constexpr int LK_W = 8;            // warps per CTA (K stride)
constexpr int LK_NARR = 8;         // [K][32] arrays in shared memory (+ RAVG per K): 4 CTAs per SM at KM = 49

__global__ void __launch_bounds__(32 * LK_W) k_loss_kfaces(const __grid_constant__ Dev d, int init_call) {
    pdl_wait();
    const DevCtl *c = d.ctl;
    if (!init_call && !c->do_loss) return;
    extern __shared__ float lsm[];
    const int KM = d.KM, KMM1 = d.KMM1, KMID = d.KMID;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i = blockIdx.x * 32 + tx + 1;
    const int j = blockIdx.y + 2;
    const bool col = i <= d.IMM1;
    // [K][32] arrays, row k-1
    float *AREA = lsm, *VXAVG = AREA + KM * 32, *VRAVG = VXAVG + KM * 32, *VTAVG = VRAVG + KM * 32;
    float *ROAVG = VTAVG + KM * 32, *TAVG = ROAVG + KM * 32;
    float *VLAM = TAVG + KM * 32, *VTURB = VLAM + KM * 32, *RAVGK = VTURB + KM * 32;   // RAVGK: [K] only
    __shared__ float s_vis[32], s_ftc[32], s_tw1[32], s_twm[32];
    __shared__ float s_w1[32][4], s_wm[32][4];     // wall-face xs, rs, ts, wv at K=1 and K=KM
#define LK(a, k) a[((k) - 1) * 32 + tx]
    const float RF_VIS = init_call ? 1.0f : d.RF_VIS;
    const float FMIXUP = init_call ? 1.0f : c->FMIXUP;
    const int NRW = A1(d.NROW, j);
    const float WREL = A1(d.WRAD, j), WHUB = A1(d.WHUB, j), WTIP = A1(d.WTIP, j);
    // 1. face averages
    for (int k = ty + 1; k <= KM; k += LK_W) {
        float RAVG = 0.5f * (A2(d.R, j, k) + A2(d.R, j - 1, k));
        if (tx == 0) RAVGK[k - 1] = RAVG;
        if (!col) continue;
        float asx = A3(d.ASX, i, j, k), asr = A3(d.ASR, i, j, k);
        float vx = 0.25f * (A3(d.VX, i, j, k) + A3(d.VX, i, j - 1, k) + A3(d.VX, i + 1, j, k) + A3(d.VX, i + 1, j - 1, k));
        float vr = 0.25f * (A3(d.VR, i, j, k) + A3(d.VR, i, j - 1, k) + A3(d.VR, i + 1, j, k) + A3(d.VR, i + 1, j - 1, k));
        float vt = 0.25f * (A3(d.VT, i, j, k) + A3(d.VT, i, j - 1, k) + A3(d.VT, i + 1, j, k) + A3(d.VT, i + 1, j - 1, k));
        LK(AREA, k) = sqrtf(asx * asx + asr * asr);
        LK(VXAVG, k) = vx;
        LK(VRAVG, k) = vr;
        LK(VTAVG, k) = vt;
        LK(ROAVG, k) = 0.25f * (A3(d.RO, i, j, k) + A3(d.RO, i, j - 1, k) + A3(d.RO, i + 1, j, k) + A3(d.RO, i + 1, j - 1, k));
        LK(TAVG, k) = 0.25f * (A3(d.T_STATIC, i, j, k) + A3(d.T_STATIC, i, j - 1, k) + A3(d.T_STATIC, i + 1, j, k) +
                               A3(d.T_STATIC, i + 1, j - 1, k));
    }
    __syncthreads();
    // 2. viscosity and wall shear stresses, one thread per column
    auto wbound = [&](int k) {
        float WTB = LK(VTAVG, k) - (k > KMID ? WTIP : WHUB) * RAVGK[k - 1];
        return sqrtf(LK(VXAVG, k) * LK(VXAVG, k) + LK(VRAVG, k) * LK(VRAVG, k) + WTB * WTB);
    };
    if (ty == 0 && col) {
        float VISLAM = c->VISLAM, FTCOND = c->FTCOND;
        if (d.REYNO < 0.0001f) {
            VISLAM = (fabsf(d.REYNO) / 100000.0f) * powf(LK(TAVG, KMID) / 288.0f, 0.62f);
            float TCOND = d.CP * VISLAM / d.PRANDTL;
            FTCOND = TCOND / VISLAM;
        }
        float TWALLK1, TWALLKM;
        if (d.YPLUSWALL < -0.001f) {
            float PERPK1 = A3(d.VOL, i, j, 1) / LK(AREA, 1);
            float ynew;
            wallfun(PERPK1, A3(d.DPDS_CELL, i, j, 1), LK(ROAVG, 1), TWALLK1, AIJ(d.YPLUS_K1, i, j), wbound(1), ynew, VISLAM,
                    d.YPLUSWALL);
            AIJ(d.YPLUS_K1, i, j) = fminf(1000.0f, ynew);
        } else if (d.YPLUSWALL < 5.0f) {
            float PERP = A3(d.VOL, i, j, 1) / LK(AREA, 1);
            float RE = PERP * LK(ROAVG, 2) * wbound(2) / VISLAM;
            TWALLK1 = skin_friction(RE, PERP, A1(d.ROUGH_H, NRW), LK(ROAVG, 2), wbound(2), VISLAM);
        } else {
            float wb = wbound(1);
            TWALLK1 = d.CFWALL * LK(ROAVG, 1) * wb * wb;
        }
        if (d.YPLUSWALL < -0.001f) {
            float PERPKM = A3(d.VOL, i, j, KMM1) / LK(AREA, KM);
            float ynew;
            wallfun(PERPKM, A3(d.DPDS_CELL, i, j, KMM1), LK(ROAVG, KMM1), TWALLKM, AIJ(d.YPLUS_KM, i, j), wbound(KMM1), ynew,
                    VISLAM, d.YPLUSWALL);
            AIJ(d.YPLUS_KM, i, j) = fminf(1000.0f, ynew);
        } else if (d.YPLUSWALL < 5.0f) {
            float PERP = A3(d.VOL, i, j, KMM1) / LK(AREA, KM);
            float RE = PERP * LK(ROAVG, KMM1) * wbound(KMM1) / VISLAM;
            TWALLKM = skin_friction(RE, PERP, A1(d.ROUGH_T, NRW), LK(ROAVG, KMM1), wbound(KMM1), VISLAM);
        } else {
            float wb = wbound(KM);
            TWALLKM = d.CFWALL * LK(ROAVG, KM) * wb * wb;
        }
        s_vis[tx] = VISLAM;
        s_ftc[tx] = FTCOND;
        s_tw1[tx] = TWALLK1;
        s_twm[tx] = TWALLKM;
        // the two wall faces (K=1 hub, K=KM casing)
        float FMULT = TWALLK1 * LK(AREA, 1) / wbound(1);
        if (d.IBOUND == 1 || d.IBOUND > 2) FMULT = 0.0f;
        float WTB1 = LK(VTAVG, 1) - (1 > KMID ? WTIP : WHUB) * RAVGK[0];
        float ts1 = FMULT * WTB1;
        s_w1[tx][0] = FMULT * LK(VXAVG, 1);
        s_w1[tx][1] = FMULT * LK(VRAVG, 1);
        s_w1[tx][2] = ts1;
        s_w1[tx][3] = ts1 * WHUB * RAVGK[0];
        float FMULTM = -TWALLKM * LK(AREA, KM) / wbound(KM);
        if (d.IBOUND >= 2) FMULTM = 0.0f;
        float WTBM = LK(VTAVG, KM) - (KM > KMID ? WTIP : WHUB) * RAVGK[KM - 1];
        float tsm = FMULTM * WTBM;
        s_wm[tx][0] = FMULTM * LK(VXAVG, KM);
        s_wm[tx][1] = FMULTM * LK(VRAVG, KM);
        s_wm[tx][2] = tsm;
        s_wm[tx][3] = tsm * WTIP * RAVGK[KM - 1];
    }
    __syncthreads();
    // 3. Y_PLUS from the wall nearer in K
    if (col) {
        const float VISLAM = s_vis[tx];
        const float VS1 = sqrtf(s_tw1[tx] / LK(ROAVG, 1)), VSM = sqrtf(s_twm[tx] / LK(ROAVG, KM));
        for (int k = ty + 1; k <= KMM1; k += LK_W) {
            float PERP = sqrtf(A3(d.DWALLSQ, i, j, k));
            float y = k <= KMID ? VS1 * PERP * LK(ROAVG, 1) / VISLAM : VSM * PERP * LK(ROAVG, KM) / VISLAM;
            y = fminf(y, 1000.0f);
            A3(d.Y_PLUS, i, j, k) = y;
        }
    }
    __syncthreads();
    // 4. laminar and mixing-length viscosities of the interior faces.  The
    //    relative speed of the faces is formed again here, and Y_PLUS is read
    //    back from this CTA's own stores of step 3 (visible after the
    //    barrier): two K-arrays fewer in shared memory lets four CTAs share
    //    an SM
    auto wabs = [&](int kq) {
        float WTAVG = LK(VTAVG, kq) - WREL * RAVGK[kq - 1];
        return sqrtf(LK(VXAVG, kq) * LK(VXAVG, kq) + LK(VRAVG, kq) * LK(VRAVG, kq) + WTAVG * WTAVG);
    };
    if (col) {
        const float VISLAM = s_vis[tx];
        for (int k = ty + 2; k <= KMM1; k += LK_W) {
            // FYPLUS keeps its previous value where Y_PLUS is NaN
            int kk = k;
            while (kk >= 2 && isnan(A3(d.Y_PLUS, i, j, kk))) --kk;
            float FYPLUS = kk >= 2 ? fyplus_of(A3(d.Y_PLUS, i, j, kk), d.YPLAM, d.YPTURB, 0.0f) : 0.0f;
            float DPERP = A3(d.VOL, i, j, k) / LK(AREA, k);
            LK(VLAM, k) = d.FKLAM[(size_t)(NRW - 1) * KM + k - 1] * VISLAM / DPERP;
            float vt = d.FKTURB[(size_t)(NRW - 1) * KM + k - 1] * LK(ROAVG, k) * fabsf(wabs(k + 1) - wabs(k - 1)) *
                       FMIXUP;
            LK(VTURB, k) = vt * FYPLUS;
        }
    }
    __syncthreads();
    // 5. transition, hub half then casing half (the casing scan sees the
    //    hub half's result at KMID)
    if (ty == 0 && col) {
        const int JROW = j - A1(d.JSTART, NRW) + 1;
        float *vt = VTURB + tx, *vl = VLAM + tx;   // column view, stride 32
        auto scan = [&](int a, int b) {
            float RMAX = 0.0f;
            for (int q = a; q <= b; ++q) {
                float RATVIS = vt[(q - 1) * 32] / vl[(q - 1) * 32];
                if (RATVIS < RMAX) continue;
                RMAX = RATVIS;
            }
            return RMAX > d.FTRANS;
        };
        bool turb = !(JROW < A1(d.JTRAN_K1, NRW)) && scan(2, KMID);
        if (!turb)
            for (int q = 2; q <= KMID; ++q) vt[(q - 1) * 32] = 0.0f;
        turb = !(JROW < A1(d.JTRAN_KM, NRW)) && scan(KMID, KMM1);
        if (!turb)
            for (int q = KMID; q <= KMM1; ++q) vt[(q - 1) * 32] = 0.0f;
    }
    __syncthreads();
    // 6. stresses on faces K and K+1 of each cell, body forces relaxed by RF_VIS
    if (col) {
        const float VISLAM = s_vis[tx], FTCOND = s_ftc[tx];
        const float RF_VIS1 = 1.0f - RF_VIS;
        auto face = [&](int kp, float &xs, float &rs, float &ts, float &qf, float &wv) {
            if (kp == 1) {
                xs = s_w1[tx][0]; rs = s_w1[tx][1]; ts = s_w1[tx][2]; qf = 0.0f; wv = s_w1[tx][3];
            } else if (kp == KM) {
                xs = s_wm[tx][0]; rs = s_wm[tx][1]; ts = s_wm[tx][2]; qf = 0.0f; wv = s_wm[tx][3];
            } else {
                float vl = LK(VLAM, kp), vtu = LK(VTURB, kp), ar = LK(AREA, kp);
                float FM = ar * (vl + vtu);
                xs = FM * (LK(VXAVG, kp + 1) - LK(VXAVG, kp - 1));
                rs = FM * (LK(VRAVG, kp + 1) - LK(VRAVG, kp - 1));
                float VISTOT = VISLAM * (1.0f + vtu / vl);
                ts = FM * (LK(VTAVG, kp + 1) - LK(VTAVG, kp - 1)) - VISTOT * ar * LK(VTAVG, kp) / RAVGK[kp - 1];
                qf = FM * FTCOND * (LK(TAVG, kp + 1) - LK(TAVG, kp - 1));
                wv = xs * LK(VXAVG, kp) + ts * LK(VTAVG, kp) + rs * LK(VRAVG, kp);
            }
        };
        for (int k = ty + 1; k <= KMM1; k += LK_W) {
            float xl, rl, tl, ql, wl, xh, rh, th, qh, wh;
            face(k, xl, rl, tl, ql, wl);
            face(k + 1, xh, rh, th, qh, wh);
            size_t n = ix3(d, i, j, k);
            d.XFORCE[n] = RF_VIS1 * d.XFORCE[n] + RF_VIS * (xl - xh);
            d.RFORCE[n] = RF_VIS1 * d.RFORCE[n] + RF_VIS * (rl - rh);
            d.TFORCE[n] = RF_VIS1 * d.TFORCE[n] + RF_VIS * (tl * RAVGK[k - 1] - th * RAVGK[k]);
            d.QSOURCE[n] = RF_VIS1 * d.QSOURCE[n] + RF_VIS * (ql - qh + wl - wh);
        }
    }
#undef LK
}

// ---------------------------------------------------------------------
// stresses on the bladewise (I = const) faces and the blade surfaces,
// LOSS DO 100 (8566-9044).  One warp per (J,K) line; the lanes cover I (coalesced), the
// line's arrays sit in this warp's slice of shared memory.
// ---------------------------------------------------------------------
constexpr int LI_W = 4;            // warps (lines) per CTA; 64 registers: 8 CTAs per SM
constexpr int LI_NARR = 16;        // per-line arrays of IM+1 floats

// Transition test of one wall's mixing-length viscosity (LOSS 8481-8510,
// 8823-8852): the reference keeps RMAX = the running value of
// "IF(RATVIS.LT.RMAX) skip, else RMAX = RATVIS" from RMAX = 0 and switches
// the wall turbulent if RMAX > FTRANS.  Without a NaN that is
// max(0, ratios) > FTRANS; a NaN ratio resets RMAX, so only the ratios after
// the last NaN count (and none after it leaves RMAX = NaN: laminar).  The
// lanes of one warp evaluate it over vt[a..b] / vl[a..b].
__device__ inline bool transition_warp(const float *vt, const float *vl, int a, int b, float FTRANS) {
    const int lane = threadIdx.x & 31;
    int lastnan = a - 1;
    for (int q0 = a; q0 <= b; q0 += 32) {
        int q = q0 + lane;
        float r = q <= b ? vt[q] / vl[q] : 0.0f;
        bool nan = q <= b && isnan(r);
        unsigned m = __ballot_sync(0xffffffffu, nan);
        if (m) lastnan = q0 + 31 - __clz((int)m);
    }
    bool t = false;
    for (int q0 = a; q0 <= b; q0 += 32) {
        int q = q0 + lane;
        if (q <= b && q > lastnan) {
            float r = vt[q] / vl[q];
            if (r > FTRANS) t = true;
        }
    }
    bool any = __any_sync(0xffffffffu, t);
    if (lastnan < a) any = any || (0.0f > FTRANS);
    return any;
}

__global__ void __launch_bounds__(32 * LI_W, 8) k_loss_ifaces(const __grid_constant__ Dev d, int init_call) {
    pdl_wait();
    const DevCtl *c = d.ctl;
    if (!init_call && !c->do_loss) return;
    extern __shared__ float lsm[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int line = blockIdx.x * LI_W + w;
    if (line >= (d.JM - 1) * d.KMM1) return;     // whole warps leave together
    const int k = line % d.KMM1 + 1, j = line / d.KMM1 + 2;
    const int IM = d.IM, IMM1 = d.IMM1, IMID = d.IMID;
    const int L = IM + 1;
    float *base = lsm + (size_t)w * LI_NARR * L;
    float *AREA = base, *VXAVG = AREA + L, *VRAVG = VXAVG + L, *VTAVG = VRAVG + L, *WTAVG = VTAVG + L;
    float *ROAVG = WTAVG + L, *TAVG = ROAVG + L, *WABS = TAVG + L, *YP = WABS + L, *VLAM = YP + L;
    float *VTURB = VLAM + L, *XSTRES = VTURB + L, *RSTRES = XSTRES + L, *TSTRES = RSTRES + L;
    float *QFLOW = TSTRES + L, *WVISC = QFLOW + L;
    const float RF_VIS = init_call ? 1.0f : d.RF_VIS;
    const float FMIXUP = init_call ? 1.0f : c->FMIXUP;
    float VISLAM = c->VISLAM, FTCOND = c->FTCOND;
    const int NRW = A1(d.NROW, j);
    const int JROW = j - A1(d.JSTART, NRW) + 1;
    const int JLEDGE = A1(d.JLE, NRW), JTEDGE = A1(d.JTE, NRW);
    const float WREL = A1(d.WRAD, j);
    const float RAVGK = A2(d.RAVG_CELL, j, k);
    const float abt = A2(d.ABT, j, k);
    for (int i = lane + 1; i <= IM; i += 32) {
        float abx = A3(d.ABX, i, j, k), abr = A3(d.ABR, i, j, k);
        AREA[i] = sqrtf(abx * abx + abr * abr + abt * abt);
        float vx = 0.25f * (A3(d.VX, i, j, k) + A3(d.VX, i, j - 1, k) + A3(d.VX, i, j - 1, k + 1) + A3(d.VX, i, j, k + 1));
        float vr = 0.25f * (A3(d.VR, i, j, k) + A3(d.VR, i, j - 1, k) + A3(d.VR, i, j - 1, k + 1) + A3(d.VR, i, j, k + 1));
        float wt = 0.25f * (A3(d.WT, i, j, k) + A3(d.WT, i, j - 1, k) + A3(d.WT, i, j - 1, k + 1) + A3(d.WT, i, j, k + 1));
        VXAVG[i] = vx;
        VRAVG[i] = vr;
        VTAVG[i] = 0.25f * (A3(d.VT, i, j, k) + A3(d.VT, i, j - 1, k) + A3(d.VT, i, j - 1, k + 1) + A3(d.VT, i, j, k + 1));
        WTAVG[i] = wt;
        ROAVG[i] = 0.25f * (A3(d.RO, i, j, k) + A3(d.RO, i, j - 1, k) + A3(d.RO, i, j - 1, k + 1) + A3(d.RO, i, j, k + 1));
        TAVG[i] = 0.25f * (A3(d.T_STATIC, i, j, k) + A3(d.T_STATIC, i, j - 1, k) + A3(d.T_STATIC, i, j - 1, k + 1) +
                           A3(d.T_STATIC, i, j, k + 1));
        float WABSQ = vx * vx + vr * vr + wt * wt;
        WABS[i] = sqrtf(WABSQ);
    }
    __syncwarp();
    if (d.REYNO < 0.0001f) {
        VISLAM = (fabsf(d.REYNO) / 100000.0f) * powf(TAVG[IMID] / 288.0f, 0.62f);
        float TCOND = d.CP * VISLAM / d.PRANDTL;
        FTCOND = TCOND / VISLAM;
    }
    const float *FIL = d.FILAM + (size_t)(NRW - 1) * IM;
    const float *FIT = d.FITURB + (size_t)(NRW - 1) * IM;
    const float *FIW = d.FIWAKE + (size_t)(NRW - 1) * IM;
    const float *FIU = d.FIUP + (size_t)(NRW - 1) * IM;
    const bool in_blade = !(j <= JLEDGE || j > JTEDGE);
    const bool in_gap = (A1(d.KTIPS, NRW) > 0) && (k >= A1(d.KTIPS, NRW)) && (k < A1(d.KTIPE, NRW));
    if (in_blade) {
        if (!in_gap) {
            // wall shear on the two blade surfaces: lane 0 the I=1 side, lane 1 the I=IM side
            float TW = 0.0f;
            if (lane < 2) {
                const bool lo = lane == 0;
                const int iw = lo ? 1 : IM, ia = lo ? 1 : IMM1, ib = lo ? 2 : IMM1;
                if (d.YPLUSWALL < -0.001f) {
                    float PERPW = A3(d.VOL, ia, j, k) / AREA[iw];
                    float ynew;
                    float *yw = lo ? &A2(d.YPLUS_I1, j, k) : &A2(d.YPLUS_IM, j, k);
                    wallfun(PERPW, A3(d.DPDS_CELL, ia, j, k), ROAVG[ia], TW, *yw, WABS[ib], ynew, VISLAM, d.YPLUSWALL);
                    *yw = fminf(1000.0f, ynew);
                } else if (d.YPLUSWALL < 5.0f) {
                    float PERP = A3(d.VOL, ia, j, k) / AREA[iw];
                    float RE = ROAVG[ib] * WABS[ib] * PERP / VISLAM;
                    TW = skin_friction(RE, PERP, lo ? A1(d.ROUGH_L, NRW) : A1(d.ROUGH_U, NRW), ROAVG[ib], WABS[ib], VISLAM);
                } else {
                    TW = d.CFWALL * ROAVG[iw] * WABS[iw] * WABS[iw];
                }
            }
            const float TWALLI1 = __shfl_sync(0xffffffffu, TW, 0), TWALLIM = __shfl_sync(0xffffffffu, TW, 1);
            const float VS1 = sqrtf(TWALLI1 / ROAVG[1]), VSM = sqrtf(TWALLIM / ROAVG[IM]);
            for (int i = lane + 1; i <= IMM1; i += 32) {
                float YPLS = i <= IMID ? VS1 * sqrtf(A3(d.DWALLSQ, i, j, k)) * ROAVG[1] / VISLAM
                                       : VSM * sqrtf(A3(d.DWALLSQ, i, j, k)) * ROAVG[IM] / VISLAM;
                float YPLSP = A3(d.Y_PLUS, i, j, k);
                float y = fminf(YPLS, YPLSP);
                A3(d.Y_PLUS, i, j, k) = y;
                YP[i] = y;
            }
            if (lane == 0) {
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
        } else {
            for (int i = lane + 2; i <= IMM1; i += 32) YP[i] = A3(d.Y_PLUS, i, j, k);
        }
        __syncwarp();
        for (int i = lane + 2; i <= IMM1; i += 32) {
            int ii = i;     // FYPLUS keeps its previous value where Y_PLUS is NaN
            while (ii >= 2 && isnan(YP[ii])) --ii;
            float FYPLUS = ii >= 2 ? fyplus_of(YP[ii], d.YPLAM, d.YPTURB, 0.0f) : 0.0f;
            float DPERP = A3(d.VOL, i, j, k) / AREA[i];
            VLAM[i] = FIL[i - 1] * VISLAM / DPERP;
            float vt = FIT[i - 1] * ROAVG[i] * fabsf(WABS[i + 1] - WABS[i - 1]) * FMIXUP;
            VTURB[i] = vt * FYPLUS;
        }
        __syncwarp();
        bool turb = !(JROW < A1(d.JTRAN_I1, NRW)) && transition_warp(VTURB, VLAM, 2, IMID, d.FTRANS);
        if (!turb)
            for (int i = lane + 2; i <= IMID; i += 32) VTURB[i] = 0.0f;
        __syncwarp();
        turb = !(JROW < A1(d.JTRAN_IM, NRW)) && transition_warp(VTURB, VLAM, IMID, IMM1, d.FTRANS);
        if (!turb)
            for (int i = lane + IMID; i <= IMM1; i += 32) VTURB[i] = 0.0f;
        __syncwarp();
        for (int i = lane + 2; i <= IMM1; i += 32) {
            float FM = (VLAM[i] + VTURB[i]) * AREA[i];
            float xs = FM * (VXAVG[i + 1] - VXAVG[i - 1]);
            float rs = FM * (VRAVG[i + 1] - VRAVG[i - 1]);
            float ts = FM * (WTAVG[i + 1] - WTAVG[i - 1]);
            XSTRES[i] = xs;
            RSTRES[i] = rs;
            TSTRES[i] = ts;
            A3(d.VISC_RAT, i, j, k) = VTURB[i] / VLAM[i];
            QFLOW[i] = FM * FTCOND * (TAVG[i + 1] - TAVG[i - 1]);
            WVISC[i] = xs * VXAVG[i] + rs * VRAVG[i] + ts * VTAVG[i];
        }
        __syncwarp();
        if (in_gap && lane == 0) {
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
        const bool wake = j > JTEDGE;
        if (wake) {
            FACJ = 0.1f * (float)(j - JTEDGE);
            if (FACJ > 1.0f) FACJ = 1.0f;
        }
        for (int i = lane + 1; i <= IM; i += 32) {
            int ISUB = (i == IM) ? IMM1 : i;
            int IM1 = (i == 1) ? IMM1 : i - 1;
            int IP1 = (i == IM) ? 2 : i + 1;
            float DPERP = A3(d.VOL, ISUB, j, k) / AREA[i];
            float vl = FIL[i - 1] * VISLAM / DPERP;
            float vt;
            if (wake) {
                float FBLEND = (FACJ * FIW[i - 1] + (1.0f - FACJ) * FIT[i - 1]) * FMIXUP;
                vt = FBLEND * ROAVG[i] * fabsf(WABS[IP1] - WABS[IM1]);
            } else {
                vt = FMIXUP * FIU[i - 1] * ROAVG[i] * fabsf(WABS[IP1] - WABS[IM1]);
            }
            A3(d.VISC_RAT, i, j, k) = vt / vl;
            float FM = AREA[i] * (vl + vt);
            float xs = FM * (VXAVG[IP1] - VXAVG[IM1]);
            float rs = FM * (VRAVG[IP1] - VRAVG[IM1]);
            float ts = FM * (WTAVG[IP1] - WTAVG[IM1]);
            XSTRES[i] = xs;
            RSTRES[i] = rs;
            TSTRES[i] = ts;
            QFLOW[i] = FM * FTCOND * (TAVG[IP1] - TAVG[IM1]);
            WVISC[i] = xs * VXAVG[i] + ts * VTAVG[i] + rs * VRAVG[i];
        }
        __syncwarp();
        if (lane == 0) {
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
    }
    __syncwarp();
    for (int i = lane + 1; i <= IMM1; i += 32) {
        size_t n = ix3(d, i, j, k);
        d.XFORCE[n] = d.XFORCE[n] + RF_VIS * (XSTRES[i] - XSTRES[i + 1]);
        d.RFORCE[n] = d.RFORCE[n] + RF_VIS * (RSTRES[i] - RSTRES[i + 1]);
        d.TFORCE[n] = d.TFORCE[n] + RF_VIS * (TSTRES[i] - TSTRES[i + 1]) * RAVGK;
        d.QSOURCE[n] = d.QSOURCE[n] + RF_VIS * (QFLOW[i] - QFLOW[i + 1] + WVISC[i] - WVISC[i + 1]);
    }
}

size_t pwallgrad_smem(const Dev &d) { return (size_t)(d.JM + 4) * 32 * sizeof(float); }
size_t loss_kfaces_smem(const Dev &d) { return ((size_t)LK_NARR * d.KM * 32 + d.KM) * sizeof(float); }
size_t loss_ifaces_smem(const Dev &d) { return (size_t)LI_W * LI_NARR * (d.IM + 1) * sizeof(float); }

cudaError_t configure_loss_kernels(const Dev &d) {
    size_t kb = loss_kfaces_smem(d), ib = loss_ifaces_smem(d), pb = pwallgrad_smem(d);
    if (d.YPLUSWALL < -10.0f) {
        if (pb > 220 * 1024) return cudaErrorInvalidValue;
        cudaError_t e = raise_smem((const void *)k_pwallgrad_smooth, pb);
        if (e != cudaSuccess) return e;
    }
    if (kb > 220 * 1024 || ib > 220 * 1024) return cudaErrorInvalidValue;   // KM <= 160: kb <= 201 KB
    cudaError_t e = raise_smem((const void *)k_loss_kfaces, kb);
    if (e != cudaSuccess) return e;
    return raise_smem((const void *)k_loss_ifaces, ib);
}

void launch_loss(const Dev &d, Launch L, bool init_call) {
    if (d.ILOS == 0) return;            // inviscid: no loss routine is called (3935-3942, 7354-7356)
    if (d.ILOS >= 200) {
        launch_spal_loss(d, L, init_call);
        return;
    }
    if (d.ILOS >= 100) {
        launch_new_loss(d, L, init_call);
        return;
    }
    launchk(L, k_loss_prologue, dim3(1), dim3(1), 0, d, init_call ? 1 : 0);
    mark(L, "k_loss_prologue");
    if (d.YPLUSWALL < -10.0f) {
        int nc = d.IMM1 * d.KMM1 * (d.JM - 1);
        launchk(L, k_pwallgrad_cells, dim3((nc + 255) / 256), dim3(256), 0, d, init_call ? 1 : 0);
        mark(L, "k_pwallgrad_cells");
        launchk(L, k_pwallgrad_smooth, dim3((unsigned)((d.IMM1 + 31) / 32), (unsigned)d.KMM1), dim3(32),
                pwallgrad_smem(d), d, init_call ? 1 : 0);
        mark(L, "k_pwallgrad_smooth");
    }
    dim3 gk((unsigned)((d.IMM1 + 31) / 32), (unsigned)(d.JM - 1));
    launchk(L, k_loss_kfaces, dim3(gk), dim3(32, LK_W), loss_kfaces_smem(d), d, init_call ? 1 : 0);
    mark(L, "k_loss_kfaces");
    int nl = (d.JM - 1) * d.KMM1;
    launchk(L, k_loss_ifaces, dim3((nl + LI_W - 1) / LI_W), dim3(32 * LI_W), loss_ifaces_smem(d), d, init_call ? 1 : 0);
    mark(L, "k_loss_ifaces");
}

// ---------------------------------------------------------------------
// every-5-step tail: mass flow per J (5665-5677), % change of Vm
// (8500-8520) with EMAX/EAVG, VREF/VMAX, and a health count
// ---------------------------------------------------------------------
constexpr int TAIL_BS = 256;

__global__ void __launch_bounds__(TAIL_BS) k_tail_flow(Dev d) {
    pdl_wait();
    if (!d.ctl->do_tail) return;
    int j = blockIdx.x + 1;
    int ncell = d.IMM1 * d.KMM1;
    const int ro = d.REDUCE_ORDER;
    double s = 0.0;
    for (int c = threadIdx.x; c < ncell; c += TAIL_BS) {
        int i = c % d.IMM1 + 1, k = c / d.IMM1 + 1;
        s = racc(ro, s, -(double)A3(d.FLOWX, i, j, k));
    }
    __shared__ double sh[TAIL_BS / 32];
    for (int o = 16; o > 0; o >>= 1) s = racc(ro, s, __shfl_down_sync(0xffffffffu, s, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < TAIL_BS / 32; ++w) t = racc(ro, t, sh[w]);
        d.BLADE_FLOW[j - 1] = ro == 2 ? (double)((float)t * (float)A1(d.NBLADE, j)) : t * (double)A1(d.NBLADE, j);
    }
}

// finishes the |W|^2 reduction of k_prim: VREF and VMAX
__global__ void k_tail_vref(Dev d, int nparts) {
    pdl_wait();
    DevCtl *c = d.ctl;
    if (!c->do_tail) return;
    const int ro = d.REDUCE_ORDER;
    double s = 0.0;
    unsigned long long key = 0ull;
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) {
        s = racc(ro, s, d.part_sum[p]);
        unsigned long long k2 = d.part_key[p];
        key = k2 > key ? k2 : key;
    }
    __shared__ double ss[32];
    __shared__ unsigned long long sk[32];
    for (int o = 16; o > 0; o >>= 1) {
        s = racc(ro, s, __shfl_down_sync(0xffffffffu, s, o));
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
            t = racc(ro, t, ss[w]);
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

// Each thread of k_tail_dvm takes TAIL_NPT nodes (TAIL_BS apart, so the
// loads stay coalesced) and adds their |DVMER| in FP32 before the FP64 tree:
// GB300 issues few FP64 instructions per clock, and a tree per node kept
// the kernel on the FP64 pipe.
constexpr int TAIL_NPT = 8;

__global__ void __launch_bounds__(TAIL_BS) k_tail_dvm(Dev d) {
    pdl_wait();
    const DevCtl *c = d.ctl;
    if (!c->do_tail) return;
    const int N = d.IM * d.JM * d.KM;                   // below 2^31: commit limits the node count
    const float RVEF = 100.0f / c->VREF;
    float sf = 0.0f;
    unsigned long long key = 0ull;
    int bad = 0;
#pragma unroll 2
    for (int u = 0; u < TAIL_NPT; ++u) {
        const int n = ((int)blockIdx.x * TAIL_NPT + u) * TAIL_BS + (int)threadIdx.x;
        if (n >= N) break;
        const int jk = n / d.IM;                         // (j-1) + JM*(k-1)
        const bool jin = jk % d.JM != 0;                 // j >= 2
        float ro = d.RO[n];
        if (!isfinite(ro) || !(ro > 0.0f) || !isfinite(d.ROE[n]) || !isfinite(d.ROVX[n]) || !isfinite(d.ROVR[n]) ||
            !isfinite(d.RORVT[n]))
            bad += 1;
        if (jin) {
            float XD = d.DX[jk], RD = d.DR[jk], SD = d.DS[jk];
            float VM_START = (XD * d.VX[n] + RD * d.VR[n]) / SD;
            float VM_END = (XD * d.ROVX[n] + RD * d.ROVR[n]) / SD / ro;
            float DVMER = (VM_END - VM_START) * RVEF;
            d.STORE[n] = DVMER;
            sf += fabsf(DVMER);
            const unsigned long long kn = max_key(fabsf(DVMER), (size_t)n);
            key = kn > key ? kn : key;
        }
    }
    double s = (double)sf;
    __shared__ double ss[TAIL_BS / 32];
    __shared__ unsigned long long sk[TAIL_BS / 32];
    __shared__ int sc[TAIL_BS / 32];
    const int ro = d.REDUCE_ORDER;
    for (int o = 16; o > 0; o >>= 1) {
        s = racc(ro, s, __shfl_down_sync(0xffffffffu, s, o));
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
            t = racc(ro, t, ss[q]);
            kk = sk[q] > kk ? sk[q] : kk;
            cnt += sc[q];
        }
        d.part_sum[blockIdx.x] = t;
        d.part_key[blockIdx.x] = kk;
        d.part_cnt[blockIdx.x] = cnt;
    }
}

__global__ void k_tail_final(Dev d, int nparts) {
    pdl_wait();
    DevCtl *c = d.ctl;
    if (!c->do_tail) return;
    const int ro = d.REDUCE_ORDER;
    double s = 0.0;
    unsigned long long key = 0ull;
    int bad = 0;
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) {
        s = racc(ro, s, d.part_sum[p]);
        unsigned long long k2 = d.part_key[p];
        key = k2 > key ? k2 : key;
        bad += d.part_cnt[p];
    }
    // the continuity error ECONT = max over J of |1 - FLOW(J)/FLOW(1)| and
    // the first J that reaches it, one J per thread as a (value, J) key
    unsigned long long ek = 0ull;
    const float cf1f = (float)d.BLADE_FLOW[0];
    for (int j = threadIdx.x + 1; j <= d.JM; j += blockDim.x) {
        float RATIO = (float)d.BLADE_FLOW[j - 1] / cf1f;
        float EMASS = fabsf(1.0f - RATIO);
        if (EMASS > 0.0f) {
            const unsigned long long kj = max_key(EMASS, (size_t)(j - 1));
            ek = kj > ek ? kj : ek;
        }
    }
    __shared__ double ss[32];
    __shared__ unsigned long long sk[32], se[32];
    __shared__ int sc[32];
    for (int o = 16; o > 0; o >>= 1) {
        s = racc(ro, s, __shfl_down_sync(0xffffffffu, s, o));
        unsigned long long ok = __shfl_down_sync(0xffffffffu, key, o);
        key = ok > key ? ok : key;
        unsigned long long oe = __shfl_down_sync(0xffffffffu, ek, o);
        ek = oe > ek ? oe : ek;
        bad += __shfl_down_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
        ss[threadIdx.x >> 5] = s;
        sk[threadIdx.x >> 5] = key;
        se[threadIdx.x >> 5] = ek;
        sc[threadIdx.x >> 5] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        unsigned long long kk = 0ull, ke = 0ull;
        int cnt = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            t = racc(ro, t, ss[w]);
            kk = sk[w] > kk ? sk[w] : kk;
            ke = se[w] > ke ? se[w] : ke;
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
        // continuity error ECONT and its station (the reference's J loop
        // keeps the first J of the largest value; none above 0 keeps JCONT)
        float econt = 0.0f;
        int jc = c->JCONT;
        if (ke) {
            econt = __uint_as_float((unsigned)(ke >> 32));
            jc = (int)(0xFFFFFFFFu - (unsigned)(ke & 0xFFFFFFFFull)) + 1;
        }
        c->ECONT = econt;
        c->CHECK_FLOW_JM = (float)d.BLADE_FLOW[d.JM - 1];   // CHECK_FLOW(JM) for the throttle
        c->JCONT = jc;
        c->flow_in = d.BLADE_FLOW[0];
        c->flow_out = d.BLADE_FLOW[d.JM - 1];
        if ((c->EAVG < d.CONLIM && c->ECONT < 0.01f) || (fabsf(c->EMAX) < 4.0f * d.CONLIM && c->ECONT < 0.01f))
            c->converged = 1;
    }
}

void launch_tail(const Dev &d, Launch L) {
    launchk(L, k_tail_flow, dim3(d.JM), dim3(TAIL_BS), 0, d);
    mark(L, "k_tail_flow");
    size_t N = (size_t)d.IM * d.JM * d.KM;
    int prim_parts = (int)grid_for(N, 256);
    launchk(L, k_tail_vref, dim3(1), dim3(1024), 0, d, prim_parts);
    mark(L, "k_tail_vref");
    int parts = (int)grid_for(N, (size_t)TAIL_BS * TAIL_NPT);
    launchk(L, k_tail_dvm, dim3(parts), dim3(TAIL_BS), 0, d);
    mark(L, "k_tail_dvm");
    launchk(L, k_tail_final, dim3(1), dim3(1024), 0, d, parts);
    mark(L, "k_tail_final");
}

// ---------------------------------------------------------------------
// STEPUP(RELAX) (7916-8002): local time step ~ c/(|W|+c), relaxed
// ---------------------------------------------------------------------
__global__ void k_stepup_node(Dev d, int gated) {
    pdl_wait();
    if (gated && (!d.ctl->do_tail || d.FROZEN)) return;
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
    pdl_wait();
    if (gated && (!d.ctl->do_tail || d.FROZEN)) return;
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
    pdl_wait();
    if (gated && (!d.ctl->do_tail || d.FROZEN)) return;
    size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t N = (size_t)d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, n, i, j, k);
    if (i >= d.IM || j < 2 || k >= d.KM) return;
    const float step = d.TMP[n], rstep = d.STORE[n];   // both loads before the stores
    d.STEP[n] = step;
    d.RSTEP[n] = rstep;
}

void launch_stepup(const Dev &d, Launch L, float relax, bool gated) {
    size_t N = (size_t)d.IM * d.JM * d.KM;
    unsigned g = grid_for(N, 256);
    launchk(L, k_stepup_node, dim3(g), dim3(256), 0, d, gated ? 1 : 0);
    mark(L, "k_stepup_node");
    launchk(L, k_stepup_cell, dim3(g), dim3(256), 0, d, relax, gated ? 1 : 0);
    mark(L, "k_stepup_cell");
    launchk(L, k_stepup_store, dim3(g), dim3(256), 0, d, gated ? 1 : 0);
    mark(L, "k_stepup_store");
}

// ---------------------------------------------------------------------
// EFICOOL node quantities (5610) and SUMFLX mass averages per J, FP64
// ---------------------------------------------------------------------
__global__ void k_int_node(Dev d) {
    pdl_wait();
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
    pdl_wait();
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
    launchk(L, k_int_node, dim3(grid_for(N, 256)), dim3(256), 0, d);
    mark(L, "k_int_node");
    launchk(L, k_int_sum, dim3(d.JM), dim3(TAIL_BS), 0, d, out);
    mark(L, "k_int_sum");
}

// ---------------------------------------------------------------------
// NEW_LOSS (ILOS 100-199, 12522-13462): the eddy viscosity of a mixing
// length and the vorticity of the relative velocity, the full viscous
// stress tensor and heat flux from GRADVEL (13468-13508) in every cell,
// transition, the wall shear stress on the blade surfaces and endwalls (log
// law with roughness, or the Shih wall functions), and the stresses summed
// over the I and K faces into the body forces.  The reference scatters each
// face's stress into its two cells; here every cell gathers its faces in
// the order the reference adds them, so each force is the same FP32 sum.
//   k_loss_prologue (as LOSS)            VISLAM, FTCOND (12545-12568)
//   k_nl_cells        one thread a cell  strain rates, VISC_RAT, VISC_LAM (DO 150)
//   k_nl_transition   one CTA a J plane  laminar lines (DO 160)
//   k_pwallgrad_*     YPLUSWALL < -10    DPDS_CELL
//   k_nl_walls        one thread a wall face: shear stress and wall forces
//   k_nl_forces       one thread a cell  face sums, Y_PLUS, relaxation (DO 500)
// Work (d.NLS): the nine strain rates TXR TXX TXT TRR TRT TTT QXX QRR QTT
// (N each), then per wall face XF RF TF ES VSTAR 0.25*ROAVG for the I=1 and
// I=IM blade surfaces ((JM,KM) each) and the hub and casing ((IM,JM) each).
// ---------------------------------------------------------------------
size_t new_loss_work_floats(const Dev &d) {
    return (size_t)9 * d.IM * d.JM * d.KM + (size_t)12 * d.JM * d.KM + (size_t)12 * d.IM * d.JM;
}

// the log-law skin friction of NEW_LOSS with roughness (12879-12925 and its
// three copies), written on the sums of four corner values RO4 and W4
__device__ inline float nl_twall(float RE, float DPERP, float ROUGH, float RO4, float W4, float VISLAM) {
    const float RELOG = 1.0f / logf(RE);
    float CF;
    if (ROUGH > 1.0E-7f) {
        if (ROUGH > DPERP) ROUGH = DPERP;
        float REK = RE * ROUGH / DPERP;
        REK = REK - 80.0f;
        if (REK < 0.0f) REK = 0.0f;
        const float REKSQ = REK * REK;
        const float A1c = -.00178493f + .0000814923f * REK + .000000150445f * REKSQ;
        const float A2c = .029072f - .001584f * REK - .00000225194f * REKSQ;
        const float A3c = .270313f + .0091409f * REK + .00000451537f * REKSQ + .00000000464767f * REKSQ * REK;
        CF = A1c + A2c * RELOG + A3c * RELOG * RELOG;
    } else {
        CF = -0.00178493f + 0.029072f * RELOG + 0.270313f * RELOG * RELOG;
    }
    const float CFLAM = 2.0f / RE;
    CF = fmaxf(CF, CFLAM);
    if (RE < 125.0f) CF = CFLAM;
    if (ROUGH > 1.0E-7f) {
        const float TW = CF * RO4 * W4 * W4 / 128.0f;
        const float VSTAR = sqrtf(TW / (RO4 / 4.0f));
        const float PLUSK = ROUGH * VSTAR * RO4 / VISLAM / 4.0f;
        const float RELOG10 = log10f(DPERP / ROUGH);
        const float FUNCN = 5.75f * RELOG10 + 8.5f;
        const float CF_FULL_ROUGH = 2.0f / (FUNCN * FUNCN);
        if (PLUSK > 45.0f && CF > CF_FULL_ROUGH) CF = CF_FULL_ROUGH;
    }
    return CF * RO4 * W4 * W4 / 128.0f;
}

// the cell (i, j, k), i fastest, of thread t; false past the last cell
__device__ inline bool nl_cell(const Dev &d, int t, int &i, int &j, int &k) {
    const int IMM1 = d.IMM1, JC = d.JM - 1;
    if (t >= IMM1 * JC * d.KMM1) return false;
    i = t % IMM1 + 1;
    const int q = t / IMM1;
    j = q % JC + 2;
    k = q / JC + 1;
    return true;
}

// cell-average density for NEW_LOSS, every step after TSTEP(RO) (4255-4267)
__global__ void __launch_bounds__(256) k_roavg_cell(const __grid_constant__ Dev d) {
    pdl_wait();
    int i, j, k;
    if (!nl_cell(d, blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const int sJ = d.IM, sK = d.IM * d.JM, n = ix3(d, i, j, k);
    const float *A = d.RO;
    d.ROAVG_CELL[n] = 0.125f * (A[n] + A[n + 1] + A[n + 1 + sK] + A[n + sK] + A[n - sJ] + A[n + 1 - sJ] +
                                A[n + 1 - sJ + sK] + A[n - sJ + sK]);
}

void launch_roavg_cell(const Dev &d, Launch L) {
    const int nc = d.IMM1 * d.KMM1 * (d.JM - 1);
    launchk(L, k_roavg_cell, dim3((nc + 255) / 256), dim3(256), 0, d);
    mark(L, "k_roavg_cell");
}

// DO 150: strain rates, vorticity, the eddy viscosity and its ratio
__global__ void __launch_bounds__(256) k_nl_cells(const __grid_constant__ Dev d, int init_call) {
    pdl_wait();
    const DevCtl *c = d.ctl;
    if (!init_call && !c->do_loss) return;
    int i, j, k;
    if (!nl_cell(d, blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const int sJ = d.IM, sK = d.IM * d.JM, n = ix3(d, i, j, k);
    const int o000 = n, o100 = n + 1, o0m0 = n - sJ, o1m0 = n + 1 - sJ;
    const int o001 = n + sK, o101 = n + 1 + sK, o0m1 = n - sJ + sK, o1m1 = n + 1 - sJ + sK;
    const float FMIXUP = init_call ? 1.0f : c->FMIXUP;
    float VISLAM = c->VISLAM;
    auto avg8 = [&](const float *A) {
        return 0.125f * (A[o000] + A[o100] + A[o101] + A[o001] + A[o0m0] + A[o1m0] + A[o1m1] + A[o0m1]);
    };
    const float WTAVG = avg8(d.WT);
    const float ROAVG = d.ROAVG_CELL[n];
    const float TSAVG = avg8(d.T_STATIC);
    const float RAVG = A2(d.RAVG_CELL, j, k);
    const float RVOL = 0.25f / d.VOL[n];
    const float aqx0 = d.AQX[n], aqx1 = d.AQX[n - sJ], abx0 = d.ABX[n], abx1 = d.ABX[n + 1], asx0 = d.ASX[n],
                asx1 = d.ASX[n + sK];
    const float aqr0 = d.AQR[n], aqr1 = d.AQR[n - sJ], abr0 = d.ABR[n], abr1 = d.ABR[n + 1], asr0 = d.ASR[n],
                asr1 = d.ASR[n + sK];
    const float abt = A2(d.ABT, j, k);
    auto grad = [&](const float *V, float &dx, float &dr, float &dt) {
        const float VAVGJ1 = V[o0m0] + V[o1m0] + V[o1m1] + V[o0m1];
        const float VAVGJ2 = V[o000] + V[o100] + V[o101] + V[o001];
        const float VAVGI1 = V[o000] + V[o0m0] + V[o0m1] + V[o001];
        const float VAVGI2 = V[o100] + V[o1m0] + V[o1m1] + V[o101];
        const float VAVGK1 = V[o000] + V[o100] + V[o1m0] + V[o0m0];
        const float VAVGK2 = V[o001] + V[o101] + V[o1m1] + V[o0m1];
        const float VAVGCELL = 0.125f * (VAVGJ1 + VAVGJ2);
        dx = -((VAVGJ2 * aqx0 - VAVGJ1 * aqx1 + VAVGI1 * abx0 - VAVGI2 * abx1 + VAVGK1 * asx0 - VAVGK2 * asx1) * RVOL);
        dr = -((VAVGJ2 * aqr0 - VAVGJ1 * aqr1 + VAVGI1 * abr0 - VAVGI2 * abr1 + VAVGK1 * asr0 - VAVGK2 * asr1) * RVOL) -
             VAVGCELL / RAVG;
        dt = -((VAVGI1 - VAVGI2) * abt * RVOL);
    };
    float DVXDX, DVXDR, DVXDT, DVRDX, DVRDR, DVRDT, DWTDX, DWTDR, DWTDT, DTDX, DTDR, DTDT;
    grad(d.VX, DVXDX, DVXDR, DVXDT);
    grad(d.VR, DVRDX, DVRDR, DVRDT);
    grad(d.WT, DWTDX, DWTDR, DWTDT);
    grad(d.T_STATIC, DTDX, DTDR, DTDT);
    const float XLEN = d.XLENGTH[n], FST = d.FST_RAT[n], YP = d.Y_PLUS[n];
    const size_t N = (size_t)d.IM * d.JM * d.KM;
    float *W = d.NLS;
    W[n] = DVXDR + DVRDX;                      // TXR
    W[N + n] = DVXDX;                          // TXX
    W[2 * N + n] = DWTDX + DVXDT;              // TXT
    W[3 * N + n] = DVRDR;                      // TRR
    W[4 * N + n] = DWTDR + DVRDT - WTAVG / RAVG;   // TRT
    W[5 * N + n] = DWTDT;                      // TTT
    W[6 * N + n] = DTDX;                       // QXX
    W[7 * N + n] = DTDR;                       // QRR
    W[8 * N + n] = DTDT;                       // QTT
    const float VORTX = DVRDT - DWTDR - WTAVG / RAVG;
    const float VORTR = DWTDX - DVXDT;
    const float VORTT = DVXDR - DVRDX;
    float VORT = sqrtf(VORTX * VORTX + VORTR * VORTR + VORTT * VORTT);
    if (VORT > d.VORT_MAX) VORT = d.VORT_MAX;
    float TURBVIS_WALL = ROAVG * XLEN * VORT * FMIXUP;
    TURBVIS_WALL = TURBVIS_WALL * fyplus_of(YP, d.YPLAM, d.YPTURB, 0.0f);
    if (d.REYNO < 0.0001f) VISLAM = (fabsf(d.REYNO) / 100000.0f) * powf(TSAVG / 288.0f, 0.62f);
    float VISTOT = VISLAM * (1.0f + FST) + TURBVIS_WALL;
    const float VISLIM = d.TURBVIS_LIM * VISLAM;
    if (VISTOT > VISLIM) VISTOT = VISLIM;
    d.VISC_RAT[n] = VISTOT / VISLAM;
    d.VISC_LAM[n] = VISLAM;
}

// DO 160: a line whose largest viscosity ratio stays at or below FTRANS, or
// that lies upstream of its transition point, is laminar.  The hub and
// casing lines of every I come first, then the I=1 and I=IM lines of every
// K, as the reference orders them within a J plane.
__global__ void __launch_bounds__(128) k_nl_transition(const __grid_constant__ Dev d, int init_call) {
    pdl_wait();
    if (!init_call && !d.ctl->do_loss) return;
    const int j = blockIdx.x + 2;
    const int NRW = A1(d.NROW, j);
    const int JROW = j - A1(d.JSTART, NRW) + 1;
    const int KMID = d.KMID, IMID = d.IMID, KMM1 = d.KMM1, IMM1 = d.IMM1;
    float *VRAT = d.VISC_RAT;
    auto line = [&](bool upstream, int n0, int stride, int cnt) {
        bool lam = upstream;
        if (!lam) {
            float RMAX = 0.0f;
            for (int q = 0; q < cnt; ++q) {
                const float r = VRAT[n0 + q * stride];
                if (!(r < RMAX)) RMAX = r;
            }
            lam = !(RMAX > d.FTRANS);
        }
        if (lam)
            for (int q = 0; q < cnt; ++q) VRAT[n0 + q * stride] = 1.0f;
    };
    const int sK = d.IM * d.JM;
    for (int i = threadIdx.x + 1; i <= IMM1; i += blockDim.x) {
        line(JROW < A1(d.JTRAN_K1, NRW), ix3(d, i, j, 1), sK, KMID);
        line(JROW < A1(d.JTRAN_KM, NRW), ix3(d, i, j, KMID), sK, KMM1 - KMID + 1);
    }
    __syncthreads();
    for (int k = threadIdx.x + 1; k <= KMM1; k += blockDim.x) {
        line(JROW < A1(d.JTRAN_I1, NRW), ix3(d, 1, j, k), 1, IMID);
        line(JROW < A1(d.JTRAN_IM, NRW), ix3(d, IMID, j, k), 1, IMM1 - IMID + 1);
    }
    // the COMMON VISLAM leaves NEW_LOSS as the last cell's laminar viscosity
    if (blockIdx.x == 0 && threadIdx.x == 0 && d.REYNO < 0.0001f) d.ctl->VISLAM = A3(d.VISC_LAM, IMM1, d.JM, KMM1);
}

// the wall shear stress of one wall face and its force on the wall cell:
// the I=1 and I=IM blade surfaces of every (J,K) outside a tip gap
// (12825-13052), the hub and casing of every (I,J) (13168-13390)
__global__ void __launch_bounds__(256) k_nl_walls(const __grid_constant__ Dev d, int init_call) {
    pdl_wait();
    const DevCtl *c = d.ctl;
    if (!init_call && !c->do_loss) return;
    const int nb = (d.JM - 1) * d.KMM1, ne = (d.JM - 1) * d.IMM1;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * nb + 2 * ne) return;
    const float VISLAM = c->VISLAM;
    const float VISLAM16 = VISLAM * 16.0f;
    const size_t N = (size_t)d.IM * d.JM * d.KM, SB = (size_t)d.JM * d.KM, SE = (size_t)d.IM * d.JM;
    float *WB = d.NLS + 9 * N, *WE = WB + 12 * SB;
    const int sJ = d.IM, sK = d.IM * d.JM;
    if (t < 2 * nb) {
        const int side = t / nb, r = t % nb;
        const int j = r % (d.JM - 1) + 2, k = r / (d.JM - 1) + 1;
        const int NRW = A1(d.NROW, j);
        if (A1(d.IND, j) == 0) return;
        if (A1(d.KTIPS, NRW) > 0 && k >= A1(d.KTIPS, NRW) && k < A1(d.KTIPE, NRW)) return;
        const int iw = side == 0 ? 2 : d.IMM1;       // node line of the averages
        const int ic = side == 0 ? 1 : d.IMM1;       // wall cell
        const int ia = side == 0 ? 1 : d.IM;         // wall face
        const int a = ix3(d, iw, j, k);
        auto s4 = [&](const float *A) { return A[a] + A[a - sJ] + A[a - sJ + sK] + A[a + sK]; };
        const float VXAVG = s4(d.VX), VRAVG = s4(d.VR), WTAVG = s4(d.WT), ROAVG = s4(d.RO);
        const float WAVG = sqrtf(WTAVG * WTAVG + VXAVG * VXAVG + VRAVG * VRAVG);
        const int fa = ix3(d, ia, j, k);
        const float abt = A2(d.ABT, j, k);
        const float AREA = sqrtf(d.ABX[fa] * d.ABX[fa] + d.ABR[fa] * d.ABR[fa] + abt * abt);
        const int nc = ix3(d, ic, j, k);
        const float DPERP = d.VOL[nc] / AREA;
        float TW;
        if (d.YPLUSWALL < -0.001f) {
            float &yp = side == 0 ? A2(d.YPLUS_I1, j, k) : A2(d.YPLUS_IM, j, k);
            float YN;
            wallfun(DPERP, d.DPDS_CELL[nc], 0.25f * ROAVG, TW, yp, 0.25f * WAVG, YN, VISLAM, d.YPLUSWALL);
            yp = fminf(1000.0f, YN);
        } else {
            const float RE = DPERP * ROAVG * WAVG / VISLAM16;
            TW = nl_twall(RE, DPERP, side == 0 ? A1(d.ROUGH_L, NRW) : A1(d.ROUGH_U, NRW), ROAVG, WAVG, VISLAM);
        }
        const float DEN = 0.25f * ROAVG;
        const float FMULT = -TW * AREA / WAVG;
        const float TF = FMULT * WTAVG;
        const size_t o = (size_t)ix2(d, j, k);
        float *w = WB + (size_t)side * 6 * SB;
        // SPAL_LOSS sets Y_PLUS on the I = IM side up to I = IM itself (14236)
        if (d.ILOS >= 200 && side == 1) {
            const int m = ix3(d, d.IM, j, k);
            d.Y_PLUS[m] = fminf(1000.0f, sqrtf(TW / DEN) * sqrtf(d.DWALLSQ[m]) * DEN / VISLAM);
        }
        w[o] = FMULT * VXAVG;
        w[SB + o] = FMULT * VRAVG;
        w[2 * SB + o] = TF;
        w[3 * SB + o] = TF * A1(d.WRAD, j) * A2(d.RAVG_CELL, j, k);
        w[4 * SB + o] = sqrtf(TW / DEN);
        w[5 * SB + o] = DEN;
        return;
    }
    t -= 2 * nb;
    const int side = t / ne, r = t % ne;
    const int i = r % d.IMM1 + 1, j = r / d.IMM1 + 2;
    const int NRW = A1(d.NROW, j);
    const int kn = side == 0 ? 2 : d.KMM1;           // node line of the averages
    const int kc = side == 0 ? 1 : d.KMM1;           // wall cell
    const int ka = side == 0 ? 1 : d.KM;             // wall face
    const int a = ix3(d, i, j, kn);
    auto s4 = [&](const float *A) { return A[a] + A[a + 1] + A[a + 1 - sJ] + A[a - sJ]; };
    const float VXAVG = s4(d.VX), VRAVG = s4(d.VR), VTAVG = s4(d.VT), ROAVG = s4(d.RO);
    const float RAVG = A2(d.R, j, kn) + A2(d.R, j, kn) + A2(d.R, j - 1, kn) + A2(d.R, j - 1, kn);
    const float WW = side == 0 ? A1(d.WHUB, j) : A1(d.WTIP, j);
    const float WTAVG = VTAVG - WW * RAVG;
    const float WAVG = sqrtf(VXAVG * VXAVG + VRAVG * VRAVG + WTAVG * WTAVG);
    const int fa = ix3(d, i, j, ka);
    const float AREA = sqrtf(d.ASX[fa] * d.ASX[fa] + d.ASR[fa] * d.ASR[fa]);
    const int nc = ix3(d, i, j, kc);
    const float DPERP = d.VOL[nc] / AREA;
    float TW;
    if (d.YPLUSWALL < -0.001f) {
        float &yp = side == 0 ? AIJ(d.YPLUS_K1, i, j) : AIJ(d.YPLUS_KM, i, j);
        float YN;
        wallfun(DPERP, d.DPDS_CELL[nc], 0.25f * ROAVG, TW, yp, 0.25f * WAVG, YN, VISLAM, d.YPLUSWALL);
        yp = fminf(1000.0f, YN);
    } else {
        const float RE = DPERP * ROAVG * WAVG / VISLAM16;
        TW = nl_twall(RE, DPERP, side == 0 ? A1(d.ROUGH_H, NRW) : A1(d.ROUGH_T, NRW), ROAVG, WAVG, VISLAM);
    }
    const float DEN = 0.25f * ROAVG;
    float FMULT = -TW * AREA / WAVG;
    if (side == 0 ? (d.IBOUND == 1 || d.IBOUND > 2) : (d.IBOUND >= 2)) FMULT = 0.0f;
    const float TF = FMULT * WTAVG;
    const size_t o = (size_t)ixij(d, i, j);
    float *w = WE + (size_t)side * 6 * SE;
    w[o] = FMULT * VXAVG;
    w[SE + o] = FMULT * VRAVG;
    w[2 * SE + o] = TF;
    w[3 * SE + o] = TF * 0.25f * WW * RAVG;
    w[4 * SE + o] = sqrtf(TW / DEN);
    w[5 * SE + o] = DEN;
}

struct NlStress {
    float txr, txx, txt, trr, trt, ttt, qxx, qrr, qtt;
};

// DO 190 for one cell: the strain rates times the final viscosity
__device__ inline NlStress nl_stress(const Dev &d, const float *W, size_t N, int m) {
    const float VIS = d.VISC_RAT[m] * d.VISC_LAM[m];
    const float TH = d.CP * VIS / d.PRANDTL;
    const float VIS2 = 2.0f * VIS;
    NlStress s;
    s.txr = VIS * W[m];
    s.txx = VIS2 * W[N + m];
    s.txt = VIS * W[2 * N + m];
    s.trr = VIS2 * W[3 * N + m];
    s.trt = VIS * W[4 * N + m];
    s.ttt = VIS2 * W[5 * N + m];
    s.qxx = -TH * W[6 * N + m];
    s.qrr = -TH * W[7 * N + m];
    s.qtt = -TH * W[8 * N + m];
    return s;
}

// Each cell's forces: the blade-wall and periodic terms, its I faces, the
// endwall terms and its K faces, in the reference's order of addition; then
// Y_PLUS from the wall shear stresses, and the relaxation into XFORCE,
// RFORCE, TFORCE and QSOURCE (DO 500).
__global__ void __launch_bounds__(256) k_nl_forces(const __grid_constant__ Dev d, int init_call) {
    pdl_wait();
    const DevCtl *c = d.ctl;
    if (!init_call && !c->do_loss) return;
    int i, j, k;
    if (!nl_cell(d, blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const float VISLAM = c->VISLAM;
    const float RF_VIS = init_call ? 1.0f : d.RF_VIS;
    const size_t N = (size_t)d.IM * d.JM * d.KM, SB = (size_t)d.JM * d.KM, SE = (size_t)d.IM * d.JM;
    const float *W = d.NLS, *WB = W + 9 * N, *WE = WB + 12 * SB;
    const int sJ = d.IM, sK = d.IM * d.JM, n = ix3(d, i, j, k);
    const int IMM1 = d.IMM1, KMM1 = d.KMM1;
    const int NRW = A1(d.NROW, j), IND = A1(d.IND, j);
    const int KTS = A1(d.KTIPS, NRW), KTE = A1(d.KTIPE, NRW);
    const bool blade = IND != 0 && !(KTS > 0 && k >= KTS && k < KTE);
    // 13063: (IND(J).EQ.1).AND.(K.LT.KTIPS).OR.(K.GT.KTIPE) skips the periodic face
    const bool periodic = !((IND == 1 && k < KTS) || k > KTE);
    const float xf0 = d.XFORCE[n], rf0 = d.RFORCE[n], tf0 = d.TFORCE[n], qs0 = d.QSOURCE[n];
    const float ravg = A2(d.RAVG_CELL, j, k), dw = sqrtf(d.DWALLSQ[n]), yp0 = d.Y_PLUS[n];
    auto wb = [&](int side, int f) { return WB[((size_t)side * 6 + f) * SB + (size_t)ix2(d, j, k)]; };
    auto we = [&](int side, int f) { return WE[((size_t)side * 6 + f) * SE + (size_t)ixij(d, i, j)]; };
    auto iface = [&](int I, int cI, int cmI, float &XF, float &RF, float &TF, float &Q, float &WV) {
        const NlStress a = nl_stress(d, W, N, ix3(d, cI, j, k)), b = nl_stress(d, W, N, ix3(d, cmI, j, k));
        const int f = ix3(d, I, j, k);
        const float abr = d.ABR[f], abx = d.ABX[f], abt = A2(d.ABT, j, k);
        XF = 0.5f * ((a.txr + b.txr) * abr + (a.txt + b.txt) * abt + (a.txx + b.txx) * abx);
        RF = 0.5f * ((a.trr + b.trr) * abr + (a.trt + b.trt) * abt + (a.txr + b.txr) * abx);
        TF = 0.5f * ((a.trt + b.trt) * abr + (a.ttt + b.ttt) * abt + (a.txt + b.txt) * abx);
        Q = 0.5f * ((a.qxx + b.qxx) * abx + (a.qrr + b.qrr) * abr + (a.qtt + b.qtt) * abt);
        const float vx = d.VX[f] + d.VX[f - sJ] + d.VX[f - sJ + sK] + d.VX[f + sK];
        const float vr = d.VR[f] + d.VR[f - sJ] + d.VR[f - sJ + sK] + d.VR[f + sK];
        const float vt = d.VT[f] + d.VT[f - sJ] + d.VT[f - sJ + sK] + d.VT[f + sK];
        WV = -0.25f * (XF * vx + RF * vr + TF * vt);
    };
    auto kface = [&](int K, float &XF, float &RF, float &TF, float &Q, float &WV) {
        const NlStress a = nl_stress(d, W, N, ix3(d, i, j, K)), b = nl_stress(d, W, N, ix3(d, i, j, K - 1));
        const int f = ix3(d, i, j, K);
        const float asr = d.ASR[f], asx = d.ASX[f];
        XF = 0.5f * ((a.txr + b.txr) * asr + (a.txx + b.txx) * asx);
        RF = 0.5f * ((a.trr + b.trr) * asr + (a.txr + b.txr) * asx);
        TF = 0.5f * ((a.trt + b.trt) * asr + (a.txt + b.txt) * asx);
        Q = 0.5f * ((a.qxx + b.qxx) * asx + (a.qrr + b.qrr) * asr);
        const float vx = d.VX[f] + d.VX[f + 1] + d.VX[f + 1 - sJ] + d.VX[f - sJ];
        const float vr = d.VR[f] + d.VR[f + 1] + d.VR[f + 1 - sJ] + d.VR[f - sJ];
        const float vt = d.VT[f] + d.VT[f + 1] + d.VT[f + 1 - sJ] + d.VT[f - sJ];
        WV = -0.25f * (XF * vx + RF * vr + TF * vt);
    };
    float fx = 0.0f, fr = 0.0f, ft = 0.0f, es = 0.0f;
    float XF, RF, TF, Q, WV;
    if (i == 1 || i == IMM1) {
        // FORCE*(1) and FORCE*(IM-1) after the blade-wall terms, then the
        // periodic face and the average of the two cells
        float p1[4] = {0.0f, 0.0f, 0.0f, 0.0f}, pm[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (blade)
            for (int f = 0; f < 4; ++f) {
                p1[f] = 0.0f + wb(0, f);
                pm[f] = 0.0f + wb(1, f);
            }
        if (periodic) {
            iface(1, 1, IMM1, XF, RF, TF, Q, WV);
            const float fl[3] = {XF, RF, TF};
            for (int f = 0; f < 3; ++f) {
                pm[f] = pm[f] + fl[f];
                p1[f] = p1[f] - fl[f];
                const float avg = 0.5f * (p1[f] + pm[f]);
                p1[f] = avg;
                pm[f] = avg;
            }
            p1[3] = p1[3] + Q + WV;
            pm[3] = pm[3] - Q - WV;
            const float avg = 0.5f * (p1[3] + pm[3]);
            p1[3] = avg;
            pm[3] = avg;
        }
        const float *p = i == 1 ? p1 : pm;
        fx = p[0];
        fr = p[1];
        ft = p[2];
        es = p[3];
    }
    if (i >= 2) {
        iface(i, i, i - 1, XF, RF, TF, Q, WV);
        fx = fx - XF;
        fr = fr - RF;
        ft = ft - TF;
        es = es + Q + WV;
    }
    if (i + 1 <= IMM1) {
        iface(i + 1, i + 1, i, XF, RF, TF, Q, WV);
        fx = fx + XF;
        fr = fr + RF;
        ft = ft + TF;
        es = es - Q - WV;
    }
    if (k == 1) {
        fx = fx + we(0, 0);
        fr = fr + we(0, 1);
        ft = ft + we(0, 2);
        es = es + we(0, 3);
    }
    if (k == KMM1) {
        fx = fx + we(1, 0);
        fr = fr + we(1, 1);
        ft = ft + we(1, 2);
        es = es + we(1, 3);
    }
    if (k >= 2) {
        kface(k, XF, RF, TF, Q, WV);
        fx = fx - XF;
        fr = fr - RF;
        ft = ft - TF;
        es = es + Q + WV;
    }
    if (k + 1 <= KMM1) {
        kface(k + 1, XF, RF, TF, Q, WV);
        fx = fx + XF;
        fr = fr + RF;
        ft = ft + TF;
        es = es - Q - WV;
    }
    // Y_PLUS: the blade surface of the cell's half pitch, then the lower of
    // that and the hub or casing value (12965-12970, 13036-13040, 13249-13257, 13365-13373)
    float yp = yp0;
    if (blade) {
        const int side = i <= d.IMID ? 0 : 1;
        yp = fminf(1000.0f, wb(side, 4) * dw * wb(side, 5) / VISLAM);
    }
    if (k <= d.KMID && (d.IBOUND == 0 || d.IBOUND == 2)) yp = fminf(we(0, 4) * dw * we(0, 5) / VISLAM, yp);
    if (k > d.KMID && d.IBOUND <= 1) yp = fminf(we(1, 4) * dw * we(1, 5) / VISLAM, yp);
    d.Y_PLUS[n] = yp;
    const float RF_VIS1 = 1.0f - RF_VIS;
    d.XFORCE[n] = RF_VIS1 * xf0 - RF_VIS * fx;
    d.TFORCE[n] = RF_VIS1 * tf0 - RF_VIS * ft * ravg;
    d.RFORCE[n] = RF_VIS1 * rf0 - RF_VIS * fr;
    d.QSOURCE[n] = RF_VIS1 * qs0 - RF_VIS * es;
}

void launch_loss_prologue(const Dev &d, Launch L, bool init_call) {
    launchk(L, k_loss_prologue, dim3(1), dim3(1), 0, d, init_call ? 1 : 0);
    mark(L, "k_loss_prologue");
}

void launch_pwallgrad(const Dev &d, Launch L, bool init_call) {
    const int ic = init_call ? 1 : 0;
    const int nc = d.IMM1 * d.KMM1 * (d.JM - 1);
    launchk(L, k_pwallgrad_cells, dim3((nc + 255) / 256), dim3(256), 0, d, ic);
    mark(L, "k_pwallgrad_cells");
    launchk(L, k_pwallgrad_smooth, dim3((unsigned)((d.IMM1 + 31) / 32), (unsigned)d.KMM1), dim3(32),
            pwallgrad_smem(d), d, ic);
    mark(L, "k_pwallgrad_smooth");
}

void launch_viscous_walls_and_forces(const Dev &d, Launch L, bool init_call) {
    const int ic = init_call ? 1 : 0;
    const int nc = d.IMM1 * d.KMM1 * (d.JM - 1);
    const int nw = 2 * (d.JM - 1) * d.KMM1 + 2 * (d.JM - 1) * d.IMM1;
    launchk(L, k_nl_walls, dim3((nw + 255) / 256), dim3(256), 0, d, ic);
    mark(L, "k_nl_walls");
    launchk(L, k_nl_forces, dim3((nc + 255) / 256), dim3(256), 0, d, ic);
    mark(L, "k_nl_forces");
}

void launch_new_loss(const Dev &d, Launch L, bool init_call) {
    const int ic = init_call ? 1 : 0;
    launch_loss_prologue(d, L, init_call);
    const int nc = d.IMM1 * d.KMM1 * (d.JM - 1);
    launchk(L, k_nl_cells, dim3((nc + 255) / 256), dim3(256), 0, d, ic);
    mark(L, "k_nl_cells");
    launchk(L, k_nl_transition, dim3(d.JM - 1), dim3(128), 0, d, ic);
    mark(L, "k_nl_transition");
    if (d.YPLUSWALL < -10.0f) launch_pwallgrad(d, L, init_call);
    launch_viscous_walls_and_forces(d, L, init_call);
}

}  // namespace mgpu
