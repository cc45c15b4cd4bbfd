// mgpu_tstep.cu -- SUBROUTINE TSTEP (multall-open-18.3.f:5470-5932) with
// SMOOTH_VAR (15352-15594) and SMOOTH_RESID (14833-14917) on the GPU.
//
// Per call, for one conserved variable D with its SCREE history DIFF:
//   prep     tip-gap TFLUX balance and mixing-plane flux extrapolation
//   delta    flux sum -> STORE, DIFF update (one thread per cell)
//   mp1      pitchwise redistribution of STORE at the mixing planes
//   restrict level-1/level-2 block sums, one thread per block walking its
//            cells in the reference's (K,J,I) order; per-J-plane sums (FP64)
//            for the superblocks
//   prolong  STORE*STEP + block corrections*RSTEP (one CTA per J-plane;
//            also the per-plane sum of |STORE| for the negative feedback)
//   avgblk   per-row mean |STORE| and its row smoothing (AVG_BLK)
//   damp     negative feedback, then mp2 (plain pitchwise mean at the MP)
//   scatter  each node gathers its <= 8 cell changes in the order the
//            reference's scatter loop adds them, so no atomics are needed
//   smooth   streamwise 2nd+4th order smoothing (gather, J+-2), then one
//            CTA per J-plane in shared memory: pitchwise and spanwise
//            smoothing, corners, exit smoothing, periodic, tip-gap and
//            mixing-plane averaging of D.
#include "mgpu_internal.cuh"

namespace mgpu {

static inline unsigned grid_for(size_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

// ---------------------------------------------------------------------
// tip-gap flux balance (5503-5510) and mixing-plane extrapolation of the
// upstream fluxes into SOURCE (5516-5555)
// ---------------------------------------------------------------------
__global__ void k_ts_prep(Dev d) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int ntip = (d.JM - 1) * d.KMM1;
    if (t < ntip) {
        int j = t / d.KMM1 + 2, k = t % d.KMM1 + 1;
        int nr = A1(d.NROW, j);
        int ks = A1(d.KTIPS, nr);
        if (ks > 0 && k >= ks && k <= A1(d.KTIPE, nr) - 1) {
            float a = 0.5f * (A3(d.TFLUX, 1, j, k) + A3(d.TFLUX, d.IM, j, k));
            A3(d.TFLUX, 1, j, k) = a;
            A3(d.TFLUX, d.IM, j, k) = a;
        }
        return;
    }
    t -= ntip;
    if (t >= d.NRWSM1 * d.KMM1) return;
    if (d.FEXTRAP < 0.001f) return;
    int nr = t / d.KMM1 + 1, k = t % d.KMM1 + 1;
    int j = A1(d.JMIX, nr), jp1 = j + 1, jm1 = j - 1, jp2 = j + 2;
    float FLOWDIRN = -A3(d.FLOWX, d.IMID, j, k);
    float AVFLXJM1 = 0.0f, AVFLXJP2 = 0.0f;
    for (int i = 1; i <= d.IMM1; ++i) {
        AVFLXJM1 = AVFLXJM1 + A3(d.XFLUX, i, jm1, k);
        AVFLXJP2 = AVFLXJP2 + A3(d.XFLUX, i, jp2, k);
    }
    for (int i = 1; i <= d.IMM1; ++i) {
        if (FLOWDIRN > 0.0f) {
            float DFLUX = (A3(d.XFLUX, i, jm1, k) - AVFLXJM1 * A1(d.FP, i)) * d.FEXTRAP;
            A3(d.SOURCE, i, j, k) = A3(d.SOURCE, i, j, k) - DFLUX;
        } else {
            float DFLUX = (A3(d.XFLUX, i, jp2, k) - AVFLXJP2 * A1(d.FP, i)) * d.FEXTRAP;
            A3(d.SOURCE, i, jp2, k) = A3(d.SOURCE, i, jp2, k) + DFLUX;
        }
        A3(d.SOURCE, i, jp1, k) = 0.0f;
    }
}

// flux sum and SCREE/SSS update (1000)
__global__ void k_ts_delta(Dev d, float *__restrict__ DIFF) {
    size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t N = (size_t)d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, n, i, j, k);
    if (i >= d.IM || j < 2 || k >= d.KM) return;
    float RATPITCH = (float)A1(d.NBLADE, j - 1) / (float)A1(d.NBLADE, j);
    float DELTA = d.XFLUX[n] - A3(d.XFLUX, i, j - 1, k) * RATPITCH + d.RFLUX[n] - A3(d.RFLUX, i, j, k + 1) + d.TFLUX[n] -
                  A3(d.TFLUX, i + 1, j, k) - d.SOURCE[n];
    float df = DIFF[n];
    d.STORE[n] = d.F1 * DELTA + d.F2 * df;
    DIFF[n] = DELTA + d.F3 * df;
}

// pitchwise redistribution of the change at the mixing planes (1750);
// plain=1 gives the second, plain-mean averaging after the multigrid (1850)
__global__ void k_ts_mp(Dev d, int plain) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.NRWSM1 * d.KMM1) return;
    int nr = t / d.KMM1 + 1, k = t % d.KMM1 + 1;
    int j = A1(d.JMIX, nr);
    float FLOWDIRN = -A3(d.FLOWX, d.IMID, j, k);
    bool lowx = d.FEXTRAP < 0.001f;
    for (int pass = 0; pass < 2; ++pass) {
        bool on = pass == 0 ? (FLOWDIRN > 0.0f || lowx) : (FLOWDIRN < 0.0f || lowx);
        if (!on) continue;
        int jj = pass == 0 ? j + 2 : j;
        float SUM_STORE = 0.0f;
        for (int i = 1; i <= d.IMM1; ++i) SUM_STORE = SUM_STORE + A3(d.STORE, i, jj, k);
        if (plain) {
            SUM_STORE = SUM_STORE / (float)d.IMM1;
            for (int i = 1; i <= d.IMM1; ++i) A3(d.STORE, i, jj, k) = SUM_STORE;
        } else {
            for (int i = 1; i <= d.IMM1; ++i) A3(d.STORE, i, jj, k) = SUM_STORE * A1(d.FP, i);
        }
    }
}

// multigrid restriction (700): level-1 and level-2 block sums.  Each thread
// owns one block and adds its cells in the reference's (K,J,I) loop order.
__global__ void k_ts_restrict(Dev d) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int n1 = d.NIB1 * (d.NJB1 + 1) * d.NKB1;
    int n2 = d.NIB2 * (d.NJB2 + 1) * d.NKB2;
    const int *JS, *JE, *IS, *IE, *KS, *KE;
    int nib, njb;
    float *out;
    if (t < n1) {
        nib = d.NIB1; njb = d.NJB1;
        JS = d.JB1_START; JE = d.JB1_END; IS = d.IB1_S; IE = d.IB1_E; KS = d.KB1_S; KE = d.KB1_E;
        out = d.B1CHG;
    } else if (t < n1 + n2) {
        t -= n1;
        nib = d.NIB2; njb = d.NJB2;
        JS = d.JB2_START; JE = d.JB2_END; IS = d.IB2_S; IE = d.IB2_E; KS = d.KB2_S; KE = d.KB2_E;
        out = d.B2CHG;
    } else {
        return;
    }
    int ib = t % nib + 1;
    int jb = (t / nib) % (njb + 1) + 1;
    int kb = t / (nib * (njb + 1)) + 1;
    float s = 0.0f;
    if (jb <= njb) {
        int j0 = JS[jb - 1], j1 = JE[jb - 1];
        int i0 = IS[ib - 1], i1 = IE[ib - 1];
        int k0 = KS[kb - 1], k1 = KE[kb - 1];
        for (int k = k0; k <= k1; ++k)
            for (int j = j0; j <= j1; ++j)
                for (int i = i0; i <= i1; ++i) s = s + A3(d.STORE, i, j, k);
    }
    out[t] = s;
}

// per-J-plane sums of STORE (abs=0) or |STORE| (abs=1) in FP64
template <int BS>
__device__ inline double block_sum(double v) {
    __shared__ double sh[BS / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = l < BS / 32 ? sh[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    return r;
}

constexpr int PLANE_BS = 256;

__global__ void __launch_bounds__(PLANE_BS) k_ts_plane_sum(Dev d, int absval, double *out) {
    int j = blockIdx.x + 2;
    int ncell = d.IMM1 * d.KMM1;
    double s = 0.0;
    for (int c = threadIdx.x; c < ncell; c += PLANE_BS) {
        int i = c % d.IMM1 + 1, k = c / d.IMM1 + 1;
        float v = A3(d.STORE, i, j, k);
        s += absval ? (double)fabsf(v) : (double)v;
    }
    s = block_sum<PLANE_BS>(s);
    if (threadIdx.x == 0) out[j - 1] = s;
}

// prolongation and time step (1500); with the negative feedback on and no
// residual smoothing the per-plane sum of |STORE| is formed here too
__global__ void __launch_bounds__(PLANE_BS) k_ts_prolong(Dev d, int want_abs) {
    int j = blockIdx.x + 2;
    __shared__ float s_sb;
    if (threadIdx.x < 32) {
        int sb = A1(d.JSBLK, j);
        int a = A1(d.SB_START, sb), b = A1(d.SB_END, sb);
        double s = 0.0;
        for (int jj = a + (int)threadIdx.x; jj <= b; jj += 32) s += d.plane_sum[jj - 1];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) s_sb = (float)s;
    }
    __syncthreads();
    float SBCHG = s_sb;
    int jsb = A1(d.JSBLK, j);
    float SSB = A1(d.STEPSBK, jsb);
    int j1 = A1(d.JB1, j), j2 = A1(d.JB2, j);
    int ncell = d.IMM1 * d.KMM1;
    double sabs = 0.0;
    for (int c = threadIdx.x; c < ncell; c += PLANE_BS) {
        int i = c % d.IMM1 + 1, k = c / d.IMM1 + 1;
        int i1 = A1(d.IB1, i), i2 = A1(d.IB2, i), k1 = A1(d.KB1, k), k2 = A1(d.KB2, k);
        size_t b1 = (size_t)(i1 - 1) + (size_t)d.NIB1 * ((size_t)(j1 - 1) + (size_t)(d.NJB1 + 1) * (k1 - 1));
        size_t b2 = (size_t)(i2 - 1) + (size_t)d.NIB2 * ((size_t)(j2 - 1) + (size_t)(d.NJB2 + 1) * (k2 - 1));
        size_t n = ix3(d, i, j, k);
        float DELTA = d.STORE[n] * d.STEP[n] +
                      (d.B1CHG[b1] * d.STEP1[b1] + d.B2CHG[b2] * d.STEP2[b2] + SBCHG * SSB) * d.RSTEP[n];
        d.STORE[n] = DELTA;
        sabs += (double)fabsf(DELTA);
    }
    if (want_abs) {
        sabs = block_sum<PLANE_BS>(sabs);
        if (threadIdx.x == 0) d.plane_abs[j - 1] = sabs;
    }
}

// per-row average change AVG_CHG and its smoothing AVG_BLK (1501-1515)
__global__ void k_ts_avgblk(Dev d) {
    __shared__ float chg[64];
    if (!d.ctl->damp_on) return;
    int NROWS = d.NROWS;
    for (int nr = threadIdx.x + 1; nr <= NROWS; nr += blockDim.x) {
        int JST = A1(d.JSTART, nr) + 1, JEN = A1(d.JMIX, nr) - 1;
        int JCHANGE = JEN - JST + 1;
        int NSUM = d.IMM1 * d.KMM1 * JCHANGE;
        double s = 0.0;
        for (int j = JST; j <= JEN; ++j) s += d.plane_abs[j - 1];
        chg[nr - 1] = (float)s / (float)NSUM;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float *B = d.AVG_BLK;
        if (NROWS == 1) B[0] = chg[0];
        if (NROWS == 2) {
            B[1] = 0.5f * (chg[0] + chg[1]);
            B[0] = B[1];
        }
        if (NROWS > 2) {
            for (int nr = 2; nr <= NROWS - 1; ++nr) B[nr - 1] = 0.25f * (chg[nr - 2] + chg[nr]) + 0.5f * chg[nr - 1];
            B[NROWS - 1] = 0.5f * (chg[NROWS - 2] + chg[NROWS - 1]);
            B[0] = 0.5f * (chg[0] + chg[1]);
        }
    }
}

// negative feedback (1525)
__global__ void k_ts_damp(Dev d) {
    size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t N = (size_t)d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, n, i, j, k);
    if (i >= d.IM || j < 2 || k >= d.KM) return;
    if (!d.ctl->damp_on) return;
    float DAMP = d.ctl->DAMP;
    int nr = A1(d.NROW, j);
    float DELTA = d.STORE[n];
    float ABSCHG = fabsf(DELTA);
    float FDAMP = ABSCHG / A1(d.AVG_BLK, nr);
    d.STORE[n] = DELTA / (1.0f + FDAMP / DAMP);
}

// corner distribution (1100) as a gather: node (I,J,K) adds, in the order
// the reference's cell loop reaches it, the weighted change of each of its
// <= 8 neighbouring cells
__global__ void k_ts_scatter(Dev d, float *__restrict__ D) {
    size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t N = (size_t)d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, n, i, j, k);
    float v = D[n];
    for (int kc = k - 1; kc <= k; ++kc) {
        if (kc < 1 || kc > d.KMM1) continue;
        for (int jc = j; jc <= j + 1; ++jc) {
            if (jc < 2 || jc > d.JM) continue;
            float fac = (jc == j) ? A1(d.FACDWN, jc) : A1(d.FACUP, jc);
            for (int ic = i - 1; ic <= i; ++ic) {
                if (ic < 1 || ic > d.IMM1) continue;
                float w;
                if (ic == i) w = (kc == k) ? AIK(d.FBL, ic, kc) : AIK(d.FTL, ic, kc);
                else w = (kc == k) ? AIK(d.FBR, ic, kc) : AIK(d.FTR, ic, kc);
                v = v + A3(d.STORE, ic, jc, kc) * w * fac;
            }
        }
    }
    D[n] = v;
}

// ---------------------------------------------------------------------
// SMOOTH_VAR: streamwise part (3900-4015) as a gather into TMP
// ---------------------------------------------------------------------
__global__ void k_sv_stream(Dev d, const float *__restrict__ D) {
    size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t N = (size_t)d.IM * d.JM * d.KM;
    const DevCtl *c = d.ctl;
    if (c->SFX < 0.0001f) return;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, n, i, j, k);
    int nr = A1(d.NROW, j);
    int J1 = A1(d.JSTART, nr), J2 = A1(d.JMIX, nr);
    float SFX = c->SFX, SFX1 = c->SFX1, SFXB = c->SFXB, SFXB1 = c->SFXB1, SFXBH = c->SFXBH;
#define DV(jj) A3(D, i, (jj), k)
    float v = D[n];
    if (j >= J1 + 3 && j <= J2 - 3) {
        float AVERG = 0.5f * (DV(j + 1) + DV(j - 1));
        float CURV = AVERG - 0.5f * v - 0.25f * (DV(j - 2) + DV(j + 2));
        v = SFX1 * v + SFX * (AVERG + d.FAC_4TH * CURV);
    }
    if (j == J2) v = D[n];
    if (j == J1) v = D[n];
    if (j == J1 + 2) v = SFXB1 * DV(J1 + 2) + SFXBH * (DV(J1 + 3) + DV(J1 + 1));
    if (j == J1 + 1) v = SFXB1 * DV(J1 + 1) + SFXB * (1.25f * DV(J1 + 2) + 0.5f * DV(J1 + 3) - 0.75f * DV(J1 + 4));
    if (j == J2 - 2) v = SFXB1 * DV(J2 - 2) + SFXBH * (DV(J2 - 1) + DV(J2 - 3));
    if (j == J2 - 1) v = SFXB1 * DV(J2 - 1) + SFXB * (1.25f * DV(J2 - 2) + 0.5f * DV(J2 - 3) - 0.75f * DV(J2 - 4));
#undef DV
    if (i == 1 || i == d.IM) {
        for (int r = 1; r <= d.NROWS; ++r) {
            int JL = A1(d.JLED, r);
            if (j == JL - 2 || j == JL - 1)
                v = c->SFXHM1 * D[n] + c->SFX14 * (A3(D, 2, j, k) + A3(D, d.IMM1, j, k));
            if (j == JL) {
                if (i == 1) v = c->SFXHM1 * D[n] + c->SFX14 * (A3(D, 1, j + 1, k) + A3(D, d.IM, j, k));
                else v = c->SFXHM1 * D[n] + c->SFX14 * (A3(D, d.IM, j + 1, k) + A3(D, 1, j, k));
            }
        }
    }
    d.TMP[n] = v;
}

// ---------------------------------------------------------------------
// SMOOTH_VAR pitchwise + spanwise + corners + exit smoothing (9000-8602),
// then TSTEP's periodic (8000), tip-gap (510) and mixing-plane (100)
// averaging of D: one CTA per J-plane, the plane held in shared memory.
// ---------------------------------------------------------------------
constexpr int SV_BS = 512;

__global__ void __launch_bounds__(SV_BS) k_sv_plane(Dev d, float *__restrict__ D) {
    extern __shared__ float sm[];
    const int IM = d.IM, KM = d.KM, IMM1 = d.IMM1, KMM1 = d.KMM1;
    const int np = IM * KM;
    float *a = sm, *b = sm + np;
    const int j = blockIdx.x + 1;
    const DevCtl *c = d.ctl;
    const float *src = (c->SFX < 0.0001f) ? D : d.TMP;
    for (int t = threadIdx.x; t < np; t += SV_BS) {
        int i = t % IM + 1, k = t / IM + 1;
        a[t] = A3(src, i, j, k);
    }
    __syncthreads();
#define P(buf, i, k) buf[((i) - 1) + IM * ((k) - 1)]
    const bool periodic_j = !(A1(d.IND, j) == 1 || A1(d.INDLE, j) == 1);
    if (j >= 2 && !(c->SFT < 0.0001f)) {
        const float SFT = c->SFT, SFT1 = c->SFT1, F4 = d.FAC_4TH;
        // pitchwise, Jacobi per K line: a -> b
        for (int t = threadIdx.x; t < np; t += SV_BS) {
            int i = t % IM + 1, k = t / IM + 1;
            auto curve = [&](int ii) -> float {   // CURVE(ii), ii in 1..IM
                if (ii == 1 || ii == IM) {
                    if (!periodic_j) return 0.0f;
                    float avg1 = 0.5f * (P(a, 2, k) + P(a, IMM1, k));
                    return P(a, 1, k) - avg1;
                }
                float avg = A1(d.FD, ii) * P(a, ii + 1, k) + A1(d.FU, ii) * P(a, ii - 1, k);
                return P(a, ii, k) - avg;
            };
            float AVG, SC;
            if (i == 1 || i == IM) {
                if (periodic_j) {
                    AVG = 0.5f * (P(a, 2, k) + P(a, IMM1, k));
                    SC = 0.5f * (curve(2) + curve(IMM1));
                } else {
                    if (i == 1) AVG = P(a, 2, k) + A1(d.FU, 1) * (P(a, 2, k) - P(a, 3, k));
                    else AVG = P(a, IMM1, k) + A1(d.FU, IM) * (P(a, IMM1, k) - P(a, d.IMM2, k));
                    SC = 0.0f;
                }
            } else {
                AVG = A1(d.FD, i) * P(a, i + 1, k) + A1(d.FU, i) * P(a, i - 1, k);
                SC = A1(d.FU, i) * curve(i - 1) + A1(d.FD, i) * curve(i + 1);
            }
            P(b, i, k) = SFT1 * P(a, i, k) + SFT * (AVG + F4 * SC);
        }
        __syncthreads();
        // spanwise, Jacobi per I line: b -> a
        for (int t = threadIdx.x; t < np; t += SV_BS) {
            int i = t % IM + 1, k = t / IM + 1;
            auto curvek = [&](int kk) -> float {
                if (kk == 1 || kk == KM) return 0.0f;
                float avg = A1(d.FKD, kk) * P(b, i, kk + 1) + A1(d.FKU, kk) * P(b, i, kk - 1);
                return P(b, i, kk) - avg;
            };
            float AVG, SC;
            if (k == 1) {
                AVG = P(b, i, 2) + 0.5f * A1(d.FKU, 1) * (P(b, i, 2) - P(b, i, 3));
                SC = 0.0f;
            } else if (k == KM) {
                AVG = P(b, i, KMM1) + 0.5f * A1(d.FKU, KM) * (P(b, i, KMM1) - P(b, i, d.KMM2));
                SC = 0.0f;
            } else {
                AVG = A1(d.FKD, k) * P(b, i, k + 1) + A1(d.FKU, k) * P(b, i, k - 1);
                SC = A1(d.FKU, k) * curvek(k - 1) + A1(d.FKD, k) * curvek(k + 1);
            }
            P(a, i, k) = SFT1 * P(b, i, k) + SFT * (AVG + F4 * SC);
        }
        __syncthreads();
        // the four corners read no corner, so they update together
        float cv = 0.0f;
        if (threadIdx.x < 4) {
            const float SFTH = c->SFTH;
            if (threadIdx.x == 0) cv = SFT1 * P(a, 1, 1) + SFTH * (P(a, 2, 1) + P(a, 1, 2));
            else if (threadIdx.x == 1) cv = SFT1 * P(a, IM, 1) + SFTH * (P(a, IMM1, 1) + P(a, IM, 2));
            else if (threadIdx.x == 2) cv = SFT1 * P(a, 1, KM) + SFTH * (P(a, 1, KMM1) + P(a, 2, KM));
            else cv = SFT1 * P(a, IM, KM) + SFTH * (P(a, IMM1, KM) + P(a, IM, KMM1));
        }
        __syncthreads();
        if (threadIdx.x == 0) P(a, 1, 1) = cv;
        else if (threadIdx.x == 1) P(a, IM, 1) = cv;
        else if (threadIdx.x == 2) P(a, 1, KM) = cv;
        else if (threadIdx.x == 3) P(a, IM, KM) = cv;
        __syncthreads();
    }
    // exit-flow smoothing (8502), Gauss-Seidel along I then along K
    if (!(d.SFEXIT < 0.0001f) && j >= d.JM + 1 - d.NSFEXIT) {
        const float SE = d.SFEXIT, SE1 = 1.0f - SE, SEH = 0.5f * SE;
        for (int k = threadIdx.x + 1; k <= KM; k += SV_BS) {
            for (int i = 2; i <= IMM1; ++i) P(a, i, k) = SE1 * P(a, i, k) + SEH * (P(a, i + 1, k) + P(a, i - 1, k));
            P(a, 1, k) = P(a, 1, k) + SE * (2.0f * P(a, 2, k) - P(a, 3, k) - P(a, 1, k));
            P(a, IM, k) = P(a, IM, k) + SE * (2.0f * P(a, IMM1, k) - P(a, d.IMM2, k) - P(a, IM, k));
        }
        __syncthreads();
        for (int i = threadIdx.x + 1; i <= IM; i += SV_BS) {
            for (int k = 2; k <= KMM1; ++k) P(a, i, k) = SE1 * P(a, i, k) + SEH * (P(a, i, k - 1) + P(a, i, k + 1));
            P(a, i, 1) = P(a, i, 1) + SE * (2.0f * P(a, i, 2) - P(a, i, 3) - P(a, i, 1));
            P(a, i, KM) = P(a, i, KM) + SE * (2.0f * P(a, i, KMM1) - P(a, i, d.KMM2) - P(a, i, KM));
        }
        __syncthreads();
    }
    // periodic boundaries and tip-gap periodicity
    int nr = A1(d.NROW, j);
    int K1 = A1(d.KTIPS, nr), K2 = A1(d.KTIPE, nr);
    bool tip = K1 > 0;
    if (tip) {
        if (K1 == 1) K2 = K2 - 1;
        if (K2 == KM) K1 = K1 + 1;
    }
    for (int k = threadIdx.x + 1; k <= KM; k += SV_BS) {
        if (periodic_j) {
            float v = 0.5f * (P(a, 1, k) + P(a, IM, k));
            P(a, 1, k) = v;
            P(a, IM, k) = v;
        }
        if (tip && k >= K1 && k <= K2) {
            float v = 0.5f * (P(a, 1, k) + P(a, IM, k));
            P(a, 1, k) = v;
            P(a, IM, k) = v;
        }
    }
    __syncthreads();
    // pitchwise average of D on both faces of each mixing plane
    bool mp = false;
    if (d.IFMIX != 0)
        for (int r = 1; r <= d.NRWSM1; ++r)
            if (j == A1(d.JMIX, r) || j == A1(d.JMIX, r) + 1) mp = true;
    if (mp) {
        for (int k = threadIdx.x + 1; k <= KM; k += SV_BS) {
            float s = 0.0f;
            for (int i = 1; i <= IMM1; ++i) s = s + A1(d.FP, i) * (P(a, i, k) + P(a, i + 1, k));
            b[k - 1] = 0.5f * s;
        }
        __syncthreads();
        for (int t = threadIdx.x; t < np; t += SV_BS) a[t] = b[t / IM];
        __syncthreads();
    }
#undef P
    for (int t = threadIdx.x; t < np; t += SV_BS) {
        int i = t % IM + 1, k = t / IM + 1;
        A3(D, i, j, k) = a[t];
    }
}

// ---------------------------------------------------------------------
// SMOOTH_RESID (14833-14917): one Jacobi pass along J, I or K of the cell
// changes inside each row, src -> dst (cells outside every row are copied)
// ---------------------------------------------------------------------
__global__ void k_resid_pass(Dev d, int dir, float smfac, const float *__restrict__ src, float *__restrict__ dst) {
    size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t N = (size_t)d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, n, i, j, k);
    if (i >= d.IM || j < 2 || k >= d.KM) return;
    float SFAC1 = 1.0f - smfac, SFACH = 0.5f * smfac;
    int nr = A1(d.NROW, j);
    int J1P1 = A1(d.JSTART, nr) + 1, J1P2 = J1P1 + 1, J2 = A1(d.JMIX, nr), J2M1 = J2 - 1;
    float v = src[n];
    if (j < J1P1 || j > J2) {
        dst[n] = v;
        return;
    }
#define S(ii, jj, kk) A3(src, ii, jj, kk)
    if (dir == 0) {
        if (j >= J1P2 && j <= J2M1) v = SFAC1 * v + SFACH * (S(i, j + 1, k) + S(i, j - 1, k));
        if (j == J1P1) v = S(i, J1P1, k) + SFACH * (S(i, J1P2, k) - S(i, J1P1, k));
        if (j == J2) v = S(i, J2, k) + SFACH * (S(i, J2M1, k) - S(i, J2, k));
    } else if (dir == 1) {
        int IMM1 = d.IMM1, IMM2 = d.IMM2;
        if (i >= 2 && i <= IMM2) v = SFAC1 * v + SFACH * (S(i + 1, j, k) + S(i - 1, j, k));
        if (i == 1) v = S(1, j, k) + SFACH * (S(2, j, k) - S(1, j, k));
        if (i == IMM1) v = S(IMM1, j, k) + SFACH * (S(IMM2, j, k) - S(IMM1, j, k));
    } else {
        int KMM1 = d.KMM1, KMM2 = d.KMM2;
        if (k >= 2 && k <= KMM2) v = SFAC1 * v + SFACH * (S(i, j, k + 1) + S(i, j, k - 1));
        if (k == 1) v = S(i, j, 1) + SFACH * (S(i, j, 2) - S(i, j, 1));
        if (k == KMM1) v = S(i, j, KMM1) + SFACH * (S(i, j, KMM2) - S(i, j, KMM1));
    }
#undef S
    dst[n] = v;
}

__global__ void k_copy(const float *__restrict__ src, float *__restrict__ dst, size_t n) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = src[t];
}

cudaError_t configure_kernels(const Dev &d) {
    int smem = 2 * d.IM * d.KM * (int)sizeof(float);
    return cudaFuncSetAttribute(k_sv_plane, cudaFuncAttributeMaxDynamicSharedMemorySize, smem > 48 * 1024 ? smem : 48 * 1024);
}

void launch_tstep(const Dev &d, Launch L, float *D, float *DIFF) {
    size_t N = (size_t)d.IM * d.JM * d.KM;
    unsigned gN = grid_for(N, 256);
    int nprep = (d.JM - 1) * d.KMM1 + d.NRWSM1 * d.KMM1;
    k_ts_prep<<<grid_for(nprep, 128), 128, 0, L.s>>>(d);
    k_ts_delta<<<gN, 256, 0, L.s>>>(d, DIFF);
    if (d.NRWSM1 > 0) k_ts_mp<<<grid_for(d.NRWSM1 * d.KMM1, 64), 64, 0, L.s>>>(d, 0);
    bool mg = !(d.IR <= 1 && d.JR <= 1 && d.KR <= 1);
    if (mg) {
        int nb = d.NIB1 * (d.NJB1 + 1) * d.NKB1 + d.NIB2 * (d.NJB2 + 1) * d.NKB2;
        k_ts_restrict<<<grid_for(nb, 64), 64, 0, L.s>>>(d);
        k_ts_plane_sum<<<d.JM - 1, PLANE_BS, 0, L.s>>>(d, 0, d.plane_sum);
    }
    k_ts_prolong<<<d.JM - 1, PLANE_BS, 0, L.s>>>(d, d.NRSMTH == 0 ? 1 : 0);
    if (d.NRSMTH > 0) {
        for (int it = 0; it < d.NRSMTH; ++it) {
            k_resid_pass<<<gN, 256, 0, L.s>>>(d, 0, d.RSMTH, d.STORE, d.TMP);
            k_resid_pass<<<gN, 256, 0, L.s>>>(d, 1, d.RSMTH, d.TMP, d.STORE);
            k_resid_pass<<<gN, 256, 0, L.s>>>(d, 2, d.RSMTH, d.STORE, d.TMP);
            k_copy<<<gN, 256, 0, L.s>>>(d.TMP, d.STORE, N);
        }
        k_ts_plane_sum<<<d.JM - 1, PLANE_BS, 0, L.s>>>(d, 1, d.plane_abs);
    }
    k_ts_avgblk<<<1, 32, 0, L.s>>>(d);
    k_ts_damp<<<gN, 256, 0, L.s>>>(d);
    if (d.NRWSM1 > 0) k_ts_mp<<<grid_for(d.NRWSM1 * d.KMM1, 64), 64, 0, L.s>>>(d, 1);
    k_ts_scatter<<<gN, 256, 0, L.s>>>(d, D);
    k_sv_stream<<<gN, 256, 0, L.s>>>(d, D);
    size_t smem = (size_t)2 * d.IM * d.KM * sizeof(float);
    k_sv_plane<<<d.JM, SV_BS, smem, L.s>>>(d, D);
}

}  // namespace mgpu
