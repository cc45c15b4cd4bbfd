// mgpu_tstep.cu -- SUBROUTINE TSTEP (multall-open-18.3.f:5470-5932) with
// SMOOTH_VAR (15352-15594) and SMOOTH_RESID (14833-14917) on the GPU.
//
// One call updates one conserved variable D with its SCREE history DIFF in
// four kernels, each with one CTA per J-plane (a J-plane of the largest
// configuration, 73 x 57 points, is 16 KB: it lives in shared memory):
//   cells    tip-gap TFLUX balance, mixing-plane flux extrapolation into
//            SOURCE, the flux sum DELTA -> STORE and DIFF, the pitchwise
//            redistribution of STORE on the mixing-plane cells, and this
//            plane's partial sums for the three multigrid levels
//   prolong  block sums assembled from the plane partials (level-1 blocks
//            span <= JR planes, level-2 <= JRBB, superblocks a row part);
//            STORE*STEP + corrections*RSTEP; per-plane sum of |STORE|
//   update   per-row mean |STORE| (negative feedback, 1501-1525) applied to
//            the cell planes J and J+1, the second mixing-plane average
//            (1850), then every node of plane J gathers its <= 8 cell
//            changes in the order the reference's scatter loop adds them
//            (1100) -- no atomics, result written to TMP
//   smooth   streamwise smoothing of plane J from TMP planes J-2..J+2, then
//            pitchwise, spanwise, corners, exit smoothing, periodic,
//            tip-gap and mixing-plane averaging in shared memory -> D
// With REDUCE_ORDER=1 the level sums and the row mean are instead formed by
// single threads in the reference's sequential REAL*4 order (parity checks);
// with REDUCE_ORDER=2 (the plain FP32 path) they are the default path's
// trees with FP32 adds.
#include "mgpu_internal.cuh"

namespace mgpu {

static inline unsigned grid_for(size_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

// Threads per J-plane CTA: 128, 192, 256 (the default) or 512, chosen per
// problem and pass by mgpu_autotune (Dev::ts_bs); each size keeps 1024
// threads of 64 registers resident per SM (960 for 192: five CTAs).  A pass
// of 3 x 241 CTAs fills five 192-thread slots per SM in one wave, where four
// 256-thread slots take 1.2 waves.
constexpr int TS_U = 3;          // cells per thread whose loads are issued together
constexpr int TS_UG = 4;         // the same for the damping and gather phases of update
constexpr int SV_U = 3;          // points per thread whose streamwise loads are issued together
constexpr int SM_SEG = 8;        // points per thread of one pitchwise or spanwise smoothing segment
constexpr int UG_SEG = 3;        // nodes per thread of one K column in the pair update's gather

// CTA sum of one double-float per thread (thread 0 receives it)
template <int BS>
__device__ inline df block_sum(int order, df v, df *sh) {
    for (int o = 16; o > 0; o >>= 1) v = dacc(order, v, df_shfl_down(v, o));
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    df r = df_of(0.0f);
    if (w == 0) {
        r = l < BS / 32 ? sh[l] : df_of(0.0f);
        for (int o = 16; o > 0; o >>= 1) r = dacc(order, r, df_shfl_down(r, o));
    }
    __syncthreads();
    return r;
}

// position of plane j relative to the mixing planes: 1 = JMIX, 2 = JMIX+1,
// 3 = JMIX+2 (0 otherwise); *nr receives the row interface
__device__ inline int mp_role(const Dev &d, int j, int *nr) {
    for (int r = 1; r <= d.NRWSM1; ++r) {
        int jx = A1(d.JMIX, r);
        if (j == jx) { *nr = r; return 1; }
        if (j == jx + 1) { *nr = r; return 2; }
        if (j == jx + 2) { *nr = r; return 3; }
    }
    *nr = 0;
    return 0;
}

// Pitchwise sum of a mixing-plane line in I order, REAL*4 as the reference
// forms it (REDUCE_ORDER 1, and the plain FP32 path, 2).
__device__ inline float mp_line_sum(const float *row, int n) {
    float s = 0.0f;
    for (int i = 0; i < n; ++i) s = s + row[i];
    return s;
}

// The default precision split's form of the same sum: accumulated in
// double-float and rounded once, by one warp (every lane calls it, with the
// same n).  Each lane adds every 32nd term, then a shuffle tree; every lane
// gets the total.
template <class F>
__device__ inline float warp_sum64(int n, F term) {
    df s = df_of(0.0f);
    for (int i = (int)(threadIdx.x & 31); i < n; i += 32) s = df_add(s, df_of(term(i)));
    for (int o = 16; o > 0; o >>= 1) s = df_add(s, df_shfl_xor(s, o));
    return df_val(s);
}

// (i, k) of the points t = start, start + stride, ... of an ni-wide plane,
// 1-based, advanced without a division per point
struct Walk2 {
    int i, k, di, dk, ni;
    __device__ Walk2(int ni_, int start, int stride) : ni(ni_) {
        i = start % ni_ + 1;
        k = start / ni_ + 1;
        di = stride % ni_;
        dk = stride / ni_;
    }
    __device__ void next() {
        i += di;
        k += dk;
        if (i > ni) {
            i -= ni;
            ++k;
        }
    }
};

// ---------------------------------------------------------------------
// cells: 5503-5510 (tip gap), 5516-5555 (MP extrapolation), 1000 (flux
// sum), 1750 (MP redistribution) and the multigrid partial sums
// ---------------------------------------------------------------------
template <int BS>
__global__ void __launch_bounds__(BS, 1024 / BS) k_ts_cells(const __grid_constant__ Dev d, int v0) {
    pdl_wait();
    extern __shared__ float sm[];
    const VarSet &V = d.var[v0 + blockIdx.y];
    float *__restrict__ DIFF = V.DIFF;
    __shared__ df shd[BS / 32];
    const int j = blockIdx.x + 2;
    const int IM = d.IM, IMM1 = d.IMM1, KMM1 = d.KMM1;
    const int nc = IMM1 * KMM1;
    float *st = sm;              // STORE of this plane, [k-1][i-1]
    float *lsum = sm + nc;       // per-K line sums
    int mnr;
    const int role = mp_role(d, j, &mnr);
    const bool lowx = d.FEXTRAP < 0.001f;
    const int jmx = role ? A1(d.JMIX, mnr) : 0;
    if ((role == 1 || role == 3) && !lowx) {
        // stage the XFLUX plane in shared memory (coalesced), then add each
        // I-line in the reference's order
        int jj = role == 1 ? j - 1 : j;
        Walk2 wx(IMM1, threadIdx.x, BS);
        for (int c = threadIdx.x; c < nc; c += BS, wx.next()) st[c] = A3(V.XF, wx.i, jj, wx.k);
        __syncthreads();
        if (d.REDUCE_ORDER != 0) {
            for (int k = threadIdx.x + 1; k <= KMM1; k += BS) {
                const float *row = st + (size_t)(k - 1) * IMM1;
                lsum[k - 1] = mp_line_sum(row, IMM1);
            }
        } else {
            for (int k = (int)(threadIdx.x >> 5) + 1; k <= KMM1; k += BS / 32) {
                const float *row = st + (size_t)(k - 1) * IMM1;
                float s = warp_sum64(IMM1, [&](int i) { return row[i]; });
                if ((threadIdx.x & 31) == 0) lsum[k - 1] = s;
            }
        }
    }
    __syncthreads();
    const float RATPITCH = (float)A1(d.NBLADE, j - 1) / (float)A1(d.NBLADE, j);
    const int nr = A1(d.NROW, j);
    const int kts = A1(d.KTIPS, nr), kte = A1(d.KTIPE, nr);
    const float F1 = d.F1, F2 = d.F2, F3 = d.F3;
    const float *__restrict__ XF = V.XF;
    const float *__restrict__ RF = V.RF;
    const float *__restrict__ TF = V.TF;
    const float *__restrict__ SR = V.SR;
    // each thread first loads the operands of its TS_U cells, then computes:
    // the loads of all cells are in flight together.  Offsets are 32-bit
    // (a node array holds fewer than 2^31 points: commit limits IM, KM and JM)
    const int ks = IM * d.JM, pj = IM * (j - 1);
    Walk2 w(IMM1, threadIdx.x, BS);
    for (int c0 = threadIdx.x; c0 < nc; c0 += TS_U * BS) {
        float xf[TS_U], xm[TS_U], rf[TS_U], rk[TS_U], ta[TS_U], tb1[TS_U], sr[TS_U], df[TS_U];
        int ci[TS_U], ck[TS_U];
#pragma unroll
        for (int u = 0; u < TS_U; ++u) {
            ci[u] = w.i;
            ck[u] = w.k;
            w.next();
            if (c0 + u * BS < nc) {
                const int n = pj + (ci[u] - 1) + ks * (ck[u] - 1);
                xf[u] = XF[n];
                xm[u] = XF[n - IM];
                rf[u] = RF[n];
                rk[u] = RF[n + ks];
                ta[u] = TF[n];
                tb1[u] = TF[n + 1];
                sr[u] = SR[n];
                df[u] = DIFF[n];
            }
        }
#pragma unroll
        for (int u = 0; u < TS_U; ++u) {
            const int c = c0 + u * BS;
            if (c >= nc) break;
            const int i = ci[u], k = ck[u];
            const int n = pj + (i - 1) + ks * (k - 1);
            float t0 = ta[u], t1 = tb1[u];
            if (kts > 0 && k >= kts && k <= kte - 1) {
                if (i == 1 || i + 1 == IM) {
                    float tb = 0.5f * (A3(TF, 1, j, k) + A3(TF, IM, j, k));
                    if (i == 1) t0 = tb;
                    if (i + 1 == IM) t1 = tb;
                }
            }
            float src = sr[u];
            if (role && !lowx) {
                float FLOWDIRN = -A3(d.FLOWX, d.IMID, jmx, k);
                if (role == 1 && FLOWDIRN > 0.0f) src = src - (xm[u] - lsum[k - 1] * A1(d.FP, i)) * d.FEXTRAP;
                if (role == 2) src = 0.0f;
                if (role == 3 && !(FLOWDIRN > 0.0f)) src = src + (xf[u] - lsum[k - 1] * A1(d.FP, i)) * d.FEXTRAP;
            }
            float DELTA = xf[u] - xm[u] * RATPITCH + rf[u] - rk[u] + t0 - t1 - src;
            st[c] = F1 * DELTA + F2 * df[u];
            DIFF[n] = DELTA + F3 * df[u];
        }
    }
    __syncthreads();
    if (role == 1 || role == 3) {
        const bool lane_par = d.REDUCE_ORDER == 0;
        const int k0 = lane_par ? (int)(threadIdx.x >> 5) + 1 : (int)threadIdx.x + 1;
        const int kstep = lane_par ? BS / 32 : BS;
        for (int k = k0; k <= KMM1; k += kstep) {
            float FLOWDIRN = -A3(d.FLOWX, d.IMID, jmx, k);
            bool on = role == 3 ? (FLOWDIRN > 0.0f || lowx) : (FLOWDIRN < 0.0f || lowx);
            if (!on) continue;
            float *row = st + (size_t)(k - 1) * IMM1;
            if (lane_par) {
                float s = warp_sum64(IMM1, [&](int i) { return row[i]; });
                __syncwarp();
                for (int i = (int)(threadIdx.x & 31); i < IMM1; i += 32) row[i] = s * A1(d.FP, i + 1);
            } else {
                float s = mp_line_sum(row, IMM1);
                for (int i = 0; i < IMM1; ++i) row[i] = s * A1(d.FP, i + 1);
            }
        }
        __syncthreads();
    }
    // plane sum: a thread's dozen cells in FP32, the threads' partials in
    // double-float
    float psf = 0.0f;
    {
        float *__restrict__ STj = V.ST + pj;
        Walk2 wp(IMM1, threadIdx.x, BS);
        for (int c = threadIdx.x; c < nc; c += BS, wp.next()) {
            float v = st[c];
            STj[(wp.i - 1) + ks * (wp.k - 1)] = v;
            psf += v;
        }
    }
    const df ps = block_sum<BS>(d.REDUCE_ORDER, df_of(psf), shd);
    if (threadIdx.x == 0) V.psum[j - 1] = ps;
    // level-1 and level-2 partial sums of this plane
    const int n1 = d.NIB1 * d.NKB1, n2 = d.NIB2 * d.NKB2;
    if (d.mg_nested) {
        // every level-2 block is a union of level-1 blocks: the level-1
        // partials first (in shared memory), then each level-2 partial as the
        // sum of its level-1 partials (a 9-term chain for 3 x 3 blocks of
        // 3 x 3 cells, where the direct sum is an 81-term chain)
        float *p1 = lsum + KMM1;
        for (int u = threadIdx.x; u < n1; u += BS) {
            const int ib = u % d.NIB1 + 1, kb = u / d.NIB1 + 1;
            const int i0 = A1(d.IB1_S, ib), i1 = A1(d.IB1_E, ib), k0 = A1(d.KB1_S, kb), k1 = A1(d.KB1_E, kb);
            float s = 0.0f;
            for (int k = k0; k <= k1; ++k)
                for (int i = i0; i <= i1; ++i) s = s + st[(k - 1) * IMM1 + (i - 1)];
            p1[u] = s;
            V.P1[(size_t)(j - 1) * n1 + u] = s;
        }
        __syncthreads();
        for (int u = threadIdx.x; u < n2; u += BS) {
            const int ib = u % d.NIB2 + 1, kb = u / d.NIB2 + 1;
            const int a0 = A1(d.IB1, A1(d.IB2_S, ib)), a1 = A1(d.IB1, A1(d.IB2_E, ib));
            const int c0 = A1(d.KB1, A1(d.KB2_S, kb)), c1 = A1(d.KB1, A1(d.KB2_E, kb));
            float s = 0.0f;
            for (int kb1 = c0; kb1 <= c1; ++kb1)
                for (int ib1 = a0; ib1 <= a1; ++ib1) s = s + p1[(kb1 - 1) * d.NIB1 + (ib1 - 1)];
            V.P2[(size_t)(j - 1) * n2 + u] = s;
        }
        return;
    }
    for (int t = threadIdx.x; t < n1 + n2; t += BS) {
        const bool lv1 = t < n1;
        int u = lv1 ? t : t - n1;
        int nib = lv1 ? d.NIB1 : d.NIB2;
        int ib = u % nib + 1, kb = u / nib + 1;
        int i0 = lv1 ? A1(d.IB1_S, ib) : A1(d.IB2_S, ib), i1 = lv1 ? A1(d.IB1_E, ib) : A1(d.IB2_E, ib);
        int k0 = lv1 ? A1(d.KB1_S, kb) : A1(d.KB2_S, kb), k1 = lv1 ? A1(d.KB1_E, kb) : A1(d.KB2_E, kb);
        float s = 0.0f;
        for (int k = k0; k <= k1; ++k)
            for (int i = i0; i <= i1; ++i) s = s + st[(k - 1) * IMM1 + (i - 1)];
        if (lv1) V.P1[(size_t)(j - 1) * n1 + u] = s;
        else V.P2[(size_t)(j - 1) * n2 + u] = s;
    }
}

// ---------------------------------------------------------------------
// reference-order level sums (REDUCE_ORDER=1): one thread per block walks
// its cells in the (K,J,I) loop order of 700; superblocks likewise
// ---------------------------------------------------------------------
__global__ void k_ts_restrict_seq(const __grid_constant__ Dev d, int v0) {
    pdl_wait();
    const VarSet &V = d.var[v0 + blockIdx.y];
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int n1 = d.NIB1 * (d.NJB1 + 1) * d.NKB1;
    int n2 = d.NIB2 * (d.NJB2 + 1) * d.NKB2;
    if (t >= n1 + n2 + d.NSBLK) return;
    if (t >= n1 + n2) {
        int sb = t - n1 - n2 + 1;
        int a = A1(d.SB_START, sb), b = A1(d.SB_END, sb);
        float s = 0.0f;
        for (int k = 1; k <= d.KMM1; ++k)
            for (int j = a; j <= b; ++j)
                for (int i = 1; i <= d.IMM1; ++i) s = s + A3(V.ST, i, j, k);
        A1(V.SBSUM, sb) = s;
        return;
    }
    const bool lv1 = t < n1;
    int u = lv1 ? t : t - n1;
    int nib = lv1 ? d.NIB1 : d.NIB2, njb = lv1 ? d.NJB1 : d.NJB2;
    int ib = u % nib + 1;
    int jb = (u / nib) % (njb + 1) + 1;
    int kb = u / (nib * (njb + 1)) + 1;
    float s = 0.0f;
    if (jb <= njb) {
        int j0 = lv1 ? A1(d.JB1_START, jb) : A1(d.JB2_START, jb), j1 = lv1 ? A1(d.JB1_END, jb) : A1(d.JB2_END, jb);
        int i0 = lv1 ? A1(d.IB1_S, ib) : A1(d.IB2_S, ib), i1 = lv1 ? A1(d.IB1_E, ib) : A1(d.IB2_E, ib);
        int k0 = lv1 ? A1(d.KB1_S, kb) : A1(d.KB2_S, kb), k1 = lv1 ? A1(d.KB1_E, kb) : A1(d.KB2_E, kb);
        for (int k = k0; k <= k1; ++k)
            for (int j = j0; j <= j1; ++j)
                for (int i = i0; i <= i1; ++i) s = s + A3(V.ST, i, j, k);
    }
    (lv1 ? V.B1CHG : V.B2CHG)[u] = s;
}

// Sum over the J planes a..e of one block's per-plane partial sums, added in
// J order in REAL*4; the loads of three planes (a level-1 block, a third of a
// level-2 block) are issued before their adds.
__device__ __forceinline__ float plane_partials_sum(const float *__restrict__ P, int n, int t, int a, int e) {
    float s = 0.0f;
    int jj = a;
    for (; jj + 2 <= e; jj += 3) {
        const float x0 = P[(size_t)(jj - 1) * n + t], x1 = P[(size_t)jj * n + t], x2 = P[(size_t)(jj + 1) * n + t];
        s = s + x0;
        s = s + x1;
        s = s + x2;
    }
    for (; jj <= e; ++jj) s = s + P[(size_t)(jj - 1) * n + t];
    return s;
}

// ---------------------------------------------------------------------
// prolong: 1500, with the block sums assembled from the plane partials
// ---------------------------------------------------------------------
template <int BS>
__global__ void __launch_bounds__(BS, 1024 / BS) k_ts_prolong(const __grid_constant__ Dev d, int v0, int want_abs) {
    pdl_wait();
    extern __shared__ float sm[];
    const VarSet &V = d.var[v0 + blockIdx.y];
    __shared__ df shd[BS / 32];
    __shared__ float s_sb;
    const int j = blockIdx.x + 2;
    const int IMM1 = d.IMM1, KMM1 = d.KMM1;
    const int n1 = d.NIB1 * d.NKB1, n2 = d.NIB2 * d.NKB2;
    float *b1 = sm, *b2 = sm + n1;
    const int j1 = A1(d.JB1, j), j2 = A1(d.JB2, j), jsb = A1(d.JSBLK, j);
    const int nc = IMM1 * KMM1;
    const int ks = d.IM * d.JM, pj = d.IM * (j - 1);
    const int m1 = d.NIB1 * (d.NJB1 + 1), m2 = d.NIB2 * (d.NJB2 + 1);
    // operands of this thread's first TS_U cells, loaded before the block
    // sums so their latency overlaps the assembly below
    float pst[TS_U], pstp[TS_U], prs[TS_U], ps1[TS_U], ps2[TS_U];
    int pb1[TS_U], pb2[TS_U];
    Walk2 w(IMM1, threadIdx.x, BS);
#pragma unroll
    for (int u = 0; u < TS_U; ++u) {
        const int i = w.i, k = w.k;
        w.next();
        if (threadIdx.x + u * BS < nc) {
            const int n = pj + (i - 1) + ks * (k - 1);
            const int i1 = A1(d.IB1, i), i2 = A1(d.IB2, i), k1 = A1(d.KB1, k), k2 = A1(d.KB2, k);
            pst[u] = V.ST[n];
            pstp[u] = d.STEP[n];
            prs[u] = d.RSTEP[n];
            ps1[u] = d.STEP1[(i1 - 1) + d.NIB1 * (j1 - 1) + m1 * (k1 - 1)];
            ps2[u] = d.STEP2[(i2 - 1) + d.NIB2 * (j2 - 1) + m2 * (k2 - 1)];
            pb1[u] = (k1 - 1) * d.NIB1 + (i1 - 1);
            pb2[u] = (k2 - 1) * d.NIB2 + (i2 - 1);
        }
    }
    if (d.REDUCE_ORDER == 1) {
        for (int t = threadIdx.x; t < n1; t += BS) {
            int ib = t % d.NIB1 + 1, kb = t / d.NIB1 + 1;
            b1[t] = V.B1CHG[(ib - 1) + d.NIB1 * (j1 - 1) + m1 * (kb - 1)];
        }
        for (int t = threadIdx.x; t < n2; t += BS) {
            int ib = t % d.NIB2 + 1, kb = t / d.NIB2 + 1;
            b2[t] = V.B2CHG[(ib - 1) + d.NIB2 * (j2 - 1) + m2 * (kb - 1)];
        }
        if (threadIdx.x == 0) s_sb = A1(V.SBSUM, jsb);
    } else {
        // the J planes of this plane's level-1 and level-2 blocks (empty past
        // the last block); each sum adds the planes' partials in J order
        const int a1 = j1 <= d.NJB1 ? A1(d.JB1_START, j1) : 1, e1 = j1 <= d.NJB1 ? A1(d.JB1_END, j1) : 0;
        const int a2 = j2 <= d.NJB2 ? A1(d.JB2_START, j2) : 1, e2 = j2 <= d.NJB2 ? A1(d.JB2_END, j2) : 0;
        for (int t = threadIdx.x; t < n1; t += BS) b1[t] = plane_partials_sum(V.P1, n1, t, a1, e1);
        for (int t = threadIdx.x; t < n2; t += BS) b2[t] = plane_partials_sum(V.P2, n2, t, a2, e2);
        if (threadIdx.x < 32) {
            int a = A1(d.SB_START, jsb), b = A1(d.SB_END, jsb);
            const int ro = d.REDUCE_ORDER;
            df s = df_of(0.0f);
            for (int jj = a + (int)threadIdx.x; jj <= b; jj += 32) s = dacc(ro, s, V.psum[jj - 1]);
            for (int o = 16; o > 0; o >>= 1) s = dacc(ro, s, df_shfl_down(s, o));
            if (threadIdx.x == 0) s_sb = df_val(s);
        }
    }
    if (d.IR <= 1 && d.JR <= 1 && d.KR <= 1) {
        // no multigrid: TSTEP skips the restriction (5613) and the block
        // changes keep the zeros they start from (5490-5498)
        for (int t = threadIdx.x; t < n1; t += BS) b1[t] = 0.0f;
        for (int t = threadIdx.x; t < n2; t += BS) b2[t] = 0.0f;
        if (threadIdx.x == 0) s_sb = 0.0f;
    }
    __syncthreads();
    const float SBCHG = s_sb, SSB = A1(d.STEPSBK, jsb);
    float sabs = 0.0f;            // FP32 per thread, double-float across threads (as in k_ts_cells)
    w = Walk2(IMM1, threadIdx.x, BS);
#pragma unroll
    for (int u = 0; u < TS_U; ++u) {
        const int i = w.i, k = w.k;
        w.next();
        if (threadIdx.x + u * BS < nc) {
            const int n = pj + (i - 1) + ks * (k - 1);
            float DELTA = pst[u] * pstp[u] + (b1[pb1[u]] * ps1[u] + b2[pb2[u]] * ps2[u] + SBCHG * SSB) * prs[u];
            V.ST[n] = DELTA;
            sabs += fabsf(DELTA);
        }
    }
    // the remaining cells, TS_U at a time: their loads are issued together,
    // before the stores of the group (a store of ST keeps later loads behind it)
    for (int c0 = threadIdx.x + TS_U * BS; c0 < nc; c0 += TS_U * BS) {
        int cn[TS_U];
#pragma unroll
        for (int u = 0; u < TS_U; ++u) {
            const int i = w.i, k = w.k;
            w.next();
            cn[u] = -1;
            if (c0 + u * BS < nc) {
                const int n = pj + (i - 1) + ks * (k - 1);
                const int i1 = A1(d.IB1, i), i2 = A1(d.IB2, i), k1 = A1(d.KB1, k), k2 = A1(d.KB2, k);
                cn[u] = n;
                pst[u] = V.ST[n];
                pstp[u] = d.STEP[n];
                prs[u] = d.RSTEP[n];
                ps1[u] = d.STEP1[(i1 - 1) + d.NIB1 * (j1 - 1) + m1 * (k1 - 1)];
                ps2[u] = d.STEP2[(i2 - 1) + d.NIB2 * (j2 - 1) + m2 * (k2 - 1)];
                pb1[u] = (k1 - 1) * d.NIB1 + (i1 - 1);
                pb2[u] = (k2 - 1) * d.NIB2 + (i2 - 1);
            }
        }
#pragma unroll
        for (int u = 0; u < TS_U; ++u) {
            if (cn[u] < 0) continue;
            float DELTA = pst[u] * pstp[u] + (b1[pb1[u]] * ps1[u] + b2[pb2[u]] * ps2[u] + SBCHG * SSB) * prs[u];
            V.ST[cn[u]] = DELTA;
            sabs += fabsf(DELTA);
        }
    }
    if (want_abs) {
        const df t = block_sum<BS>(d.REDUCE_ORDER, df_of(sabs), shd);
        if (threadIdx.x == 0) V.pabs[j - 1] = t;
    }
}

// per-J-plane sum of |STORE| (after residual smoothing)
template <int BS>
__global__ void __launch_bounds__(BS, 1024 / BS) k_ts_plane_abs(const __grid_constant__ Dev d, int v0) {
    pdl_wait();
    __shared__ df shd[BS / 32];
    const VarSet &V = d.var[v0 + blockIdx.y];
    int j = blockIdx.x + 2;
    int nc = d.IMM1 * d.KMM1;
    float sf = 0.0f;
    for (int c = threadIdx.x; c < nc; c += BS) {
        int i = c % d.IMM1 + 1, k = c / d.IMM1 + 1;
        sf += fabsf(A3(V.ST, i, j, k));
    }
    const df s = block_sum<BS>(d.REDUCE_ORDER, df_of(sf), shd);
    if (threadIdx.x == 0) V.pabs[j - 1] = s;
}

// AVG_CHG / AVG_BLK with the reference's sequential REAL*4 sum (1501-1515)
__global__ void k_ts_avgblk_seq(const __grid_constant__ Dev d, int v0) {
    pdl_wait();
    __shared__ float chg[64];
    const VarSet &V = d.var[v0 + blockIdx.y];
    if (!d.ctl->damp_on) return;
    int NROWS = d.NROWS;
    for (int nr = threadIdx.x + 1; nr <= NROWS; nr += blockDim.x) {
        int JST = A1(d.JSTART, nr) + 1, JEN = A1(d.JMIX, nr) - 1;
        int NSUM = d.IMM1 * d.KMM1 * (JEN - JST + 1);
        float SUMCHG = 0.0f;
        for (int k = 1; k <= d.KMM1; ++k)
            for (int j = JST; j <= JEN; ++j)
                for (int i = 1; i <= d.IMM1; ++i) SUMCHG = SUMCHG + fabsf(A3(V.ST, i, j, k));
        chg[nr - 1] = SUMCHG / (float)NSUM;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float *B = V.AVG_BLK;
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

// ---------------------------------------------------------------------
// update: negative feedback, second MP average, corner gather -> TMP
// ---------------------------------------------------------------------
template <int BS>
__global__ void __launch_bounds__(BS, 1024 / BS) k_ts_update(const __grid_constant__ Dev d, int v0) {
    pdl_wait();
    extern __shared__ float sm[];
    const VarSet &V = d.var[v0 + blockIdx.y];
    const float *__restrict__ D = V.D;
    __shared__ float s_blk[64];
    __shared__ float chg[64];
    const int j = blockIdx.x + 1;
    const int IM = d.IM, IMM1 = d.IMM1, KM = d.KM, KMM1 = d.KMM1;
    const int nc = IMM1 * KMM1;
    float *cA = sm, *cB = sm + nc;            // cell planes j and j+1
    const DevCtl *ctl = d.ctl;
    const int damp_on = ctl->damp_on;
    const float DAMP = ctl->DAMP;
    if (damp_on) {
        if (d.REDUCE_ORDER == 1) {
            for (int r = threadIdx.x; r < d.NROWS; r += BS) s_blk[r] = V.AVG_BLK[r];
        } else {
            int w = threadIdx.x >> 5, l = threadIdx.x & 31;
            for (int nr = w + 1; nr <= d.NROWS; nr += BS / 32) {
                int JST = A1(d.JSTART, nr) + 1, JEN = A1(d.JMIX, nr) - 1;
                const int ro = d.REDUCE_ORDER;
                df s = df_of(0.0f);
                for (int jj = JST + l; jj <= JEN; jj += 32) s = dacc(ro, s, V.pabs[jj - 1]);
                for (int o = 16; o > 0; o >>= 1) s = dacc(ro, s, df_shfl_down(s, o));
                if (l == 0) chg[nr - 1] = df_val(s) / (float)(IMM1 * KMM1 * (JEN - JST + 1));
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                int NROWS = d.NROWS;
                if (NROWS == 1) s_blk[0] = chg[0];
                if (NROWS == 2) {
                    s_blk[1] = 0.5f * (chg[0] + chg[1]);
                    s_blk[0] = s_blk[1];
                }
                if (NROWS > 2) {
                    for (int nr = 2; nr <= NROWS - 1; ++nr)
                        s_blk[nr - 1] = 0.25f * (chg[nr - 2] + chg[nr]) + 0.5f * chg[nr - 1];
                    s_blk[NROWS - 1] = 0.5f * (chg[NROWS - 2] + chg[NROWS - 1]);
                    s_blk[0] = 0.5f * (chg[0] + chg[1]);
                }
            }
        }
        __syncthreads();
    }
    // damped cell changes of the two planes this node plane touches
    for (int h = 0; h < 2; ++h) {
        int jc = j + h;
        if (jc < 2 || jc > d.JM) continue;
        float *c = h ? cB : cA;
        const float blk = damp_on ? s_blk[A1(d.NROW, jc) - 1] : 1.0f;
        const float *__restrict__ stp = V.ST + (size_t)IM * (jc - 1);     // plane jc, (i, k) at i-1 + IM*JM*(k-1)
        const size_t kstride = (size_t)IM * d.JM;
        Walk2 w(IMM1, threadIdx.x, BS);
        for (int t0 = threadIdx.x; t0 < nc; t0 += TS_UG * BS) {
            float sv[TS_UG];
#pragma unroll
            for (int u = 0; u < TS_UG; ++u) {
                if (t0 + u * BS < nc) sv[u] = stp[(size_t)(w.i - 1) + kstride * (w.k - 1)];
                w.next();
            }
#pragma unroll
            for (int u = 0; u < TS_UG; ++u) {
                const int t = t0 + u * BS;
                if (t >= nc) break;
                float v = sv[u];
                if (damp_on) {
                    float FDAMP = fabsf(v) / blk;
                    v = v / (1.0f + FDAMP / DAMP);
                }
                c[t] = v;
            }
        }
    }
    __syncthreads();
    // second pitchwise average on the mixing-plane cells (1850)
    const bool lowx = d.FEXTRAP < 0.001f;
    bool any = false;
    for (int h = 0; h < 2; ++h) {
        int jc = j + h;
        if (jc < 2 || jc > d.JM) continue;
        int mnr;
        int role = mp_role(d, jc, &mnr);
        if (role != 1 && role != 3) continue;
        any = true;
        float *c = h ? cB : cA;
        int jmx = A1(d.JMIX, mnr);
        const bool lane_par = d.REDUCE_ORDER == 0;
        const int k0 = lane_par ? (int)(threadIdx.x >> 5) + 1 : (int)threadIdx.x + 1;
        const int kstep = lane_par ? BS / 32 : BS;
        for (int k = k0; k <= KMM1; k += kstep) {
            float FLOWDIRN = -A3(d.FLOWX, d.IMID, jmx, k);
            bool on = role == 3 ? (FLOWDIRN > 0.0f || lowx) : (FLOWDIRN < 0.0f || lowx);
            if (!on) continue;
            float *row = c + (size_t)(k - 1) * IMM1;
            if (lane_par) {
                float s = warp_sum64(IMM1, [&](int i) { return row[i]; }) / (float)IMM1;
                __syncwarp();
                for (int i = (int)(threadIdx.x & 31); i < IMM1; i += 32) row[i] = s;
            } else {
                float s = mp_line_sum(row, IMM1) / (float)IMM1;
                for (int i = 0; i < IMM1; ++i) row[i] = s;
            }
        }
    }
    if (any) __syncthreads();
    // gather (1100): cells (kc, jc, ic) in the reference's loop order
    const int np = IM * KM;
    const float fdn = A1(d.FACDWN, j);
    const float fup = j + 1 <= d.JM ? A1(d.FACUP, j + 1) : 0.0f;
    const bool hA = j >= 2, hB = j + 1 <= d.JM;
    const float *__restrict__ FBL = d.FBL;
    const float *__restrict__ FBR = d.FBR;
    const float *__restrict__ FTL = d.FTL;
    const float *__restrict__ FTR = d.FTR;
    const size_t nbase = (size_t)IM * (j - 1), kstride = (size_t)IM * d.JM;
    Walk2 w(IM, threadIdx.x, BS);
    for (int t0 = threadIdx.x; t0 < np; t0 += TS_UG * BS) {
        // loads of TS_UG nodes first: the node value and, for interior nodes,
        // the four corner weights
        float dv[TS_UG], wtr[TS_UG], wtl[TS_UG], wbr[TS_UG], wbl[TS_UG];
        int ni[TS_UG], nk[TS_UG];
#pragma unroll
        for (int u = 0; u < TS_UG; ++u) {
            const int i = w.i, k = w.k;
            ni[u] = i;
            nk[u] = k;
            w.next();
            if (t0 + u * BS < np) {
                dv[u] = D[nbase + (size_t)(i - 1) + kstride * (k - 1)];
                if (hA && hB && i >= 2 && i <= IMM1 && k >= 2 && k <= KMM1) {
                    wtr[u] = FTR[(i - 2) + IM * (k - 2)];
                    wtl[u] = FTL[(i - 1) + IM * (k - 2)];
                    wbr[u] = FBR[(i - 2) + IM * (k - 1)];
                    wbl[u] = FBL[(i - 1) + IM * (k - 1)];
                }
            }
        }
#pragma unroll
        for (int u = 0; u < TS_UG; ++u) {
            if (t0 + u * BS >= np) break;
            const int i = ni[u], k = nk[u];
            const size_t n = nbase + (size_t)(i - 1) + kstride * (k - 1);
            float v = dv[u];
            if (hA && hB && i >= 2 && i <= IMM1 && k >= 2 && k <= KMM1) {
                // interior node: all eight cells, weights FTR/FTL of row k-1 and FBR/FBL of row k
                const int lo = (i - 2) + IMM1 * (k - 2), hi = lo + IMM1;   // cells (i-1, k-1), (i-1, k)
                v = v + cA[lo] * wtr[u] * fdn;
                v = v + cA[lo + 1] * wtl[u] * fdn;
                v = v + cB[lo] * wtr[u] * fup;
                v = v + cB[lo + 1] * wtl[u] * fup;
                v = v + cA[hi] * wbr[u] * fdn;
                v = v + cA[hi + 1] * wbl[u] * fdn;
                v = v + cB[hi] * wbr[u] * fup;
                v = v + cB[hi + 1] * wbl[u] * fup;
            } else {
                for (int kc = k - 1; kc <= k; ++kc) {
                    if (kc < 1 || kc > KMM1) continue;
                    for (int h = 0; h < 2; ++h) {
                        if (!(h ? hB : hA)) continue;
                        const float *c = h ? cB : cA;
                        float fac = h ? fup : fdn;
                        for (int ic = i - 1; ic <= i; ++ic) {
                            if (ic < 1 || ic > IMM1) continue;
                            float wt;
                            if (ic == i) wt = (kc == k) ? AIK(FBL, ic, kc) : AIK(FTL, ic, kc);
                            else wt = (kc == k) ? AIK(FBR, ic, kc) : AIK(FTR, ic, kc);
                            v = v + c[(kc - 1) * IMM1 + (ic - 1)] * wt * fac;
                        }
                    }
                }
            }
            V.TM[n] = v;
        }
    }
}

// ---------------------------------------------------------------------
// update over a pair of node planes: the same result as k_ts_update for
// node planes j0 and j0+1, from one CTA of PBS threads.  The CTA damps the
// three cell planes j0, j0+1, j0+2 once each (k_ts_update damps every cell
// plane in the two CTAs that read it: 2 dampings per cell plane, here 1.5),
// and each thread gathers the same (i, k) on both node planes, so the four
// corner weights, the index arithmetic and the reads of the middle cell
// plane serve both planes.  Every value is formed by the same expressions
// in the same order as in k_ts_update.
// ---------------------------------------------------------------------
template <int PBS>
__global__ void __launch_bounds__(PBS, 1024 / PBS) k_ts_update_pair(const __grid_constant__ Dev d, int v0) {
    pdl_wait();
    extern __shared__ float sm[];
    const VarSet &V = d.var[v0 + blockIdx.y];
    const float *__restrict__ D = V.D;
    float *__restrict__ TM = V.TM;
    __shared__ float s_blk[64];
    __shared__ float chg[64];
    const int j0 = 2 * blockIdx.x + 1;
    const int IM = d.IM, JM = d.JM, IMM1 = d.IMM1, KM = d.KM, KMM1 = d.KMM1;
    const int nc = IMM1 * KMM1;
    const bool two = j0 + 1 <= JM;              // the second node plane exists
    const DevCtl *ctl = d.ctl;
    const int damp_on = ctl->damp_on;
    const float DAMP = ctl->DAMP;
    if (damp_on) {
        if (d.REDUCE_ORDER == 1) {
            for (int r = threadIdx.x; r < d.NROWS; r += PBS) s_blk[r] = V.AVG_BLK[r];
        } else {
            const int ro = d.REDUCE_ORDER;
            int w = threadIdx.x >> 5, l = threadIdx.x & 31;
            for (int nr = w + 1; nr <= d.NROWS; nr += PBS / 32) {
                int JST = A1(d.JSTART, nr) + 1, JEN = A1(d.JMIX, nr) - 1;
                df s = df_of(0.0f);
                for (int jj = JST + l; jj <= JEN; jj += 32) s = dacc(ro, s, V.pabs[jj - 1]);
                for (int o = 16; o > 0; o >>= 1) s = dacc(ro, s, df_shfl_down(s, o));
                if (l == 0) chg[nr - 1] = df_val(s) / (float)(IMM1 * KMM1 * (JEN - JST + 1));
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                int NROWS = d.NROWS;
                if (NROWS == 1) s_blk[0] = chg[0];
                if (NROWS == 2) {
                    s_blk[1] = 0.5f * (chg[0] + chg[1]);
                    s_blk[0] = s_blk[1];
                }
                if (NROWS > 2) {
                    for (int nr = 2; nr <= NROWS - 1; ++nr)
                        s_blk[nr - 1] = 0.25f * (chg[nr - 2] + chg[nr]) + 0.5f * chg[nr - 1];
                    s_blk[NROWS - 1] = 0.5f * (chg[NROWS - 2] + chg[NROWS - 1]);
                    s_blk[0] = 0.5f * (chg[0] + chg[1]);
                }
            }
        }
        __syncthreads();
    }
    // damped cell changes of the cell planes j0, j0+1, j0+2 (those in 2..JM)
    const int ks = IM * JM;
    for (int h = 0; h < 3; ++h) {
        const int jc = j0 + h;
        if (jc < 2 || jc > JM) continue;
        float *c = sm + h * nc;
        const float blk = damp_on ? s_blk[A1(d.NROW, jc) - 1] : 1.0f;
        const float *__restrict__ stp = V.ST + IM * (jc - 1);
        Walk2 w(IMM1, threadIdx.x, PBS);
        for (int t0 = threadIdx.x; t0 < nc; t0 += TS_UG * PBS) {
            float sv[TS_UG];
#pragma unroll
            for (int u = 0; u < TS_UG; ++u) {
                if (t0 + u * PBS < nc) sv[u] = stp[(w.i - 1) + ks * (w.k - 1)];
                w.next();
            }
#pragma unroll
            for (int u = 0; u < TS_UG; ++u) {
                const int t = t0 + u * PBS;
                if (t >= nc) break;
                float v = sv[u];
                if (damp_on) {
                    float FDAMP = fabsf(v) / blk;
                    v = v / (1.0f + FDAMP / DAMP);
                }
                c[t] = v;
            }
        }
    }
    __syncthreads();
    // second pitchwise average on the mixing-plane cells (1850)
    const bool lowx = d.FEXTRAP < 0.001f;
    bool any = false;
    for (int h = 0; h < 3; ++h) {
        const int jc = j0 + h;
        if (jc < 2 || jc > JM) continue;
        int mnr;
        const int role = mp_role(d, jc, &mnr);
        if (role != 1 && role != 3) continue;
        any = true;
        float *c = sm + h * nc;
        const int jmx = A1(d.JMIX, mnr);
        const bool lane_par = d.REDUCE_ORDER == 0;
        const int k0 = lane_par ? (int)(threadIdx.x >> 5) + 1 : (int)threadIdx.x + 1;
        const int kstep = lane_par ? PBS / 32 : PBS;
        for (int k = k0; k <= KMM1; k += kstep) {
            float FLOWDIRN = -A3(d.FLOWX, d.IMID, jmx, k);
            bool on = role == 3 ? (FLOWDIRN > 0.0f || lowx) : (FLOWDIRN < 0.0f || lowx);
            if (!on) continue;
            float *row = c + (k - 1) * IMM1;
            if (lane_par) {
                float s = warp_sum64(IMM1, [&](int i) { return row[i]; }) / (float)IMM1;
                __syncwarp();
                for (int i = (int)(threadIdx.x & 31); i < IMM1; i += 32) row[i] = s;
            } else {
                float s = mp_line_sum(row, IMM1) / (float)IMM1;
                for (int i = 0; i < IMM1; ++i) row[i] = s;
            }
        }
    }
    if (any) __syncthreads();
    // gather (1100) on both node planes
    const float *c0 = sm, *c1 = sm + nc, *c2 = sm + 2 * nc;
    const float fdn0 = A1(d.FACDWN, j0), fup0 = two ? A1(d.FACUP, j0 + 1) : 0.0f;
    const float fdn1 = two ? A1(d.FACDWN, j0 + 1) : 0.0f;
    const float fup1 = j0 + 2 <= JM ? A1(d.FACUP, j0 + 2) : 0.0f;
    const bool hA0 = j0 >= 2, hB0 = two;         // cell planes of node plane j0
    const bool hB1 = j0 + 2 <= JM;               // node plane j0 + 1 always has its cell plane j0 + 1
    const float *__restrict__ FBL = d.FBL;
    const float *__restrict__ FBR = d.FBR;
    const float *__restrict__ FTL = d.FTL;
    const float *__restrict__ FTR = d.FTR;
    const int nb0 = IM * (j0 - 1);
    const int np = IM * KM;
    // one node of a node plane from its <= 8 cells (kc, h, ic), cA the cell
    // plane before it and cB the one after, added in the reference's order
    // (kc outer, then the plane, then ic); a cell outside the grid is
    // skipped.  One thread per column of UG_SEG nodes along K at one I, the
    // lanes on successive I: walking up the column, the cells above a node
    // are the cells below the next one, so each cell value is read from
    // shared memory once per column and the boundary nodes take the same
    // predicated path as the inner ones
    const bool pv0 = hA0, pv1 = two, pv2 = hB1;  // cell planes j0, j0 + 1, j0 + 2 present
    const int nsk = (KM + UG_SEG - 1) / UG_SEG;
    Walk2 w(IM, threadIdx.x, PBS);
    for (int t = threadIdx.x; t < IM * nsk; t += PBS, w.next()) {
        const int i = w.i, k0 = 1 + UG_SEG * (w.k - 1);
        const int len = min(UG_SEG, KM - k0 + 1);
        const bool hL = i >= 2, hR = i <= IMM1;
        // the global operands of the column's nodes, loaded together
        float dv0[UG_SEG], dv1[UG_SEG], wtr[UG_SEG], wtl[UG_SEG], wbr[UG_SEG], wbl[UG_SEG];
#pragma unroll
        for (int q = 0; q < UG_SEG; ++q) {
            if (q >= len) break;
            const int k = k0 + q;
            const int n = nb0 + (i - 1) + ks * (k - 1);
            const bool hD = k >= 2, hU = k <= KMM1;
            dv0[q] = D[n];
            dv1[q] = two ? D[n + IM] : 0.0f;
            wtr[q] = (hL && hD) ? FTR[(i - 2) + IM * (k - 2)] : 0.0f;
            wtl[q] = (hR && hD) ? FTL[(i - 1) + IM * (k - 2)] : 0.0f;
            wbr[q] = (hL && hU) ? FBR[(i - 2) + IM * (k - 1)] : 0.0f;
            wbl[q] = (hR && hU) ? FBL[(i - 1) + IM * (k - 1)] : 0.0f;
        }
        // cells (i-1, r) and (i, r) of the three cell planes, r = the cell
        // row below the node (dn) and above it (up)
        float dn0l = 0.0f, dn0r = 0.0f, dn1l = 0.0f, dn1r = 0.0f, dn2l = 0.0f, dn2r = 0.0f;
        const int cl = i - 2;                       // cell (i-1, r) at cl + IMM1*(r-1)
        if (k0 >= 2) {
            const int o = cl + IMM1 * (k0 - 2);
            if (pv0 && hL) dn0l = c0[o];
            if (pv0 && hR) dn0r = c0[o + 1];
            if (pv1 && hL) dn1l = c1[o];
            if (pv1 && hR) dn1r = c1[o + 1];
            if (pv2 && hL) dn2l = c2[o];
            if (pv2 && hR) dn2r = c2[o + 1];
        }
#pragma unroll
        for (int q = 0; q < UG_SEG; ++q) {
            if (q >= len) break;
            const int k = k0 + q;
            const bool hD = k >= 2, hU = k <= KMM1;
            float up0l = 0.0f, up0r = 0.0f, up1l = 0.0f, up1r = 0.0f, up2l = 0.0f, up2r = 0.0f;
            if (hU) {
                const int o = cl + IMM1 * (k - 1);
                if (pv0 && hL) up0l = c0[o];
                if (pv0 && hR) up0r = c0[o + 1];
                if (pv1 && hL) up1l = c1[o];
                if (pv1 && hR) up1r = c1[o + 1];
                if (pv2 && hL) up2l = c2[o];
                if (pv2 && hR) up2r = c2[o + 1];
            }
            const int n = nb0 + (i - 1) + ks * (k - 1);
            // node plane j0: cell planes j0 and j0 + 1
            float v = dv0[q];
            if (hD) {
                if (hA0 && hL) v = v + dn0l * wtr[q] * fdn0;
                if (hA0 && hR) v = v + dn0r * wtl[q] * fdn0;
                if (hB0 && hL) v = v + dn1l * wtr[q] * fup0;
                if (hB0 && hR) v = v + dn1r * wtl[q] * fup0;
            }
            if (hU) {
                if (hA0 && hL) v = v + up0l * wbr[q] * fdn0;
                if (hA0 && hR) v = v + up0r * wbl[q] * fdn0;
                if (hB0 && hL) v = v + up1l * wbr[q] * fup0;
                if (hB0 && hR) v = v + up1r * wbl[q] * fup0;
            }
            TM[n] = v;
            if (two) {
                // node plane j0 + 1: cell planes j0 + 1 and j0 + 2
                float v1 = dv1[q];
                if (hD) {
                    if (hL) v1 = v1 + dn1l * wtr[q] * fdn1;
                    if (hR) v1 = v1 + dn1r * wtl[q] * fdn1;
                    if (hB1 && hL) v1 = v1 + dn2l * wtr[q] * fup1;
                    if (hB1 && hR) v1 = v1 + dn2r * wtl[q] * fup1;
                }
                if (hU) {
                    if (hL) v1 = v1 + up1l * wbr[q] * fdn1;
                    if (hR) v1 = v1 + up1r * wbl[q] * fdn1;
                    if (hB1 && hL) v1 = v1 + up2l * wbr[q] * fup1;
                    if (hB1 && hR) v1 = v1 + up2r * wbl[q] * fup1;
                }
                TM[n + IM] = v1;
            }
            dn0l = up0l; dn0r = up0r; dn1l = up1l; dn1r = up1r; dn2l = up2l; dn2r = up2r;
        }
    }
}

// ---------------------------------------------------------------------
// smooth: SMOOTH_VAR (3900-9000, 8502) + periodic (8000), tip gap (510),
// mixing-plane average (100): TMP -> D, one CTA per J-plane
// ---------------------------------------------------------------------
// Streamwise smoothing case of plane j (SMOOTH_VAR 15375-15406): the
// reference tests the cases in this order and the last one that holds wins.
__device__ inline int stream_case(const Dev &d, int j) {
    int nr = A1(d.NROW, j);
    int J1 = A1(d.JSTART, nr), J2 = A1(d.JMIX, nr);
    int sc = 0;                                   // 0: unchanged
    if (j >= J1 + 3 && j <= J2 - 3) sc = 1;       // 2nd + 4th order interior
    if (j == J2) sc = 0;
    if (j == J1) sc = 0;
    if (j == J1 + 2) sc = 2;
    if (j == J1 + 1) sc = 3;
    if (j == J2 - 2) sc = 4;
    if (j == J2 - 1) sc = 5;
    return sc;
}

// Leading-edge periodic smoothing case of plane j (15417-15434): 1 on the
// two planes before a row's JLED, 2 on JLED itself; the last row that
// matches wins.
__device__ inline int le_case(const Dev &d, int j) {
    int lc = 0;
    for (int r = 1; r <= d.NROWS; ++r) {
        int JL = A1(d.JLED, r);
        if (j == JL - 2 || j == JL - 1) lc = 1;
        if (j == JL) lc = 2;
    }
    return lc;
}

template <int BS>
__global__ void __launch_bounds__(BS, 1024 / BS) k_ts_smooth(const __grid_constant__ Dev d, int v0) {
    pdl_wait();
    extern __shared__ float sm[];
    const VarSet &V = d.var[v0 + blockIdx.y];
    const float *__restrict__ S = V.TM;
    float *__restrict__ D = V.D;
    const int IM = d.IM, KM = d.KM, IMM1 = d.IMM1, KMM1 = d.KMM1;
    const int np = IM * KM;
    // the plane buffers hold (i, k) at (i-1) + IMP*(k-1); the odd row pitch
    // keeps the pitchwise pass, whose lanes step from one K line to the
    // next, free of bank conflicts
    const int IMP = IM | 1;
    float *a = sm, *b = sm + IMP * KM;
    float *cFD = b + IMP * KM, *cFU = cFD + IM, *cFKD = cFU + IM, *cFKU = cFKD + KM;   // FD, FU, FKD, FKU
    const int j = blockIdx.x + 1;
    const DevCtl *c = d.ctl;
    const bool stream = !(c->SFX < 0.0001f);
    for (int t = threadIdx.x; t < IM; t += BS) {
        cFD[t] = d.FD[t];
        cFU[t] = d.FU[t];
    }
    for (int t = threadIdx.x; t < KM; t += BS) {
        cFKD[t] = d.FKD[t];
        cFKU[t] = d.FKU[t];
    }
    const int ks = IM * d.JM;                        // K stride of a node array
    const float *__restrict__ Sj = S + IM * (j - 1);  // plane j: (i, k) at i-1 + ks*(k-1)
    {
        const int sc = stream ? stream_case(d, j) : 0;
        const int lc = stream ? le_case(d, j) : 0;
        const int nr = A1(d.NROW, j);
        const int J1 = A1(d.JSTART, nr), J2 = A1(d.JMIX, nr);
        const float SFX = c->SFX, SFX1 = c->SFX1, SFXB = c->SFXB, SFXB1 = c->SFXB1, SFXBH = c->SFXBH;
        const float SFXHM1 = c->SFXHM1, SFX14 = c->SFX14, F4 = d.FAC_4TH;
        // the J planes each case reads, as node offsets from plane j
        int nq = 0;
        ptrdiff_t off[4] = {0, 0, 0, 0};
        auto add = [&](int jj) { off[nq++] = (ptrdiff_t)IM * (jj - j); };
        if (sc == 1) { add(j + 1); add(j - 1); add(j - 2); add(j + 2); }
        if (sc == 2) { add(J1 + 3); add(J1 + 1); }
        if (sc == 3) { add(J1 + 2); add(J1 + 3); add(J1 + 4); }
        if (sc == 4) { add(J2 - 1); add(J2 - 3); }
        if (sc == 5) { add(J2 - 2); add(J2 - 3); add(J2 - 4); }
        Walk2 w(IM, threadIdx.x, BS);
        for (int t0 = threadIdx.x; t0 < np; t0 += SV_U * BS) {
            float d0[SV_U], x[SV_U][4];
            int pi[SV_U], pk[SV_U];
#pragma unroll
            for (int u = 0; u < SV_U; ++u) {
                pi[u] = w.i;
                pk[u] = w.k;
                w.next();
                if (t0 + u * BS < np) {
                    const float *p = Sj + (pi[u] - 1) + ks * (pk[u] - 1);
                    d0[u] = p[0];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (q < nq) x[u][q] = p[off[q]];
                }
            }
#pragma unroll
            for (int u = 0; u < SV_U; ++u) {
                const int t = t0 + u * BS;
                if (t >= np) break;
                const int i = pi[u], k = pk[u];
                const float dd = d0[u];
                float v = dd;
                switch (sc) {
                case 1: {
                    float AVERG = 0.5f * (x[u][0] + x[u][1]);
                    float CURV = AVERG - 0.5f * dd - 0.25f * (x[u][2] + x[u][3]);
                    v = SFX1 * dd + SFX * (AVERG + F4 * CURV);
                    break;
                }
                case 2: case 4: v = SFXB1 * dd + SFXBH * (x[u][0] + x[u][1]); break;
                case 3: case 5: v = SFXB1 * dd + SFXB * (1.25f * x[u][0] + 0.5f * x[u][1] - 0.75f * x[u][2]); break;
                default: break;
                }
                if (lc && (i == 1 || i == IM)) {
                    const float *pkk = Sj + ks * (k - 1);
                    if (lc == 1) v = SFXHM1 * dd + SFX14 * (pkk[1] + pkk[IMM1 - 1]);
                    else if (i == 1) v = SFXHM1 * dd + SFX14 * (pkk[IM + 0] + pkk[IM - 1]);
                    else v = SFXHM1 * dd + SFX14 * (pkk[IM + IM - 1] + pkk[0]);
                }
                a[(i - 1) + IMP * (k - 1)] = v;
            }
        }
    }
    __syncthreads();
#define P(buf, i, k) buf[((i) - 1) + IMP * ((k) - 1)]
    const bool periodic_j = !(A1(d.IND, j) == 1 || A1(d.INDLE, j) == 1);
    if (j >= 2 && !(c->SFT < 0.0001f)) {
        const float SFT = c->SFT, SFT1 = c->SFT1, F4 = d.FAC_4TH;
        // the points I = 2..IMM1 first, in segments of SM_SEG points of one K
        // line per thread, the lanes on successive K lines: each point's
        // curvature is formed once and the segment's values stay in
        // registers.  The curvature at I = 1 and IM, which the points I = 2
        // and IMM1 take, is one value per line (the reference's CURVE there
        // is the I = 1 value, or 0 off the periodic planes)
        const int nsi = (IM - 2 + SM_SEG - 1) / SM_SEG;
        Walk2 w(KM, threadIdx.x, BS);
        for (int t = threadIdx.x; t < nsi * KM; t += BS, w.next()) {
            const int k = w.i, i0 = 2 + SM_SEG * (w.k - 1);
            const int len = min(SM_SEG, IMM1 - i0 + 1);
            const float *ak = a + IMP * (k - 1) - 1;     // ak[i] = P(a, i, k)
            float x[SM_SEG + 4];                          // x[q] = P(a, i0 - 2 + q, k)
#pragma unroll
            for (int q = 0; q < SM_SEG + 4; ++q) {
                const int ii = i0 - 2 + q;
                x[q] = (q < len + 4 && ii >= 1 && ii <= IM) ? ak[ii] : 0.0f;
            }
            const float cper = periodic_j ? ak[1] - 0.5f * (ak[2] + ak[IMM1]) : 0.0f;
            float g[SM_SEG + 2];                          // g[q]: the curvature at I = i0 - 1 + q
#pragma unroll
            for (int q = 0; q < SM_SEG + 2; ++q) {
                const int ii = i0 - 1 + q;
                g[q] = (ii == 1 || ii >= IM) ? cper : x[q + 1] - (cFD[ii - 1] * x[q + 2] + cFU[ii - 1] * x[q]);
            }
            float *bk = b + IMP * (k - 1) - 1;
#pragma unroll
            for (int q = 0; q < SM_SEG; ++q) {
                if (q >= len) break;
                const int ii = i0 + q;
                const float AVG = cFD[ii - 1] * x[q + 3] + cFU[ii - 1] * x[q + 1];
                const float SC = cFU[ii - 1] * g[q] + cFD[ii - 1] * g[q + 2];
                bk[ii] = SFT1 * x[q + 2] + SFT * (AVG + F4 * SC);
            }
        }
        // then the points I = 1 and IM of every line
        for (int t = threadIdx.x; t < 2 * KM; t += BS) {
            const int i = (t & 1) ? IM : 1, k = (t >> 1) + 1;
            const float *ak = a + IMP * (k - 1) - 1;
            float AVG, SC;
            if (periodic_j) {
                AVG = 0.5f * (ak[2] + ak[IMM1]);
                const float c2 = ak[2] - (cFD[1] * ak[3] + cFU[1] * ak[1]);
                const float cm1 = ak[IMM1] - (cFD[IMM1 - 1] * ak[IM] + cFU[IMM1 - 1] * ak[d.IMM2]);
                SC = 0.5f * (c2 + cm1);
            } else {
                if (i == 1) AVG = ak[2] + cFU[0] * (ak[2] - ak[3]);
                else AVG = ak[IMM1] + cFU[IM - 1] * (ak[IMM1] - ak[d.IMM2]);
                SC = 0.0f;
            }
            P(b, i, k) = SFT1 * ak[i] + SFT * (AVG + F4 * SC);
        }
        __syncthreads();
        // spanwise: segments of SM_SEG points of one I line per thread, the
        // lanes on successive I lines
        const int nsk = (KM + SM_SEG - 1) / SM_SEG;
        w = Walk2(IM, threadIdx.x, BS);
        for (int t = threadIdx.x; t < nsk * IM; t += BS, w.next()) {
            const int i = w.i, k0 = 1 + SM_SEG * (w.k - 1);
            const int len = min(SM_SEG, KM - k0 + 1);
            const float *bi = b + (i - 1) - IMP;          // bi[IMP * kk] = P(b, i, kk)
            float y[SM_SEG + 4];                          // y[q] = P(b, i, k0 - 2 + q)
#pragma unroll
            for (int q = 0; q < SM_SEG + 4; ++q) {
                const int kk = k0 - 2 + q;
                y[q] = (q < len + 4 && kk >= 1 && kk <= KM) ? bi[IMP * kk] : 0.0f;
            }
            float h[SM_SEG + 2];                          // h[q]: the curvature at K = k0 - 1 + q
#pragma unroll
            for (int q = 0; q < SM_SEG + 2; ++q) {
                const int kk = k0 - 1 + q;
                h[q] = (kk <= 1 || kk >= KM) ? 0.0f : y[q + 1] - (cFKD[kk - 1] * y[q + 2] + cFKU[kk - 1] * y[q]);
            }
#pragma unroll
            for (int q = 0; q < SM_SEG; ++q) {
                if (q >= len) break;
                const int kk = k0 + q;
                float AVG, SC;
                if (kk == 1) {
                    AVG = y[q + 3] + 0.5f * cFKU[0] * (y[q + 3] - y[q + 4]);
                    SC = 0.0f;
                } else if (kk == KM) {
                    AVG = y[q + 1] + 0.5f * cFKU[KM - 1] * (y[q + 1] - y[q]);
                    SC = 0.0f;
                } else {
                    AVG = cFKD[kk - 1] * y[q + 3] + cFKU[kk - 1] * y[q + 1];
                    SC = cFKU[kk - 1] * h[q] + cFKD[kk - 1] * h[q + 2];
                }
                P(a, i, kk) = SFT1 * y[q + 2] + SFT * (AVG + F4 * SC);
            }
        }
        __syncthreads();
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
    if (!(d.SFEXIT < 0.0001f) && j >= d.JM + 1 - d.NSFEXIT) {
        const float SE = d.SFEXIT, SE1 = 1.0f - SE, SEH = 0.5f * SE;
        for (int k = threadIdx.x + 1; k <= KM; k += BS) {
            for (int i = 2; i <= IMM1; ++i) P(a, i, k) = SE1 * P(a, i, k) + SEH * (P(a, i + 1, k) + P(a, i - 1, k));
            P(a, 1, k) = P(a, 1, k) + SE * (2.0f * P(a, 2, k) - P(a, 3, k) - P(a, 1, k));
            P(a, IM, k) = P(a, IM, k) + SE * (2.0f * P(a, IMM1, k) - P(a, d.IMM2, k) - P(a, IM, k));
        }
        __syncthreads();
        for (int i = threadIdx.x + 1; i <= IM; i += BS) {
            for (int k = 2; k <= KMM1; ++k) P(a, i, k) = SE1 * P(a, i, k) + SEH * (P(a, i, k - 1) + P(a, i, k + 1));
            P(a, i, 1) = P(a, i, 1) + SE * (2.0f * P(a, i, 2) - P(a, i, 3) - P(a, i, 1));
            P(a, i, KM) = P(a, i, KM) + SE * (2.0f * P(a, i, KMM1) - P(a, i, d.KMM2) - P(a, i, KM));
        }
        __syncthreads();
    }
    int nr = A1(d.NROW, j);
    int K1 = A1(d.KTIPS, nr), K2 = A1(d.KTIPE, nr);
    bool tip = K1 > 0;
    if (tip) {
        if (K1 == 1) K2 = K2 - 1;
        if (K2 == KM) K1 = K1 + 1;
    }
    for (int k = threadIdx.x + 1; k <= KM; k += BS) {
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
    bool mp = false;
    if (d.IFMIX != 0)
        for (int r = 1; r <= d.NRWSM1; ++r)
            if (j == A1(d.JMIX, r) || j == A1(d.JMIX, r) + 1) mp = true;
    if (mp) {
        if (d.REDUCE_ORDER != 0) {
            for (int k = threadIdx.x + 1; k <= KM; k += BS) {
                float s = 0.0f;
                for (int i = 1; i <= IMM1; ++i) s = s + A1(d.FP, i) * (P(a, i, k) + P(a, i + 1, k));
                b[k - 1] = 0.5f * s;
            }
        } else {
            for (int k = (int)(threadIdx.x >> 5) + 1; k <= KM; k += BS / 32) {
                float s = warp_sum64(IMM1, [&](int i) { return A1(d.FP, i + 1) * (P(a, i + 1, k) + P(a, i + 2, k)); });
                if ((threadIdx.x & 31) == 0) b[k - 1] = 0.5f * s;
            }
        }
        __syncthreads();
        Walk2 w(IM, threadIdx.x, BS);
        for (int t = threadIdx.x; t < np; t += BS, w.next()) P(a, w.i, w.k) = b[w.k - 1];
        __syncthreads();
    }
#undef P
    float *Dj = D + IM * (j - 1);
    Walk2 w(IM, threadIdx.x, BS);
    for (int t = threadIdx.x; t < np; t += BS, w.next()) Dj[(w.i - 1) + ks * (w.k - 1)] = a[(w.i - 1) + IMP * (w.k - 1)];
}

// ---------------------------------------------------------------------
// SMOOTH_RESID (14833-14917): one Jacobi pass along J, I or K of the cell
// changes inside each row, src -> dst (cells outside every row are copied)
// ---------------------------------------------------------------------
__global__ void k_resid_pass(const __grid_constant__ Dev d, int v0, int dir, float smfac, int st_to_tm) {
    pdl_wait();
    const VarSet &V = d.var[v0 + blockIdx.y];
    const float *__restrict__ src = st_to_tm ? V.ST : V.TM;
    float *__restrict__ dst = st_to_tm ? V.TM : V.ST;
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

// STORE = TMP after the three SMOOTH_RESID passes
__global__ void k_copy_tm_st(const __grid_constant__ Dev d, int v0, size_t n) {
    pdl_wait();
    const VarSet &V = d.var[v0 + blockIdx.y];
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) V.ST[t] = V.TM[t];
}

static size_t cells_smem(const Dev &d) {
    return ((size_t)d.IMM1 * d.KMM1 + d.KMM1 + (size_t)d.NIB1 * d.NKB1) * sizeof(float);
}
static size_t prolong_smem(const Dev &d) { return ((size_t)d.NIB1 * d.NKB1 + (size_t)d.NIB2 * d.NKB2) * sizeof(float); }
static size_t update_smem(const Dev &d) { return (size_t)2 * d.IMM1 * d.KMM1 * sizeof(float); }
static size_t update_pair_smem(const Dev &d) { return (size_t)3 * d.IMM1 * d.KMM1 * sizeof(float); }
static size_t smooth_smem(const Dev &d) { return ((size_t)2 * (d.IM | 1) * d.KM + 2 * d.IM + 2 * d.KM) * sizeof(float); }

template <int BS>
static cudaError_t configure_bs(const Dev &d) {
    struct {
        const void *f;
        size_t bytes;
    } k[] = {{(const void *)k_ts_cells<BS>, cells_smem(d)},
             {(const void *)k_ts_prolong<BS>, prolong_smem(d)},
             {(const void *)k_ts_update<BS>, update_smem(d)},
             {(const void *)k_ts_update_pair<2 * BS>, update_pair_smem(d)},
             {(const void *)k_ts_smooth<BS>, smooth_smem(d)}};
    for (auto &x : k) {
        if (x.bytes > 200 * 1024) return cudaErrorInvalidValue;
        cudaError_t e = raise_smem(x.f, x.bytes);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t configure_kernels(const Dev &d) {
    cudaError_t e = configure_bs<128>(d);
    if (e == cudaSuccess) e = configure_bs<256>(d);
    if (e == cudaSuccess) e = configure_bs<192>(d);
    if (e == cudaSuccess) e = configure_bs<512>(d);
    if (e == cudaSuccess) e = configure_loss_kernels(d);
    return e != cudaSuccess ? e : configure_flux_kernels(d);
}

// TSTEP up to the negative feedback's row means: flux sum, SCREE and the
// mixing-plane redistribution (cells), the multigrid block sums and the
// time step (prolong), SMOOTH_RESID of STORE, and |STORE| per plane (or,
// with REDUCE_ORDER=1, the row means in the reference's order)
template <int BS>
static void launch_tstep_front(const Dev &d, Launch L, int v0, int nv) {
    size_t N = (size_t)d.IM * d.JM * d.KM;
    unsigned gN = grid_for(N, 256);
    const bool seq = d.REDUCE_ORDER == 1;
    const unsigned jp = (unsigned)(d.JM - 1), vy = (unsigned)nv;
    launchk(L, k_ts_cells<BS>, dim3(jp, vy), dim3(BS), cells_smem(d), d, v0);
    mark(L, "k_ts_cells");
    if (seq) {
        int nb = d.NIB1 * (d.NJB1 + 1) * d.NKB1 + d.NIB2 * (d.NJB2 + 1) * d.NKB2 + d.NSBLK;
        launchk(L, k_ts_restrict_seq, dim3(grid_for(nb, 64), vy), dim3(64), 0, d, v0);
        mark(L, "k_ts_restrict_seq");
    }
    launchk(L, k_ts_prolong<BS>, dim3(jp, vy), dim3(BS), prolong_smem(d), d, v0, (d.NRSMTH == 0 && !seq) ? 1 : 0);
    mark(L, "k_ts_prolong");
    if (d.NRSMTH > 0) {
        for (int it = 0; it < d.NRSMTH; ++it) {
            launchk(L, k_resid_pass, dim3(gN, vy), dim3(256), 0, d, v0, 0, d.RSMTH, 1);
            mark(L, "k_resid_pass");
            launchk(L, k_resid_pass, dim3(gN, vy), dim3(256), 0, d, v0, 1, d.RSMTH, 0);
            mark(L, "k_resid_pass");
            launchk(L, k_resid_pass, dim3(gN, vy), dim3(256), 0, d, v0, 2, d.RSMTH, 1);
            mark(L, "k_resid_pass");
            launchk(L, k_copy_tm_st, dim3(gN, vy), dim3(256), 0, d, v0, N);
            mark(L, "k_copy_tm_st");
        }
        if (!seq) {
            launchk(L, k_ts_plane_abs<BS>, dim3(jp, vy), dim3(BS), 0, d, v0);
            mark(L, "k_ts_plane_abs");
        }
    }
    if (seq) {
        launchk(L, k_ts_avgblk_seq, dim3(1, vy), dim3(32), 0, d, v0);
        mark(L, "k_ts_avgblk_seq");
    }
}

template <int BS>
static void launch_tstep_bs(const Dev &d, Launch L, int v0, int nv) {
    launch_tstep_front<BS>(d, L, v0, nv);
    const unsigned ja = (unsigned)d.JM, vy = (unsigned)nv;
    if (d.TS_PAIR) {
        launchk(L, k_ts_update_pair<2 * BS>, dim3((ja + 1) / 2, vy), dim3(2 * BS), update_pair_smem(d), d, v0);
        mark(L, "k_ts_update_pair");
    } else {
        launchk(L, k_ts_update<BS>, dim3(ja, vy), dim3(BS), update_smem(d), d, v0);
        mark(L, "k_ts_update");
    }
    launchk(L, k_ts_smooth<BS>, dim3(ja, vy), dim3(BS), smooth_smem(d), d, v0);
    mark(L, "k_ts_smooth");
}

void launch_tstep_cells_prolong(const Dev &d, Launch L, int v0, int nv) {
    const int bs = d.ts_bs[0];
    if (bs == 128) launch_tstep_front<128>(d, L, v0, nv);
    else if (bs == 192) launch_tstep_front<192>(d, L, v0, nv);
    else if (bs == 512) launch_tstep_front<512>(d, L, v0, nv);
    else launch_tstep_front<256>(d, L, v0, nv);
}

void launch_tstep(const Dev &d, Launch L, int v0, int nv) {
    const int bs = d.ts_bs[nv >= 3 ? 1 : 0];
    if (bs == 128) launch_tstep_bs<128>(d, L, v0, nv);
    else if (bs == 192) launch_tstep_bs<192>(d, L, v0, nv);
    else if (bs == 512) launch_tstep_bs<512>(d, L, v0, nv);
    else launch_tstep_bs<256>(d, L, v0, nv);
}

}  // namespace mgpu
