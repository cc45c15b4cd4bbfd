// mgpu_adjoint.cu -- the discrete adjoint of one time-marching step
// (multall-open-18.3.f:3759-5240 with LOSS and STEPUP held: frozen body
// forces and time steps) and its fixed-point solve.
//
// The converged flow U* is a fixed point of the step map U -> G(U, A)
// (A: the geometry arrays).  For an objective J(U, A) the adjoint lambda
// solves lambda = (dG/dU)^T lambda + (dJ/dU)^T, iterated exactly like the
// flow itself (the transposed step has the primal's convergence rate), and
// then dJ/dA = dJ/dA|_U + lambda^T dG/dA.
//
// mgpu_adjoint_prepare runs one step from the current state with recording
// hooks and keeps what the reverse kernels need (the state before the step,
// the primitive, flux and cell-change arrays of the step, the inlet density
// and the mixing-plane inputs); the state is then restored.  Every reverse
// kernel below undoes one forward kernel of the step, in reverse order:
//   k_mixplan -> k_ts_* (momenta) -> k_flux_mom (fluxes, then PEFF) -> k_bc_apply ->
//   k_ts_* (RO, ROE) -> energy fluxes -> k_bc_sums -> mass fluxes -> k_prim
// Each takes the adjoints of its forward kernel's outputs and adds the
// adjoints of its inputs; outputs that the forward kernel overwrote get the
// adjoint of their old value (zero, or what the kernel read of it).  Where
// several forward outputs read one input, the reverse scatter uses float
// atomics; the result is not bitwise reproducible, but its rounding is far
// below the FP32 adjoint's accuracy.  Branches (limits, the flow-direction
// tests, |STORE| in the negative feedback) are taken as the recorded step
// took them.
//
// The per-node reverse kernels take Dev and Adj by value and inline their
// helpers, so every member read stays a constant-bank parameter load; only
// the J-plane kernels, which index a.v by blockIdx.y, take them as
// __grid_constant__.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "mgpu_internal.cuh"

namespace mgpu {

// adjoints of one conserved variable's TSTEP operands
struct AdjVar {
    float *D, *DIFF;             // the variable and its SCREE history (state)
    float *XF, *TF, *RF, *SR;    // face fluxes and source
    float *ST;                   // cell changes after prolongation
    float *TM;                   // node values before SMOOTH_VAR
    float *Y;                    // ST * RSTEP: the restriction operand of the transposed prolongation
    float *P1, *P2;              // per-plane block partials of Y
    df *psum;                    // (JM) per-plane sums of Y (double-float)
    double *pblk;                // (JM) per-plane sums of dJ/d(row mean |STORE|)
    const float *tST;            // recorded STORE after prolongation
    const float *tBLK;           // (NROWS) recorded row means of |STORE| after the row mixing
};

struct Adj {
    AdjVar v[NVAR];
    // adjoints of the step's node arrays (full size; between steps only the
    // state parts are nonzero: PEFF, P at J=1, HO at J=JM, ROVT at J=1)
    float *P, *HO, *VX, *VR, *VT, *ROVT, *PEFF, *FLOWX, *FLOWT, *FLOWR;
    float *PD, *PDK, *PAVG, *SSUM;   // (KM)
    // the recorded step: state before it ...
    const float *tRO, *tROVX, *tROVR, *tRORVT, *tROE, *tPEFF0, *tHOJM, *tROVT1, *tP1;
    // ... and arrays as the step formed them
    const float *tVX, *tVR, *tVT, *tROVT, *tP, *tHO, *tPEFF, *tFLOWX, *tFLOWT, *tFLOWR;
    const float *tBCBUF, *tROIN, *tMIX;
    // limiters: RO as each found it, WT of the step, the rows' limits, and
    // the density limiter's linear coefficients lim(J) = C0 RO(J) + CA ROAVG
    const float *tROL, *tROM, *tWT, *tVLIM, *tROLIM, *tDC0, *tDCA;
    const int *tDCOL;
    float *WT;                   // adjoint of WT (k_flux_mass_energy), read by the Mach limiter
    float *cf;                   // per-face coefficients of the flux reverses (MOM_NCOEF x N)
    const DevCtl *tctl;
    // geometry adjoints, accumulated when geom != 0
    float *gAQX, *gAQR, *gABX, *gABR, *gABT, *gASX, *gASR, *gVOLOR;
    int geom;
    int *flag;                   // bit 0: supersonic mixing-plane sweep met
    // objective seeds: node quantities (VX, VT, VR, HO, P) and cell FLOWX on
    // two J planes
    const float *seed;
    const int *seed_on;          // 0: the plain transposed step (Krylov products)
    int seed_j[2];
};

namespace {

inline unsigned gridn(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

// threads of the J-plane reverse kernels
constexpr int RT_BS = 256;
// Cells (or nodes) per thread whose loads the J-plane reverse kernels issue
// together before the group's stores: a store keeps every later load of the
// thread behind it, so a one-at-a-time loop costs a memory round trip per
// cell.
constexpr int RT_U = 4;

__device__ __forceinline__ void aadd(float *p, float v) {
    if (v != 0.0f) atomicAdd(p, v);
}

// =====================================================================
// R1: primitive variables (k_prim)
// =====================================================================
__global__ void rk_prim(const Dev d, const Adj a) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, (size_t)n, i, j, k);
    if (j < 2) return;
    const float RRNOW = 1.0f / A2(d.R, j, k);
    const float ro = a.tRO[n], RECIP = 1.0f / ro;
    const float vx = a.tROVX[n] * RECIP, vr = a.tROVR[n] * RECIP;
    const float rovt = a.tRORVT[n] * RRNOW, vt = rovt * RECIP;
    float gvx = a.VX[n], gvr = a.VR[n], gvt = a.VT[n], grovt = a.ROVT[n];
    float gro = 0.0f, groe = 0.0f;
    if (j <= d.JMM1) {
        const float EKE = 0.5f * (vr * vr + vt * vt + vx * vx);
        const float TS = (a.tROE[n] / ro - EKE) / d.CV;
        const float gP = a.P[n], gHO = a.HO[n];
        const float gTS = gP * ro * d.RGAS + gHO * d.CP;
        gro += gP * d.RGAS * TS;
        const float gEKE = gHO - gTS / d.CV;
        groe += gTS / d.CV / ro;
        gro -= gTS / d.CV * a.tROE[n] / (ro * ro);
        gvr += gEKE * vr;
        gvt += gEKE * vt;
        gvx += gEKE * vx;
    }
    grovt += gvt * RECIP;
    float grecip = gvt * rovt + gvx * a.tROVX[n] + gvr * a.tROVR[n];
    gro -= grecip * RECIP * RECIP;
    a.v[V_RO].D[n] += gro;
    a.v[V_ROE].D[n] += groe;
    a.v[V_ROVX].D[n] += gvx * RECIP;
    a.v[V_ROVR].D[n] += gvr * RECIP;
    a.v[V_RORVT].D[n] += grovt * RRNOW;
    // cleared after the stores that use them (stores keep their order)
    if (j <= d.JMM1) {
        a.P[n] = 0.0f;
        a.HO[n] = 0.0f;
    }
    a.VX[n] = 0.0f;
    a.VR[n] = 0.0f;
    a.VT[n] = 0.0f;
    a.ROVT[n] = 0.0f;
}

// =====================================================================
// R2: mass fluxes (the mass part of k_flux_mass_energy)
// =====================================================================
// pre-step ROVT: J=1 from the previous inlet condition, J>=2 from k_prim
__device__ __forceinline__ float pre_rovt(const Dev &d, const Adj &a, int i, int j, int k) {
    return j == 1 ? AIK(a.tROVT1, i, k) : A3(a.tROVT, i, j, k);
}

__device__ __forceinline__ void rev_flowt_raw(const Dev &d, const Adj &a, int i, int j, int k, float g) {
    if (g == 0.0f) return;
    const float c = 0.25f * g;
    const float abx = A3(d.ABX, i, j, k), abt = A2(d.ABT, j, k), abr = A3(d.ABR, i, j, k);
    const int jj[4] = {j, j - 1, j - 1, j}, kk[4] = {k, k, k + 1, k + 1};
    float sx = 0.0f, st = 0.0f, sr = 0.0f;
    for (int q = 0; q < 4; ++q) {
        const int m = ix3(d, i, jj[q], kk[q]);
        aadd(&a.v[V_ROVX].D[m], c * abx);
        aadd(&a.ROVT[m], c * abt);
        aadd(&a.v[V_RO].D[m], -c * abt * A2(d.UBLADE, jj[q], kk[q]));
        aadd(&a.v[V_ROVR].D[m], c * abr);
        if (a.geom) {
            sx += a.tROVX[m];
            st += pre_rovt(d, a, i, jj[q], kk[q]) - A2(d.UBLADE, jj[q], kk[q]) * a.tRO[m];
            sr += a.tROVR[m];
        }
    }
    if (a.geom) {
        aadd(&A3(a.gABX, i, j, k), c * sx);
        aadd(&A2(a.gABT, j, k), c * st);
        aadd(&A3(a.gABR, i, j, k), c * sr);
    }
}

// Two passes like rk_flux_mom.  Coefficients cf[q * N + owner]: FLOWX q = 0, 1
// (ROVX, ROVR on the owner's K-face nodes), FLOWT q = 2..4 (ROVX; ROVT and
// -U RO from ABT; ROVR on its I-face nodes), FLOWR q = 5, 6 (ROVX, ROVR on
// its J-face nodes).  The periodic edge faces scatter with atomics.
__global__ void rk_flux_mass_coef(const Dev d, const Adj a) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, (size_t)n, i, j, k);
    const bool fx = i < d.IM && k < d.KM, ft = j >= 2 && k < d.KM, fr = i < d.IM && j >= 2;
    const bool end = i == 1 || i == d.IM;
    const bool edge = ft && end && A1(d.IND, j) != 1;
    bool on = ft && !edge;
    if (on && end) {
        const int nr = A1(d.NROW, j);
        if (k >= A1(d.KS1, nr) && k <= A1(d.KS2, nr)) on = false;
    }
    const bool rs = fr && k >= 2 && k <= d.KMM1;
    // every load before any store
    const float gx = fx ? a.FLOWX[n] : 0.0f, gt = ft ? a.FLOWT[n] : 0.0f, gr = rs ? a.FLOWR[n] : 0.0f;
    const float aqx = fx ? d.AQX[n] : 0.0f, aqr = fx ? d.AQR[n] : 0.0f;
    const float abx = on ? d.ABX[n] : 0.0f, abt = on ? A2(d.ABT, j, k) : 0.0f, abr = on ? d.ABR[n] : 0.0f;
    const float asx = rs ? d.ASX[n] : 0.0f, asr = rs ? d.ASR[n] : 0.0f;
    float c[7];
    c[0] = 0.25f * gx * aqx;
    c[1] = 0.25f * gx * aqr;
    c[2] = 0.25f * gt * abx;
    c[3] = 0.25f * gt * abt;
    c[4] = 0.25f * gt * abr;
    c[5] = 0.25f * gr * asx;
    c[6] = 0.25f * gr * asr;
    if (edge) {
        rev_flowt_raw(d, a, 1, j, k, 0.5f * gt);
        rev_flowt_raw(d, a, d.IM, j, k, 0.5f * gt);
    }
    if (a.geom) {
        if (fx && gx != 0.0f) {
            const int m[4] = {n, ix3(d, i, j, k + 1), ix3(d, i + 1, j, k), ix3(d, i + 1, j, k + 1)};
            float sx = 0.0f, sr = 0.0f;
            for (int q = 0; q < 4; ++q) {
                sx += a.tROVX[m[q]];
                sr += a.tROVR[m[q]];
            }
            aadd(&a.gAQX[n], 0.25f * gx * sx);
            aadd(&a.gAQR[n], 0.25f * gx * sr);
        }
        if (on && gt != 0.0f) {
            const int jj[4] = {j, j - 1, j - 1, j}, kk[4] = {k, k, k + 1, k + 1};
            float sx = 0.0f, st = 0.0f, sr = 0.0f;
            for (int q = 0; q < 4; ++q) {
                const int m = ix3(d, i, jj[q], kk[q]);
                sx += a.tROVX[m];
                st += pre_rovt(d, a, i, jj[q], kk[q]) - A2(d.UBLADE, jj[q], kk[q]) * a.tRO[m];
                sr += a.tROVR[m];
            }
            aadd(&a.gABX[n], 0.25f * gt * sx);
            aadd(&A2(a.gABT, j, k), 0.25f * gt * st);
            aadd(&a.gABR[n], 0.25f * gt * sr);
        }
        if (rs && gr != 0.0f) {
            const int m[4] = {n, ix3(d, i, j - 1, k), ix3(d, i + 1, j - 1, k), ix3(d, i + 1, j, k)};
            float sx = 0.0f, sr = 0.0f;
            for (int q = 0; q < 4; ++q) {
                sx += a.tROVX[m[q]];
                sr += a.tROVR[m[q]];
            }
            aadd(&a.gASX[n], 0.25f * gr * sx);
            aadd(&a.gASR[n], 0.25f * gr * sr);
        }
    }
    for (int q = 0; q < 7; ++q) a.cf[(size_t)q * N + n] = c[q];
}

__global__ void rk_flux_mass_gather(const Dev d, const Adj a) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, (size_t)n, i, j, k);
    const float *cf = a.cf;
    auto C = [&](int q, int o) { return cf[(size_t)q * N + o]; };
    float gX = 0.0f, gR = 0.0f, gT = 0.0f;
    for (int di = 0; di < 2; ++di)
        for (int dk = 0; dk < 2; ++dk) {
            const int ii = i - di, kk = k - dk;
            if (ii < 1 || kk < 1) continue;
            const int o = ix3(d, ii, j, kk);
            gX += C(0, o); gR += C(1, o);
        }
    for (int dj = 0; dj < 2; ++dj)
        for (int dk = 0; dk < 2; ++dk) {
            const int jj = j + dj, kk = k - dk;
            if (jj > d.JM || kk < 1) continue;
            const int o = ix3(d, i, jj, kk);
            gX += C(2, o); gT += C(3, o); gR += C(4, o);
        }
    for (int di = 0; di < 2; ++di)
        for (int dj = 0; dj < 2; ++dj) {
            const int ii = i - di, jj = j + dj;
            if (ii < 1 || jj > d.JM) continue;
            const int o = ix3(d, ii, jj, k);
            gX += C(5, o); gR += C(6, o);
        }
    float gRO = -gT * A2(d.UBLADE, j, k), gRV = gT;
    // WT = (ROVT - U RO) / RO of this node
    const float gw = a.WT[n];
    if (gw != 0.0f) {
        a.WT[n] = 0.0f;
        const float ro = a.tRO[n];
        gRV += gw / ro;
        gRO -= gw * pre_rovt(d, a, i, j, k) / (ro * ro);
    }
    a.v[V_ROVX].D[n] += gX;
    a.v[V_ROVR].D[n] += gR;
    a.ROVT[n] += gRV;
    a.v[V_RO].D[n] += gRO;
    // the face-flux adjoints rk_flux_mass_coef consumed (cleared here, not
    // there: see rk_flux_mom_gather)
    a.FLOWX[n] = 0.0f; a.FLOWT[n] = 0.0f; a.FLOWR[n] = 0.0f;
}

// =====================================================================
// R3: exit pitchwise sums and the radial-equilibrium recurrence (k_bc_sums)
// IPOUT = 0: PD(1) = PDOWN_HUB, PD(K) = 0.9 PD(K) + 0.1 (PD(K-1) + DP(K))
// =====================================================================
// One CTA of RBC_BS threads.  The recurrence runs on one thread over
// shared copies of PD's adjoint and R(JM, K), which all threads load first;
// the pitchwise part issues the loads of its RT_U points before their
// read-modify-writes.
constexpr int RBC_BS = 1024;
__global__ void __launch_bounds__(RBC_BS) rk_bc_sums(const Dev d, const Adj a) {
    __shared__ float gss[512], sr[512], gpd[512];
    const int KM = d.KM, IM = d.IM, IMM1 = d.IMM1;
    for (int k = threadIdx.x; k < KM; k += blockDim.x) {
        gss[k] = 0.0f;
        sr[k] = A2(d.R, d.JM, k + 1);
        gpd[k] = a.PD[k] + a.PDK[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = KM - 1; k >= 1; --k) {
            const float g = gpd[k];
            gpd[k - 1] += 0.1f * g;
            gpd[k] = 0.9f * g;
            const float gdp = 0.1f * g;
            const float half = 0.5f * (sr[k] - sr[k - 1]);
            gss[k] += gdp * half;
            gss[k - 1] += gdp * half;
        }
        gpd[0] = 0.0f;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < KM; k += blockDim.x) {
        a.PD[k] = gpd[k];
        a.PDK[k] = 0.0f;
    }
    const int np = IM * KM;
    for (int t0 = threadIdx.x; t0 < np; t0 += RT_U * RBC_BS) {
        float gP[RT_U], gR[RT_U], gV[RT_U], tvt[RT_U], trv[RT_U], w[RT_U], gpv[RT_U], rr[RT_U];
        int kk[RT_U];
#pragma unroll
        for (int u = 0; u < RT_U; ++u) {
            const int t = t0 + u * RBC_BS;
            kk[u] = -1;
            if (t < np) {
                const int i = t % IM + 1, k = t / IM + 1;
                kk[u] = k;
                w[u] = 0.5f * ((i <= IMM1 ? A1(d.FP, i) : 0.0f) + (i >= 2 ? A1(d.FP, i - 1) : 0.0f));
                gpv[u] = a.PAVG[k - 1];
                rr[u] = A2(d.R, d.JM, k);
                gP[u] = A3(a.P, i, d.JMM1, k);
                gR[u] = A3(a.ROVT, i, d.JM, k);
                gV[u] = A3(a.VT, i, d.JM, k);
                tvt[u] = A3(a.tVT, i, d.JM, k);
                trv[u] = A3(a.tROVT, i, d.JM, k);
            }
        }
#pragma unroll
        for (int u = 0; u < RT_U; ++u) {
            if (kk[u] < 0) continue;
            const int t = t0 + u * RBC_BS, i = t % IM + 1, k = kk[u];
            A3(a.P, i, d.JMM1, k) = gP[u] + gpv[u] * w[u];
            const float gs = gss[k - 1] * w[u] / rr[u];
            A3(a.ROVT, i, d.JM, k) = gR[u] + gs * tvt[u];
            A3(a.VT, i, d.JM, k) = gV[u] + gs * trv[u];
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < KM; k += blockDim.x) a.PAVG[k] = 0.0f;
}

// =====================================================================
// R4: energy fluxes (the energy part of k_flux_mass_energy); HO(JM) and PEFF as the step began
// =====================================================================
__device__ __forceinline__ float pre_ho(const Dev &d, const Adj &a, int i, int j, int k) {
    return j == d.JM ? AIK(a.tHOJM, i, k) : A3(a.tHO, i, j, k);
}

__device__ __forceinline__ void rev_tflux_energy_raw(const Dev &d, const Adj &a, int i, int j, int k, float g) {
    if (g == 0.0f) return;
    const float c = 0.25f * g;
    const int jj[4] = {j, j - 1, j - 1, j}, kk[4] = {k, k, k + 1, k + 1};
    float sho = 0.0f;
    const float ft = A3(a.tFLOWT, i, j, k), wr = A2(d.WRABT, j, k);
    for (int q = 0; q < 4; ++q) {
        const int m = ix3(d, i, jj[q], kk[q]);
        sho += pre_ho(d, a, i, jj[q], kk[q]);
        aadd(&a.HO[m], c * ft);
        aadd(&a.PEFF[m], c * wr);
    }
    aadd(&A3(a.FLOWT, i, j, k), c * sho);
}

// Two passes.  Coefficients cf[q * N + owner]: XFLUX q = 0 (HO on the K-face
// nodes), RFLUX q = 1 (HO on the J-face nodes), TFLUX q = 2, 3 (HO, PEFF on the
// I-face nodes); the periodic edge faces scatter with atomics.
__global__ void rk_flux_energy_coef(const Dev d, const Adj a) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, (size_t)n, i, j, k);
    const AdjVar &V = a.v[V_ROE];
    const bool fx = i < d.IM && k < d.KM, fr = i < d.IM && j >= 2, ft = j >= 2 && k < d.KM;
    const bool edge = ft && (i == 1 || i == d.IM) && A1(d.IND, j) != 1;
    const bool fi = ft && !edge;
    // every load before any store
    const float gx = fx ? V.XF[n] : 0.0f, gr = fr ? V.RF[n] : 0.0f, gt = ft ? V.TF[n] : 0.0f;
    const float FX = fx ? a.tFLOWX[n] : 0.0f, FR = fr ? a.tFLOWR[n] : 0.0f, FT = fi ? a.tFLOWT[n] : 0.0f;
    const float WR = fi ? A2(d.WRABT, j, k) : 0.0f;
    const float h000 = pre_ho(d, a, i, j, k);
    const float h001 = (fx || fi) ? pre_ho(d, a, i, j, k + 1) : 0.0f;
    const float h100 = (fx || fr) ? pre_ho(d, a, i + 1, j, k) : 0.0f;
    const float h101 = fx ? pre_ho(d, a, i + 1, j, k + 1) : 0.0f;
    const float h0m0 = (fr || fi) ? pre_ho(d, a, i, j - 1, k) : 0.0f;
    const float h1m0 = fr ? pre_ho(d, a, i + 1, j - 1, k) : 0.0f;
    const float h0m1 = fi ? pre_ho(d, a, i, j - 1, k + 1) : 0.0f;
    const float ax = fx ? a.FLOWX[n] : 0.0f, ar = fr ? a.FLOWR[n] : 0.0f, at = fi ? a.FLOWT[n] : 0.0f;
    float c[4];
    c[0] = gx * FX * 0.25f;
    c[1] = 0.25f * gr * FR;
    c[2] = 0.25f * gt * FT;
    c[3] = 0.25f * gt * WR;
    if (edge) {
        rev_tflux_energy_raw(d, a, 1, j, k, 0.5f * gt);
        rev_tflux_energy_raw(d, a, d.IM, j, k, 0.5f * gt);
    }
    if (fx) a.FLOWX[n] = ax + gx * (((h000 + h001) + h100) + h101) * 0.25f;
    if (fr) a.FLOWR[n] = ar + 0.25f * gr * (((h000 + h0m0) + h1m0) + h100);
    if (fi) a.FLOWT[n] = at + 0.25f * gt * (((h000 + h0m0) + h0m1) + h001);
    for (int q = 0; q < 4; ++q) a.cf[(size_t)q * N + n] = c[q];
}

__global__ void rk_flux_energy_gather(const Dev d, const Adj a) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, (size_t)n, i, j, k);
    const float *cf = a.cf;
    auto C = [&](int q, int o) { return cf[(size_t)q * N + o]; };
    float gH = 0.0f, gP = 0.0f;
    for (int di = 0; di < 2; ++di)
        for (int dk = 0; dk < 2; ++dk) {
            const int ii = i - di, kk = k - dk;
            if (ii < 1 || kk < 1) continue;
            gH += C(0, ix3(d, ii, j, kk));
        }
    for (int di = 0; di < 2; ++di)
        for (int dj = 0; dj < 2; ++dj) {
            const int ii = i - di, jj = j + dj;
            if (ii < 1 || jj > d.JM) continue;
            gH += C(1, ix3(d, ii, jj, k));
        }
    for (int dj = 0; dj < 2; ++dj)
        for (int dk = 0; dk < 2; ++dk) {
            const int jj = j + dj, kk = k - dk;
            if (jj > d.JM || kk < 1) continue;
            const int o = ix3(d, i, jj, kk);
            gH += C(2, o);
            gP += C(3, o);
        }
    a.HO[n] += gH;
    a.PEFF[n] += gP;
    const AdjVar &V = a.v[V_ROE];
    // the ROE flux adjoints rk_flux_energy_coef consumed (see rk_flux_mom_gather)
    V.XF[n] = 0.0f; V.RF[n] = 0.0f; V.TF[n] = 0.0f; V.SR[n] = 0.0f;
}

// =====================================================================
// R6: inlet and exit conditions (k_bc_apply), IN_PRESS = 0, IN_VTAN = 0,
// IN_VR <= 0
// =====================================================================
__global__ void rk_bc_apply(const Dev d, const Adj a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.IM * d.KM) return;
    const int i = t % d.IM + 1, k = t / d.IM + 1;
    // the exit's operands are loaded first: the inlet's stores below (other
    // addresses) would otherwise keep these loads behind them
    const int ne = ix3(d, i, d.JM, k);
    const float evr = a.tVR[ne], evt = a.tVT[ne], evx = a.tVX[ne], epe = a.tP[ne], ehoe = a.tHO[ne];
    const float eP = a.P[ne], eHO = a.HO[ne], eRO = a.v[V_RO].D[ne], eROE = a.v[V_ROE].D[ne];
    // ---- inlet ----
    {
        const float PO1 = A1(d.PO1, k), TO1 = A1(d.TO1, k);
        const float RO_STAG = PO1 / d.RGAS / TO1;
        float RO_IN = a.tROIN[t];
        const bool c0 = RO_IN > 0.9999f * RO_STAG;
        if (c0) RO_IN = 0.9999f * RO_STAG;
        const float PNEW = PO1 * powf(RO_IN / RO_STAG, d.GA);
        const float p1a = d.RFIN1 * a.tP1[t] + d.RFIN * PNEW;
        const float plim = A1(d.PLIM, k);
        const bool c1 = p1a > plim;
        const float p1b = c1 ? 0.9f * p1a + 0.1f * plim : p1a;
        const bool c2 = p1b > 0.99999f * PO1;
        const float p1 = c2 ? PO1 * 0.99999f : p1b;
        const float TS = TO1 * powf(p1 * A1(d.RPO1, k), d.FGA);
        const float VABSQ = 2.0f * d.CP * (TO1 - TS);
        const float VABS = sqrtf(VABSQ);
        const float VMER = VABS * A1(d.BSCOS, k);
        const float vt1 = VABS * A1(d.BSSIN, k);
        const float vr2 = A3(a.tVR, i, 2, k);
        float VXSQ = VMER * VMER - vr2 * vr2;
        const bool c3 = VXSQ < 0.0000001f * TO1 * d.CP;
        if (c3) VXSQ = 0.0000001f * TO1 * d.CP;
        const float vx1 = sqrtf(VXSQ), vr1 = vr2;
        const float ro1 = p1 / (d.RGAS * TS);
        const int n1 = ix3(d, i, 1, k);
        const float gROE = a.v[V_ROE].D[n1], gROVX = a.v[V_ROVX].D[n1], gRORVT = a.v[V_RORVT].D[n1];
        const float gROVR = a.v[V_ROVR].D[n1], gRO = a.v[V_RO].D[n1], gROVT = a.ROVT[n1];
        float gp1 = a.P[n1] + gROE / d.GA1;
        float gro1 = gROE * 0.5f * VABSQ + gROVX * vx1 + gROVR * vr1 + gRO;
        float gVABSQ = gROE * 0.5f * ro1;
        float gvx1 = gROVX * ro1 + a.VX[n1];
        float gvr1 = gROVR * ro1 + a.VR[n1];
        const float grovt1 = gRORVT * A2(d.R, 1, k) + gROVT;
        gro1 += grovt1 * vt1;
        const float gvt1 = grovt1 * ro1 + a.VT[n1];
        gp1 += gro1 / (d.RGAS * TS);
        float gTS = -gro1 * ro1 / TS;
        float gvr2 = gvr1;
        if (!c3) {
            const float gVXSQ = gvx1 * 0.5f / vx1;
            const float gVMER = gVXSQ * 2.0f * VMER;
            gvr2 -= gVXSQ * 2.0f * vr2;
            gVABSQ += (gvt1 * A1(d.BSSIN, k) + gVMER * A1(d.BSCOS, k)) * 0.5f / VABS;
        } else {
            gVABSQ += gvt1 * A1(d.BSSIN, k) * 0.5f / VABS;
        }
        gTS -= 2.0f * d.CP * gVABSQ;
        gp1 += gTS * TS * d.FGA / p1;
        const float gp1b = c2 ? 0.0f : gp1;
        const float gp1a = c1 ? 0.9f * gp1b : gp1b;
        const float gPNEW = d.RFIN * gp1a;
        const float gROIN = c0 ? 0.0f : gPNEW * PNEW * d.GA / RO_IN;
        a.v[V_RO].D[n1] = gROIN;
        a.P[n1] = d.RFIN1 * gp1a;
        A3(a.VR, i, 2, k) += gvr2;
        a.VX[n1] = 0.0f; a.VR[n1] = 0.0f; a.VT[n1] = 0.0f; a.ROVT[n1] = 0.0f; a.HO[n1] = 0.0f;
        a.v[V_ROVX].D[n1] = 0.0f; a.v[V_ROVR].D[n1] = 0.0f; a.v[V_RORVT].D[n1] = 0.0f; a.v[V_ROE].D[n1] = 0.0f;
    }
    // ---- exit ----
    {
        const float vr = evr, vt = evt, vx = evx;
        const float EKE = 0.5f * (vr * vr + vt * vt + vx * vx);
        const float pe = epe, hoe = ehoe;
        const float TEXIT = (hoe - EKE) / d.CP;
        const float roe_ = pe / d.RGAS / TEXIT;
        const float gP = eP, gHO = eHO, gRO = eRO, gROE = eROE;
        const float groe = gROE * (d.CV * TEXIT + EKE) + gRO;
        float gTEXIT = gROE * roe_ * d.CV - groe * roe_ / TEXIT;
        float gEKE = gROE * roe_ - gTEXIT / d.CP;
        const float ghoe = gTEXIT / d.CP + gHO;
        const float gpe = groe / (d.RGAS * TEXIT) + gP;
        A3(a.HO, i, d.JMM1, k) += 2.0f * ghoe;
        A3(a.HO, i, d.JM - 2, k) -= ghoe;
        atomicAdd(&a.PDK[k - 1], gpe);
        A3(a.P, i, d.JMM1, k) += d.FEXTRAP * gpe;
        atomicAdd(&a.PAVG[k - 1], -d.FEXTRAP * gpe);
        a.VR[ne] += gEKE * vr;
        a.VT[ne] += gEKE * vt;
        a.VX[ne] += gEKE * vx;
        a.P[ne] = 0.0f; a.HO[ne] = 0.0f; a.v[V_RO].D[ne] = 0.0f; a.v[V_ROE].D[ne] = 0.0f;
    }
}

// =====================================================================
// R7: PEFF = P - PREFF + F_PDOWN (P(J+1) - P)   (formed in k_flux_mom).
// Launched only for F_PDOWN != 0; with F_PDOWN = 0 rk_flux_mom_gather
// passes the adjoint to P itself.  The clearing store follows the atomics
// that use g, so it never meets the load of the same address in flight.
// =====================================================================
__global__ void rk_peff(const Dev d, const Adj a) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.IM * d.JM * d.KM;
    if (n >= N) return;
    const float g = a.PEFF[n];
    int i, j, k;
    node_ijk(d, (size_t)n, i, j, k);
    if (j == d.JM) {
        aadd(&a.P[n], g);
    } else {
        aadd(&a.P[n], (1.0f - d.F_PDOWN) * g);
        aadd(&A3(a.P, i, j + 1, k), d.F_PDOWN * g);
    }
    a.PEFF[n] = 0.0f;
}

// =====================================================================
// R8: momentum fluxes (k_flux_mom)
// =====================================================================
// the four nodes of a face I = const: (i,j,k), (i,j-1,k), (i,j-1,k+1), (i,j,k+1)
__device__ __forceinline__ void iface_nodes(const Dev &d, int i, int j, int k, int m[4]) {
    m[0] = ix3(d, i, j, k); m[1] = ix3(d, i, j - 1, k); m[2] = ix3(d, i, j - 1, k + 1); m[3] = ix3(d, i, j, k + 1);
}

// The periodic edge faces I = 1 and IM (IND != 1) of the momentum fluxes:
// both edge columns share one face, so the face's adjoints reach the nodes
// of both columns, with atomics.
__device__ __forceinline__ void rev_mom_iface_edge(const Dev &d, const Adj &a, int i, int j, int k, float gx,
                                                   float gt, float gr, float abx, float abt, float abr, float AVGR) {
    const int IM = d.IM;
    const float *PE = a.tPEFF, *VX = a.tVX, *VT = a.tVT, *VR = a.tVR;
    const int n = ix3(d, i, j, k);
    const float FT = a.tFLOWT[n];
    int m1[4], mm[4];
    iface_nodes(d, 1, j, k, m1);
    iface_nodes(d, IM, j, k, mm);
    if (gx != 0.0f) {
        float svx = 0.0f, sp = 0.0f;
        for (int q = 0; q < 4; ++q) {
            svx += VX[m1[q]] + VX[mm[q]];
            sp += PE[m1[q]] + PE[mm[q]];
            aadd(&a.VX[m1[q]], 0.125f * gx * FT);
            aadd(&a.VX[mm[q]], 0.125f * gx * FT);
            aadd(&a.PEFF[m1[q]], 0.125f * gx * abx);
            aadd(&a.PEFF[mm[q]], 0.125f * gx * abx);
        }
        aadd(&a.FLOWT[n], 0.125f * gx * svx);
        if (a.geom) aadd(&a.gABX[n], 0.125f * gx * sp);
    }
    if (gt != 0.0f) {
        auto rev_rvt = [&](int ii, const int *mq, float g) {
            const float ft = A3(a.tFLOWT, ii, j, k);
            float svt = 0.0f, sp = 0.0f;
            for (int q = 0; q < 4; ++q) {
                svt += VT[mq[q]];
                sp += PE[mq[q]];
                aadd(&a.VT[mq[q]], g * ft * AVGR);
                aadd(&a.PEFF[mq[q]], g * abt * AVGR);
            }
            aadd(&A3(a.FLOWT, ii, j, k), g * svt * AVGR);
            if (a.geom) aadd(&A2(a.gABT, j, k), g * sp * AVGR);
        };
        rev_rvt(1, m1, 0.5f * gt);
        rev_rvt(IM, mm, 0.5f * gt);
    }
    if (gr != 0.0f) {
        const float f1 = A3(a.tFLOWT, 1, j, k), fm = A3(a.tFLOWT, IM, j, k);
        float svr1 = 0.0f, svrm = 0.0f, sp = 0.0f;
        for (int q = 0; q < 4; ++q) {
            svr1 += VR[m1[q]];
            svrm += VR[mm[q]];
            sp += PE[m1[q]] + PE[mm[q]];
            aadd(&a.VR[m1[q]], 0.125f * gr * f1);
            aadd(&a.VR[mm[q]], 0.125f * gr * fm);
            aadd(&a.PEFF[m1[q]], 0.125f * gr * abr);
            aadd(&a.PEFF[mm[q]], 0.125f * gr * abr);
        }
        aadd(&A3(a.FLOWT, 1, j, k), 0.125f * gr * svr1);
        aadd(&A3(a.FLOWT, IM, j, k), 0.125f * gr * svrm);
        if (a.geom) aadd(&a.gABR[n], 0.125f * gr * sp);
    }
}

// Two passes.  rk_flux_mom_coef: each face owner turns its flux adjoints into
// one coefficient per (face, input array) -- every node of a face gets the
// same one -- and adds its own FLOWX/FLOWR/FLOWT and geometry adjoints.
// rk_flux_mom_gather: each node sums the coefficients of the faces and cells
// it belongs to.  Only the periodic edge faces (I = 1, IM with IND != 1),
// which reach both edge columns, scatter with atomics.
// Coefficients, cf[q * N + owner]: K faces q = 0..3 (PEFF, VX, VT, VR), J faces
// 4..7 (same), radial source 8..10 (ROVT, VT, PEFF), I faces 11..14 (VX, PEFF,
// VT, VR).
// The coefficient passes issue every load before their first store and
// branch on no loaded value, and they clear none of the adjoints they read:
// the gathers clear them.  Clearing in place (a store of a constant right
// after the load of the same address) made these passes 6-12 times slower
// than their gathers, with the warps stalled on long-scoreboard waits at a
// small fraction of the memory bandwidth; moving the clears took the whole
// transposed step of the 65 x 242 x 49 stage from 0.86 to 0.60 ms.
constexpr int MOM_NCOEF = 15;

__global__ void rk_flux_mom_coef(const Dev d, const Adj a) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, (size_t)n, i, j, k);
    const int IM = d.IM;
    const bool hi = i < IM, hj = j >= 2, hk = k < d.KM;
    const bool fk = hi && hk, fj = hi && hj, fs = fj && hk, ft = hj && hk;
    const AdjVar &X = a.v[V_ROVX], &T = a.v[V_RORVT], &Rm = a.v[V_ROVR];
    const float *PE = a.tPEFF, *VX = a.tVX, *VT = a.tVT, *VR = a.tVR, *RV = a.tROVT;
    const bool edge = ft && (i == 1 || i == IM) && A1(d.IND, j) != 1;
    const bool fi = ft && !edge;
    // every load before any store: the flux adjoints, then the recorded
    // values on the cube (i..i+1, j-1..j, k..k+1); index [di][dj + 1][dk]
    const float gxk = fk ? X.XF[n] : 0.0f, gtk = fk ? T.XF[n] : 0.0f, grk = fk ? Rm.XF[n] : 0.0f;
    const float gxj = fj ? X.RF[n] : 0.0f, gtj = fj ? T.RF[n] : 0.0f, grj = fj ? Rm.RF[n] : 0.0f;
    const float gxi = ft ? X.TF[n] : 0.0f, gti = ft ? T.TF[n] : 0.0f, gri = ft ? Rm.TF[n] : 0.0f;
    const float gs = fs ? Rm.SR[n] : 0.0f;
    float pe[2][2][2], vx[2][2][2], vt[2][2][2], vr[2][2][2], rv[2][2][2];
#pragma unroll
    for (int di = 0; di < 2; ++di)
#pragma unroll
        for (int dj = 0; dj < 2; ++dj)
#pragma unroll
            for (int dk = 0; dk < 2; ++dk) {
                const bool ok = (di == 0 || hi) && (dj == 1 || hj) && (dk == 0 || hk);
                const int o = ok ? ix3(d, i + di, j + dj - 1, k + dk) : n;
                pe[di][dj][dk] = ok ? PE[o] : 0.0f;
                vx[di][dj][dk] = ok ? VX[o] : 0.0f;
                vt[di][dj][dk] = ok ? VT[o] : 0.0f;
                vr[di][dj][dk] = ok ? VR[o] : 0.0f;
                rv[di][dj][dk] = (ok && fs) ? RV[o] : 0.0f;
            }
    const float fxw = fk ? a.tFLOWX[n] : 0.0f, frw = fj ? a.tFLOWR[n] : 0.0f, FT = fi ? a.tFLOWT[n] : 0.0f;
    const float rjk = A2(d.R, j, k);
    const float rk1 = fk ? A2(d.R, j, k + 1) : 0.0f, rj1 = fj ? A2(d.R, j - 1, k) : 0.0f;
    const float aqx = fk ? d.AQX[n] : 0.0f, aqr = fk ? d.AQR[n] : 0.0f;
    const float asx = fj ? d.ASX[n] : 0.0f, asr = fj ? d.ASR[n] : 0.0f;
    const float vol = fs ? d.VOLOR[n] : 0.0f;
    const float abx = ft ? d.ABX[n] : 0.0f, abr = ft ? d.ABR[n] : 0.0f, abt = ft ? A2(d.ABT, j, k) : 0.0f;
    const float ravg = ft ? A2(d.RAVG_CELL, j, k) : 0.0f;
    const float ofx = fk ? a.FLOWX[n] : 0.0f, ofr = fj ? a.FLOWR[n] : 0.0f, oft = fi ? a.FLOWT[n] : 0.0f;
    float c[MOM_NCOEF];
    // faces K = const: nodes (i,j,k), (i,j,k+1), (i+1,j,k+1), (i+1,j,k)
    {
        const float sp = ((pe[0][1][0] + pe[0][1][1]) + pe[1][1][1]) + pe[1][1][0];
        const float svx = ((vx[0][1][0] + vx[0][1][1]) + vx[1][1][1]) + vx[1][1][0];
        const float svt = ((vt[0][1][0] + vt[0][1][1]) + vt[1][1][1]) + vt[1][1][0];
        const float svr = ((vr[0][1][0] + vr[0][1][1]) + vr[1][1][1]) + vr[1][1][0];
        const float AVGR = 0.125f * (rjk + rk1);
        c[0] = 0.25f * gxk * aqx + 0.25f * grk * aqr;
        c[1] = 0.25f * gxk * fxw;
        c[2] = gtk * fxw * AVGR;
        c[3] = 0.25f * grk * fxw;
        if (fk) {
            a.FLOWX[n] = ofx + (0.25f * gxk * svx + gtk * AVGR * svt + 0.25f * grk * svr);
            if (a.geom) {
                a.gAQX[n] += 0.25f * gxk * sp;
                a.gAQR[n] += 0.25f * grk * sp;
            }
        }
    }
    // faces J = const: nodes (i,j,k), (i,j-1,k), (i+1,j-1,k), (i+1,j,k)
    {
        const float sp = ((pe[0][1][0] + pe[0][0][0]) + pe[1][0][0]) + pe[1][1][0];
        const float svx = ((vx[0][1][0] + vx[0][0][0]) + vx[1][0][0]) + vx[1][1][0];
        const float svt = ((vt[0][1][0] + vt[0][0][0]) + vt[1][0][0]) + vt[1][1][0];
        const float svr = ((vr[0][1][0] + vr[0][0][0]) + vr[1][0][0]) + vr[1][1][0];
        const float AVGR = (rjk + rj1) * 0.125f;
        c[4] = 0.25f * gxj * asx + 0.25f * grj * asr;
        c[5] = 0.25f * gxj * frw;
        c[6] = gtj * frw * AVGR;
        c[7] = 0.25f * grj * frw;
        if (fj) {
            a.FLOWR[n] = ofr + (0.25f * gxj * svx + gtj * svt * AVGR + 0.25f * grj * svr);
            if (a.geom) {
                a.gASX[n] += 0.25f * gxj * sp;
                a.gASR[n] += 0.25f * grj * sp;
            }
        }
    }
    // radial source: the cell cube, summed in (di, dj, dk) order
    {
        float srv = 0.0f, svt8 = 0.0f, sp8 = 0.0f;
#pragma unroll
        for (int di = 0; di < 2; ++di)
#pragma unroll
            for (int dj = 0; dj < 2; ++dj)
#pragma unroll
                for (int dk = 0; dk < 2; ++dk) {
                    srv += rv[di][dj][dk];
                    svt8 += vt[di][dj][dk];
                    sp8 += pe[di][dj][dk];
                }
        const float AVGVT8 = 0.125f * svt8;
        c[8] = -gs * vol * AVGVT8;
        c[9] = -gs * vol * srv * 0.125f;
        c[10] = -gs * vol;
        if (fs && a.geom && gs != 0.0f) a.gVOLOR[n] += -gs * (srv * AVGVT8 + sp8);
    }
    // faces I = const: nodes (i,j,k), (i,j-1,k), (i,j-1,k+1), (i,j,k+1)
    {
        const float AVGR = 0.25f * ravg;
        const float svx = ((vx[0][1][0] + vx[0][0][0]) + vx[0][0][1]) + vx[0][1][1];
        const float svt = ((vt[0][1][0] + vt[0][0][0]) + vt[0][0][1]) + vt[0][1][1];
        const float svr = ((vr[0][1][0] + vr[0][0][0]) + vr[0][0][1]) + vr[0][1][1];
        const float sp = ((pe[0][1][0] + pe[0][0][0]) + pe[0][0][1]) + pe[0][1][1];
        c[11] = 0.25f * gxi * FT;
        c[12] = 0.25f * gxi * abx + gti * abt * AVGR + 0.25f * gri * abr;
        c[13] = gti * FT * AVGR;
        c[14] = 0.25f * gri * FT;
        if (fi) {
            a.FLOWT[n] = oft + (0.25f * gxi * svx + gti * svt * AVGR + 0.25f * gri * svr);
            if (a.geom) {
                a.gABX[n] += 0.25f * gxi * sp;
                a.gABR[n] += 0.25f * gri * sp;
                aadd(&A2(a.gABT, j, k), gti * sp * AVGR);
            }
        } else {
            c[11] = c[12] = c[13] = c[14] = 0.0f;
        }
        if (edge) rev_mom_iface_edge(d, a, i, j, k, gxi, gti, gri, abx, abt, abr, AVGR);
    }
    for (int q = 0; q < MOM_NCOEF; ++q) a.cf[(size_t)q * N + n] = c[q];
}

__global__ void rk_flux_mom_gather(const Dev d, const Adj a) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, (size_t)n, i, j, k);
    const float *cf = a.cf;
    auto C = [&](int q, int o) { return cf[(size_t)q * N + o]; };
    float gP = 0.0f, gVX = 0.0f, gVT = 0.0f, gVR = 0.0f, gRV = 0.0f;
    for (int di = 0; di < 2; ++di)
        for (int dk = 0; dk < 2; ++dk) {
            const int ii = i - di, kk = k - dk;
            if (ii < 1 || kk < 1) continue;
            const int o = ix3(d, ii, j, kk);       // K face of owner (ii, j, kk)
            gP += C(0, o); gVX += C(1, o); gVT += C(2, o); gVR += C(3, o);
        }
    for (int di = 0; di < 2; ++di)
        for (int dj = 0; dj < 2; ++dj) {
            const int ii = i - di, jj = j + dj;
            if (ii < 1 || jj > d.JM) continue;
            const int o = ix3(d, ii, jj, k);       // J face of owner (ii, jj, k)
            gP += C(4, o); gVX += C(5, o); gVT += C(6, o); gVR += C(7, o);
            for (int dk = 0; dk < 2; ++dk) {
                const int kk = k - dk;
                if (kk < 1) continue;
                const int o2 = ix3(d, ii, jj, kk); // radial-source cell of owner (ii, jj, kk)
                gRV += C(8, o2); gVT += C(9, o2); gP += C(10, o2);
            }
        }
    for (int dj = 0; dj < 2; ++dj)
        for (int dk = 0; dk < 2; ++dk) {
            const int jj = j + dj, kk = k - dk;
            if (jj > d.JM || kk < 1) continue;
            const int o = ix3(d, i, jj, kk);       // I face of owner (i, jj, kk)
            gVX += C(11, o); gP += C(12, o); gVT += C(13, o); gVR += C(14, o);
        }
    const bool peff_here = d.F_PDOWN == 0.0f;
    if (peff_here)
        a.P[n] += a.PEFF[n] + gP;   // PEFF = P - PREFF: its whole adjoint is P's
    else
        a.PEFF[n] += gP;            // rk_peff distributes it over P(J) and P(J+1)
    a.VX[n] += gVX;
    a.VT[n] += gVT;
    a.VR[n] += gVR;
    a.ROVT[n] += gRV;
    // clear the adjoints that rk_flux_mom_coef consumed.  Stored here, and
    // not where they were read: a store of a constant to an address whose
    // load is still in flight stalls that kernel's warps for a long time.
    if (peff_here) a.PEFF[n] = 0.0f;
    const AdjVar *W = &a.v[V_ROVX];
    for (int v = 0; v < 3; ++v) {
        const AdjVar &V = W[v];
        V.XF[n] = 0.0f; V.RF[n] = 0.0f; V.TF[n] = 0.0f; V.SR[n] = 0.0f;
    }
}

// =====================================================================
// R11: mixing plane (k_mixplan), subsonic relative flow at JP2: the outputs
// at (I, JP2) depend on the 14 inputs (IMID, JP1) x 5, (I, JP2) x 5 and
// (I, JP3) x 4, differentiated in forward mode with 14-component duals
// =====================================================================
template <int N>
struct Dual {
    float v;
    float g[N];
    __device__ Dual() : v(0.0f) {
        for (int q = 0; q < N; ++q) g[q] = 0.0f;
    }
    __device__ Dual(float x) : v(x) {
        for (int q = 0; q < N; ++q) g[q] = 0.0f;
    }
};
template <int N> __device__ inline Dual<N> lin(float v, const Dual<N> &x, float dx) {
    Dual<N> r(v);
    for (int q = 0; q < N; ++q) r.g[q] = dx * x.g[q];
    return r;
}
template <int N> __device__ inline Dual<N> lin2(float v, const Dual<N> &x, float dx, const Dual<N> &y, float dy) {
    Dual<N> r(v);
    for (int q = 0; q < N; ++q) r.g[q] = dx * x.g[q] + dy * y.g[q];
    return r;
}
template <int N> __device__ inline Dual<N> operator+(const Dual<N> &x, const Dual<N> &y) { return lin2(x.v + y.v, x, 1.0f, y, 1.0f); }
template <int N> __device__ inline Dual<N> operator-(const Dual<N> &x, const Dual<N> &y) { return lin2(x.v - y.v, x, 1.0f, y, -1.0f); }
template <int N> __device__ inline Dual<N> operator*(const Dual<N> &x, const Dual<N> &y) { return lin2(x.v * y.v, x, y.v, y, x.v); }
template <int N> __device__ inline Dual<N> operator/(const Dual<N> &x, const Dual<N> &y) {
    const float q = x.v / y.v;
    return lin2(q, x, 1.0f / y.v, y, -q / y.v);
}
template <int N> __device__ inline Dual<N> operator*(float c, const Dual<N> &x) { return lin(c * x.v, x, c); }
template <int N> __device__ inline Dual<N> operator*(const Dual<N> &x, float c) { return lin(c * x.v, x, c); }
template <int N> __device__ inline Dual<N> operator/(const Dual<N> &x, float c) { return lin(x.v / c, x, 1.0f / c); }
template <int N> __device__ inline Dual<N> operator-(const Dual<N> &x, float c) { return lin(x.v - c, x, 1.0f); }
template <int N> __device__ inline Dual<N> operator+(const Dual<N> &x, float c) { return lin(x.v + c, x, 1.0f); }
template <int N> __device__ inline Dual<N> operator-(float c, const Dual<N> &x) { return lin(c - x.v, x, -1.0f); }
template <int N> __device__ inline Dual<N> dsqrt(const Dual<N> &x) {
    const float s = sqrtf(x.v);
    return lin(s, x, s > 0.0f ? 0.5f / s : 0.0f);
}
template <int N> __device__ inline Dual<N> dasin(const Dual<N> &x) { return lin(asinf(x.v), x, rsqrtf(1.0f - x.v * x.v)); }
template <int N> __device__ inline Dual<N> datan2(const Dual<N> &y, const Dual<N> &x) {
    const float r2 = x.v * x.v + y.v * y.v;
    return lin2(atan2f(y.v, x.v), y, x.v / r2, x, -y.v / r2);
}
template <int N> __device__ inline Dual<N> dpowc(const Dual<N> &x, float e) {
    const float p = powf(x.v, e);
    return lin(p, x, e * p / x.v);
}
template <int N> __device__ inline Dual<N> dsin(const Dual<N> &x) { return lin(sinf(x.v), x, cosf(x.v)); }
template <int N> __device__ inline Dual<N> dcos(const Dual<N> &x) { return lin(cosf(x.v), x, -sinf(x.v)); }

constexpr int MIXN = 14;

__global__ void __launch_bounds__(64) rk_mixplan(const Dev d, const Adj a) {
    typedef Dual<MIXN> D;
    __shared__ float red[5][64];
    const int nr = blockIdx.x / d.KM + 1, k = blockIdx.x % d.KM + 1;
    const int IM = d.IM;
    const float RFMIX1 = 1.0f - d.RFMIX;
    const int KSUB = (k == d.KM) ? d.KM - 1 : k;
    int j = A1(d.JMIX, nr);
    int JP1, JP2, JP3;
    float F_ANGLE;
    if (A3(a.tFLOWX, d.IMID, j, KSUB) < 0.0f) {
        JP1 = j + 1; JP2 = j + 2; JP3 = j + 3;
        F_ANGLE = d.FANGLE;
    } else {
        j = A1(d.JMIX, nr) + 1;
        JP1 = j - 1; JP2 = j - 2; JP3 = j - 3;
        F_ANGLE = 0.0f;
    }
    const float F_ANGLE1 = 1.0f - F_ANGLE;
    const float *rec = a.tMIX + (size_t)blockIdx.x * mix_rec_size(IM);
    float gacc[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    for (int i = threadIdx.x + 1; i <= IM; i += blockDim.x) {
        const float *q = rec + 5 + 10 * (i - 1);
        D x[MIXN];
        for (int c = 0; c < 5; ++c) x[c] = D(rec[c]);
        for (int c = 0; c < 5; ++c) x[5 + c] = D(q[c]);
        for (int c = 0; c < 4; ++c) x[10 + c] = D(q[5 + c]);
        for (int c = 0; c < MIXN; ++c) x[c].g[c] = 1.0f;
        const float RJP1 = A2(d.R, JP1, k), UJP1 = A2(d.UBLADE, JP1, k);
        const D ROMIX = x[0];
        const D VXMIX = x[1] / ROMIX;
        const D VRMIX = x[2] / ROMIX;
        const D VTMIX = x[3] / ROMIX / RJP1;
        const D ROEMIX = x[4];
        const D VMSQ = VXMIX * VXMIX + VRMIX * VRMIX;
        const D VABSQ = VMSQ + VTMIX * VTMIX;
        const D WTMIX = VTMIX - UJP1;
        const D WMIXSQ = VMSQ + WTMIX * WTMIX;
        const D WMIX = dsqrt(WMIXSQ);
        const D ALPHAMIX = dasin(WTMIX / WMIX);
        const D GAMAMIX = datan2(VRMIX, VXMIX);
        const D TMIX = (ROEMIX / ROMIX - 0.5f * VABSQ) / d.CV;
        const D ROTHALPY = d.CP * TMIX + 0.5f * (WMIXSQ - UJP1 * UJP1);
        const D PMIX = ROMIX * d.RGAS * TMIX;
        const float RJP2 = A2(d.R, JP2, k), UNOWJP2 = A2(d.UBLADE, JP2, k);
        const float RJP3 = A2(d.R, JP3, k), UNOWJP3 = A2(d.UBLADE, JP3, k);
        const D ROJP2 = x[5];
        const D XVELJP2 = x[6] / ROJP2;
        const D RVELJP2 = x[7] / ROJP2;
        const D TVELJP2 = x[8] / RJP2 / ROJP2;
        const D WTJP2 = TVELJP2 - UNOWJP2;
        const D VMSQJP2 = XVELJP2 * XVELJP2 + RVELJP2 * RVELJP2;
        const D VELSQJP2 = VMSQJP2 + TVELJP2 * TVELJP2;
        const D WACT_SQ_JP2 = VMSQJP2 + WTJP2 * WTJP2;
        const D WACT_JP2 = dsqrt(WACT_SQ_JP2);
        const D T_ACT_JP2 = (x[9] / ROJP2 - 0.5f * VELSQJP2) / d.CV;
        const D ROJP3 = x[10];
        const D ROVXJP3 = x[11], ROVRJP3 = x[12];
        const D ROVTJP3 = x[13] / RJP3;
        const D ROWTJP3 = ROVTJP3 - UNOWJP3 * ROJP3;
        const D ROWRELSQJP3 = ROVXJP3 * ROVXJP3 + ROVRJP3 * ROVRJP3 + ROWTJP3 * ROWTJP3;
        const D ROWRELJP3 = dsqrt(ROWRELSQJP3);
        const D ALPHAJP3 = dasin(ROWTJP3 / ROWRELJP3);
        const D GAMAJP3 = datan2(ROVRJP3, ROVXJP3);
        const D PSTAT = ROJP2 * d.RGAS * T_ACT_JP2;
        const D TISENT = TMIX * dpowc(PSTAT / PMIX, d.FGA);
        D WIS_SQ = 2.0f * (ROTHALPY - d.CP * TISENT + 0.5f * UNOWJP2 * UNOWJP2);
        const D ROISENT = PSTAT / d.RGAS / TISENT;
        if (WIS_SQ.v < 1.0f) WIS_SQ = D(1.0f);
        const D WIS = dsqrt(WIS_SQ);
        const float wm = WACT_JP2.v / sqrtf(d.GA * d.RGAS * T_ACT_JP2.v);
        if (wm > 1.0f) atomicOr(a.flag, 1);
        const D ALPHAA = F_ANGLE1 * ALPHAMIX + F_ANGLE * ALPHAJP3;
        const D GAMA = F_ANGLE1 * GAMAMIX + F_ANGLE * GAMAJP3;
        const D WT_JP2 = WIS * dsin(ALPHAA);
        const D VM_JP2 = WIS * dcos(ALPHAA);
        const D VX_JP2 = VM_JP2 * dcos(GAMA);
        const D VR_JP2 = VM_JP2 * dsin(GAMA);
        const D VT_JP2 = WT_JP2 + UNOWJP2;
        const D V_SQ = VM_JP2 * VM_JP2 + VT_JP2 * VT_JP2;
        const D ROE_JP2 = ROISENT * (d.CV * TISENT + 0.5f * V_SQ);
        D out[5];
        out[0] = RFMIX1 * x[5] + d.RFMIX * ROISENT;
        out[1] = RFMIX1 * x[6] + d.RFMIX * (ROISENT * VX_JP2);
        out[2] = RFMIX1 * x[7] + d.RFMIX * (ROISENT * VR_JP2);
        out[3] = RFMIX1 * x[8] + d.RFMIX * (ROISENT * VT_JP2 * RJP2);
        out[4] = RFMIX1 * x[9] + d.RFMIX * ROE_JP2;
        // adjoints: the output order of the state variables is RO, ROVX, ROVR, RORVT, ROE
        const int n2 = ix3(d, i, JP2, k), n3 = ix3(d, i, JP3, k);
        float *A[5] = {a.v[V_RO].D, a.v[V_ROVX].D, a.v[V_ROVR].D, a.v[V_RORVT].D, a.v[V_ROE].D};
        float go[5];
        for (int c = 0; c < 5; ++c) go[c] = A[c][n2];
        float gin[MIXN];
        for (int q = 0; q < MIXN; ++q) {
            float s = 0.0f;
            for (int c = 0; c < 5; ++c) s += go[c] * out[c].g[q];
            gin[q] = s;
        }
        for (int c = 0; c < 5; ++c) gacc[c] += gin[c];
        for (int c = 0; c < 5; ++c) A[c][n2] = gin[5 + c];
        for (int c = 0; c < 4; ++c) A[c][n3] += gin[10 + c];
    }
    for (int c = 0; c < 5; ++c) red[c][threadIdx.x] = gacc[c];
    __syncthreads();
    if (threadIdx.x < 5) {
        float s = 0.0f;
        for (int t = 0; t < (int)blockDim.x; ++t) s += red[threadIdx.x][t];
        const int n1 = ix3(d, d.IMID, JP1, k);
        float *A[5] = {a.v[V_RO].D, a.v[V_ROVX].D, a.v[V_ROVR].D, a.v[V_RORVT].D, a.v[V_ROE].D};
        atomicAdd(&A[threadIdx.x][n1], s);
    }
}

// =====================================================================
// R10: the density limiter (k_density_fix) and the Mach limiter
// (k_mach_limiter), with the limits VLIMIT/ROLIMIT of each row held at the
// recorded step's values.  Where the density limiter acts,
// lim(J) = C0(J) RO(J) + CA(J) ROAVG(J), ROAVG = (lim(J-2) + lim(J-1) +
// RO(J+1) + RO(J+2)) / 4, J walked upwards; the coefficients come from a
// replay of the recorded column (rk_density_prep).
// =====================================================================
__global__ void rk_density_prep(const Dev d, const Adj a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.IM * d.KM) return;
    const int i = t % d.IM + 1, k = t / d.IM + 1;
    float *C0 = const_cast<float *>(a.tDC0), *CA = const_cast<float *>(a.tDCA);
    int any = 0;
    const float *RO = a.tROL;
    float rm2 = A3(RO, i, 1, k), rm1 = A3(RO, i, 2, k), r0 = A3(RO, i, 3, k), rp1 = A3(RO, i, 4, k);
    for (int j = 3; j <= d.JM - 3; ++j) {
        const float rp2 = A3(RO, i, j + 2, k);
        const float ROAVG = 0.25f * (rm2 + rm1 + rp1 + rp2);
        float ro = r0, c0 = 1.0f, ca = 0.0f;
        if (ro < 0.6f * ROAVG) { ro = 0.5f * (ro + 0.6f * ROAVG); c0 *= 0.5f; ca = 0.5f * ca + 0.3f; }
        if (ro > 1.5f * ROAVG) { ro = 0.5f * (ro + 1.5f * ROAVG); c0 *= 0.5f; ca = 0.5f * ca + 0.75f; }
        if (ro < d.ROLIM) { ro = 0.5f * (ro + d.ROLIM); c0 *= 0.5f; ca *= 0.5f; }
        if (c0 != 1.0f) any = 1;
        A3(C0, i, j, k) = c0;
        A3(CA, i, j, k) = ca;
        rm2 = rm1;
        rm1 = ro;
        r0 = rp1;
        rp1 = rp2;
    }
    const_cast<int *>(a.tDCOL)[t] = any;
}

__global__ void rk_density(const Dev d, const Adj a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.IM * d.KM || !a.tDCOL[t]) return;
    const int i = t % d.IM + 1, k = t / d.IM + 1;
    float *aRO = a.v[V_RO].D;
    for (int j = d.JM - 3; j >= 3; --j) {
        const float g = A3(aRO, i, j, k);
        A3(aRO, i, j, k) = A3(a.tDC0, i, j, k) * g;
        const float q = 0.25f * A3(a.tDCA, i, j, k) * g;
        if (q == 0.0f) continue;
        A3(aRO, i, j - 1, k) += q;
        A3(aRO, i, j - 2, k) += q;
        A3(aRO, i, j + 1, k) += q;
        A3(aRO, i, j + 2, k) += q;
    }
}

__global__ void rk_mach(const Dev d, const Adj a) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, (size_t)n, i, j, k);
    const int nr = A1(d.NROW, j);
    const float VL = a.tVLIM[nr - 1], ROL = a.tROLIM[nr - 1];
    const float ro_in = a.tROM[n];
    const bool clamp = ro_in < ROL;
    const float ro = clamp ? ROL : ro_in;
    const float vx = a.tVX[n], vr = a.tVR[n], wt = a.tWT[n];
    const float WRELSQ = vx * vx + vr * vr + wt * wt;
    const float F = VL / sqrtf(WRELSQ);
    float *aRO = a.v[V_RO].D;
    if (F < 1.0f) {
        const float gX = a.v[V_ROVX].D[n], gR = a.v[V_ROVR].D[n], gT = a.v[V_RORVT].D[n];
        const float gROVT = a.ROVT[n] + gT * A2(d.R, j, k);
        const float gro = aRO[n] + (gX * vx + gR * vr + gROVT * wt) * F + gROVT * A2(d.UBLADE, j, k);
        const float gF = (gX * vx + gR * vr + gROVT * wt) * ro;
        a.VX[n] += gX * ro * F - gF * F * vx / WRELSQ;
        a.VR[n] += gR * ro * F - gF * F * vr / WRELSQ;
        a.WT[n] += gROVT * ro * F - gF * F * wt / WRELSQ;
        a.v[V_ROVX].D[n] = 0.0f;
        a.v[V_ROVR].D[n] = 0.0f;
        a.v[V_RORVT].D[n] = 0.0f;
        a.ROVT[n] = 0.0f;
        aRO[n] = clamp ? 0.0f : gro;
    } else if (clamp) {
        aRO[n] = 0.0f;
    }
}

// =====================================================================
// TSTEP, reversed: rk_ts_smooth (SMOOTH_VAR and the averaging fix-ups) ->
// rk_ts_gather (corner gather, second mixing-plane average, negative
// feedback) -> rk_ts_damp (the row-mean term of the negative feedback, the
// restriction partials) -> rk_ts_cells (prolongation, mixing-plane
// redistribution, SCREE, flux sum)
// =====================================================================

__device__ inline int mp_role_r(const Dev &d, int j, int *nr) {
    for (int r = 1; r <= d.NRWSM1; ++r) {
        int jx = A1(d.JMIX, r);
        if (j == jx) { *nr = r; return 1; }
        if (j == jx + 1) { *nr = r; return 2; }
        if (j == jx + 2) { *nr = r; return 3; }
    }
    *nr = 0;
    return 0;
}
__device__ inline int stream_case_r(const Dev &d, int j) {
    int nr = A1(d.NROW, j);
    int J1 = A1(d.JSTART, nr), J2 = A1(d.JMIX, nr);
    int sc = 0;
    if (j >= J1 + 3 && j <= J2 - 3) sc = 1;
    if (j == J2) sc = 0;
    if (j == J1) sc = 0;
    if (j == J1 + 2) sc = 2;
    if (j == J1 + 1) sc = 3;
    if (j == J2 - 2) sc = 4;
    if (j == J2 - 1) sc = 5;
    return sc;
}
__device__ inline int le_case_r(const Dev &d, int j) {
    int lc = 0;
    for (int r = 1; r <= d.NROWS; ++r) {
        int JL = A1(d.JLED, r);
        if (j == JL - 2 || j == JL - 1) lc = 1;
        if (j == JL) lc = 2;
    }
    return lc;
}
// the mixing-plane row of cell plane jc at K is averaged (1750, 1850)
__device__ inline bool mp_row_on(const Dev &d, const Adj &a, int role, int mnr, int k) {
    const bool lowx = d.FEXTRAP < 0.001f;
    const float FLOWDIRN = -A3(a.tFLOWX, d.IMID, A1(d.JMIX, mnr), k);
    return role == 3 ? (FLOWDIRN > 0.0f || lowx) : (FLOWDIRN < 0.0f || lowx);
}

__global__ void __launch_bounds__(RT_BS) rk_ts_smooth(const __grid_constant__ Dev d, const __grid_constant__ Adj a, int v0) {
    extern __shared__ float sm[];
    const AdjVar &V = a.v[v0 + blockIdx.y];
    const int IM = d.IM, KM = d.KM, IMM1 = d.IMM1, KMM1 = d.KMM1;
    const int np = IM * KM;
    float *A_ = sm, *B_ = sm + np, *C_ = sm + 2 * np;
    const int j = blockIdx.x + 1;
    const DevCtl *c = a.tctl;
    const size_t ks = (size_t)IM * d.JM;
#define P(buf, i, k) buf[((i) - 1) + IM * ((k) - 1)]
    for (int t = threadIdx.x; t < np; t += RT_BS) {
        const int i = t % IM + 1, k = t / IM + 1;
        A_[t] = A3(V.D, i, j, k);
    }
    __syncthreads();
    // mixing-plane average of the variable (100)
    bool mp = false;
    if (d.IFMIX != 0)
        for (int r = 1; r <= d.NRWSM1; ++r)
            if (j == A1(d.JMIX, r) || j == A1(d.JMIX, r) + 1) mp = true;
    if (mp) {
        for (int k = threadIdx.x + 1; k <= KM; k += RT_BS) {
            float s = 0.0f;
            for (int i = 1; i <= IM; ++i) s += P(A_, i, k);
            B_[k - 1] = s;
        }
        __syncthreads();
        for (int t = threadIdx.x; t < np; t += RT_BS) {
            const int i = t % IM + 1, k = t / IM + 1;
            A_[t] = 0.5f * B_[k - 1] * ((i <= IMM1 ? A1(d.FP, i) : 0.0f) + (i >= 2 ? A1(d.FP, i - 1) : 0.0f));
        }
        __syncthreads();
    }
    // tip-gap and periodic averaging of I=1 and I=IM (510, 8000)
    const bool periodic_j = !(A1(d.IND, j) == 1 || A1(d.INDLE, j) == 1);
    {
        int nr = A1(d.NROW, j);
        int K1 = A1(d.KTIPS, nr), K2 = A1(d.KTIPE, nr);
        const bool tip = K1 > 0;
        if (tip) {
            if (K1 == 1) K2 = K2 - 1;
            if (K2 == KM) K1 = K1 + 1;
        }
        for (int k = threadIdx.x + 1; k <= KM; k += RT_BS) {
            if (tip && k >= K1 && k <= K2) {
                float v = 0.5f * (P(A_, 1, k) + P(A_, IM, k));
                P(A_, 1, k) = v;
                P(A_, IM, k) = v;
            }
            if (periodic_j) {
                float v = 0.5f * (P(A_, 1, k) + P(A_, IM, k));
                P(A_, 1, k) = v;
                P(A_, IM, k) = v;
            }
        }
        __syncthreads();
    }
    if (!(d.SFEXIT < 0.0001f) && j >= d.JM + 1 - d.NSFEXIT) {
        // exit smoothing is rejected when the adjoint is prepared
    }
    if (j >= 2 && !(c->SFT < 0.0001f)) {
        const float SFT = c->SFT, SFT1 = c->SFT1, SFTH = c->SFTH, F4 = d.FAC_4TH;
        // corners
        float cv = 0.0f;
        if (threadIdx.x < 4) {
            const int ci = (threadIdx.x & 1) ? IM : 1, ck = (threadIdx.x & 2) ? KM : 1;
            cv = P(A_, ci, ck);
        }
        __syncthreads();
        if (threadIdx.x < 4) {
            const int ci = (threadIdx.x & 1) ? IM : 1, ck = (threadIdx.x & 2) ? KM : 1;
            const int ni = ci == 1 ? 2 : IMM1, nk = ck == 1 ? 2 : KMM1;
            P(A_, ci, ck) = SFT1 * cv;
            P(A_, ni, ck) += SFTH * cv;
            P(A_, ci, nk) += SFTH * cv;
        }
        __syncthreads();
        // The spanwise pass (b -> a, per I column) and the pitchwise pass
        // (a -> b, per K line) reversed in gather form: each point sums the
        // terms of the outputs that read it, so no shared-memory atomics.
        // Curvatures first: c(m) = x(m) - FD(m) x(m+1) - FU(m) x(m-1) for an
        // interior m, read by the smoothed values at m-1 and m+1.
        const float h = SFT * F4;
        // spanwise: A_ = adjoint of its output; B_ = curvature adjoints
        for (int t = threadIdx.x; t < np; t += RT_BS) {
            const int i = t % IM + 1, k = t / IM + 1;
            float cb = 0.0f;
            if (k >= 2 && k <= KMM1) {
                if (k + 1 <= KMM1) cb += A1(d.FKU, k + 1) * P(A_, i, k + 1);
                if (k - 1 >= 2) cb += A1(d.FKD, k - 1) * P(A_, i, k - 1);
            }
            B_[t] = h * cb;
        }
        __syncthreads();
        // C_ = adjoint of the pitchwise output
        for (int t = threadIdx.x; t < np; t += RT_BS) {
            const int i = t % IM + 1, k = t / IM + 1;
            float g = SFT1 * P(A_, i, k);
            if (k - 1 >= 2 && k - 1 <= KMM1) g += SFT * A1(d.FKD, k - 1) * P(A_, i, k - 1);
            if (k + 1 >= 2 && k + 1 <= KMM1) g += SFT * A1(d.FKU, k + 1) * P(A_, i, k + 1);
            if (k == 2) g += SFT * P(A_, i, 1) * (1.0f + 0.5f * A1(d.FKU, 1));
            if (k == 3) g -= SFT * P(A_, i, 1) * 0.5f * A1(d.FKU, 1);
            if (k == KMM1) g += SFT * P(A_, i, KM) * (1.0f + 0.5f * A1(d.FKU, KM));
            if (k == d.KMM2) g -= SFT * P(A_, i, KM) * 0.5f * A1(d.FKU, KM);
            if (k >= 2 && k <= KMM1) g += P(B_, i, k);
            if (k - 1 >= 2 && k - 1 <= KMM1) g -= A1(d.FKD, k - 1) * P(B_, i, k - 1);
            if (k + 1 >= 2 && k + 1 <= KMM1) g -= A1(d.FKU, k + 1) * P(B_, i, k + 1);
            C_[t] = g;
        }
        __syncthreads();
        // pitchwise: C_ = adjoint of its output; B_ = curvature adjoints, the
        // end curvature c(1) = c(IM) = a(1) - (a(2) + a(IMM1))/2 of a periodic
        // plane at I = 1 and IM
        for (int t = threadIdx.x; t < np; t += RT_BS) {
            const int i = t % IM + 1, k = t / IM + 1;
            float cb = 0.0f;
            if (i >= 2 && i <= IMM1) {
                if (i + 1 <= IMM1) cb += A1(d.FU, i + 1) * P(C_, i + 1, k);
                if (i - 1 >= 2) cb += A1(d.FD, i - 1) * P(C_, i - 1, k);
            } else if (periodic_j) {
                if (i == 1 && IMM1 >= 2) cb += A1(d.FU, 2) * P(C_, 2, k);
                if (i == IM && IMM1 >= 2) cb += A1(d.FD, IMM1) * P(C_, IMM1, k);
            }
            if (periodic_j) {
                const float e = 0.5f * (P(C_, 1, k) + P(C_, IM, k));
                if (i == 2) cb += e;
                if (i == IMM1) cb += e;
            }
            B_[t] = h * cb;
        }
        __syncthreads();
        for (int t = threadIdx.x; t < np; t += RT_BS) {
            const int i = t % IM + 1, k = t / IM + 1;
            float g = SFT1 * P(C_, i, k);
            if (i - 1 >= 2 && i - 1 <= IMM1) g += SFT * A1(d.FD, i - 1) * P(C_, i - 1, k);
            if (i + 1 >= 2 && i + 1 <= IMM1) g += SFT * A1(d.FU, i + 1) * P(C_, i + 1, k);
            if (periodic_j) {
                const float e = 0.5f * SFT * (P(C_, 1, k) + P(C_, IM, k));
                if (i == 2) g += e;
                if (i == IMM1) g += e;
            } else {
                if (i == 2) g += SFT * P(C_, 1, k) * (1.0f + A1(d.FU, 1));
                if (i == 3) g -= SFT * P(C_, 1, k) * A1(d.FU, 1);
                if (i == IMM1) g += SFT * P(C_, IM, k) * (1.0f + A1(d.FU, IM));
                if (i == d.IMM2) g -= SFT * P(C_, IM, k) * A1(d.FU, IM);
            }
            if (i >= 2 && i <= IMM1) g += P(B_, i, k);
            if (i - 1 >= 2 && i - 1 <= IMM1) g -= A1(d.FD, i - 1) * P(B_, i - 1, k);
            if (i + 1 >= 2 && i + 1 <= IMM1) g -= A1(d.FU, i + 1) * P(B_, i + 1, k);
            if (periodic_j) {
                const float e = P(B_, 1, k) + P(B_, IM, k);
                if (i == 1) g += e;
                if (i == 2) g -= 0.5f * e;
                if (i == IMM1) g -= 0.5f * e;
            }
            A_[t] = g;
        }
        __syncthreads();
    }
    // streamwise and leading-edge smoothing: scatter into TMP's adjoint
    const bool stream = !(c->SFX < 0.0001f);
    const int sc = stream ? stream_case_r(d, j) : 0;
    const int lc = stream ? le_case_r(d, j) : 0;
    const int nr = A1(d.NROW, j);
    const int J1 = A1(d.JSTART, nr), J2 = A1(d.JMIX, nr);
    const float SFX = c->SFX, SFX1 = c->SFX1, SFXB = c->SFXB, SFXB1 = c->SFXB1, SFXBH = c->SFXBH;
    const float SFXHM1 = c->SFXHM1, SFX14 = c->SFX14, F4 = d.FAC_4TH;
    int nq = 0, jq[4] = {0, 0, 0, 0};
    float cq[4] = {0.0f, 0.0f, 0.0f, 0.0f}, c0 = 1.0f;
    auto addq = [&](int jj, float cc) { jq[nq] = jj; cq[nq] = cc; ++nq; };
    switch (sc) {
    case 1:
        c0 = SFX1 - 0.5f * SFX * F4;
        addq(j + 1, 0.5f * SFX * (1.0f + F4)); addq(j - 1, 0.5f * SFX * (1.0f + F4));
        addq(j - 2, -0.25f * SFX * F4); addq(j + 2, -0.25f * SFX * F4);
        break;
    case 2: c0 = SFXB1; addq(J1 + 3, SFXBH); addq(J1 + 1, SFXBH); break;
    case 3: c0 = SFXB1; addq(J1 + 2, 1.25f * SFXB); addq(J1 + 3, 0.5f * SFXB); addq(J1 + 4, -0.75f * SFXB); break;
    case 4: c0 = SFXB1; addq(J2 - 1, SFXBH); addq(J2 - 3, SFXBH); break;
    case 5: c0 = SFXB1; addq(J2 - 2, 1.25f * SFXB); addq(J2 - 3, 0.5f * SFXB); addq(J2 - 4, -0.75f * SFXB); break;
    default: break;
    }
    for (int t = threadIdx.x; t < np; t += RT_BS) {
        const int i = t % IM + 1, k = t / IM + 1;
        const float g = A_[t];
        if (g == 0.0f) continue;
        float *tm = V.TM + (size_t)(i - 1) + ks * (k - 1);     // tm[IM*(jj-1)] = TMP(i, jj, k)
        if (lc && (i == 1 || i == IM)) {
            aadd(&tm[(size_t)IM * (j - 1)], SFXHM1 * g);
            float *tk = V.TM + ks * (k - 1) + (size_t)IM * (j - 1);   // tk[x] = TMP(x+1, j, k)
            if (lc == 1) {
                aadd(&tk[1], SFX14 * g);
                aadd(&tk[IMM1 - 1], SFX14 * g);
            } else if (i == 1) {
                aadd(&tk[IM], SFX14 * g);
                aadd(&tk[IM - 1], SFX14 * g);
            } else {
                aadd(&tk[IM + IM - 1], SFX14 * g);
                aadd(&tk[0], SFX14 * g);
            }
            continue;
        }
        aadd(&tm[(size_t)IM * (j - 1)], c0 * g);
        for (int q = 0; q < nq; ++q) aadd(&tm[(size_t)IM * (jq[q] - 1)], cq[q] * g);
    }
#undef P
}

__global__ void __launch_bounds__(RT_BS) rk_ts_gather(const __grid_constant__ Dev d, const __grid_constant__ Adj a, int v0) {
    extern __shared__ float sm[];
    __shared__ double shd[RT_BS / 32];
    const AdjVar &V = a.v[v0 + blockIdx.y];
    const int IM = d.IM, IMM1 = d.IMM1, KMM1 = d.KMM1;
    const int j = blockIdx.x + 1;
    // the variable's own adjoint: D = TMP + gather, so dJ/dD(old) = dJ/dTMP
    {
        const int np = IM * d.KM;
        for (int t0 = threadIdx.x; t0 < np; t0 += RT_U * RT_BS) {
            float v[RT_U];
            int o[RT_U];
#pragma unroll
            for (int u = 0; u < RT_U; ++u) {
                const int t = t0 + u * RT_BS;
                o[u] = -1;
                if (t < np) {
                    o[u] = ix3(d, t % IM + 1, j, t / IM + 1);
                    v[u] = V.TM[o[u]];
                }
            }
#pragma unroll
            for (int u = 0; u < RT_U; ++u)
                if (o[u] >= 0) V.D[o[u]] = v[u];
        }
    }
    if (j < 2) return;
    const int jc = j;
    const int nc = IMM1 * KMM1;
    float *av = sm;
    const float fdn = A1(d.FACDWN, jc), fup = A1(d.FACUP, jc);
    // RT_U cells at a time, their loads issued together
    for (int c0 = threadIdx.x; c0 < nc; c0 += RT_U * RT_BS) {
        float tA[RT_U][4], tB[RT_U][4], wt[RT_U][4];
#pragma unroll
        for (int u = 0; u < RT_U; ++u) {
            const int c = c0 + u * RT_BS;
            if (c >= nc) continue;
            const int i = c % IMM1 + 1, k = c / IMM1 + 1;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int ii = i + (q & 1), kk = k + (q >> 1);   // (i,k) (i+1,k) (i,k+1) (i+1,k+1)
                tA[u][q] = A3(V.TM, ii, jc, kk);
                tB[u][q] = A3(V.TM, ii, jc - 1, kk);
            }
            wt[u][0] = AIK(d.FBL, i, k);
            wt[u][1] = AIK(d.FBR, i, k);
            wt[u][2] = AIK(d.FTL, i, k);
            wt[u][3] = AIK(d.FTR, i, k);
        }
#pragma unroll
        for (int u = 0; u < RT_U; ++u) {
            const int c = c0 + u * RT_BS;
            if (c >= nc) continue;
            float s = wt[u][0] * (fdn * tA[u][0] + fup * tB[u][0]);
            s += wt[u][1] * (fdn * tA[u][1] + fup * tB[u][1]);
            s += wt[u][2] * (fdn * tA[u][2] + fup * tB[u][2]);
            s += wt[u][3] * (fdn * tA[u][3] + fup * tB[u][3]);
            av[c] = s;
        }
    }
    __syncthreads();
    // second mixing-plane average (1850): a row set to its mean
    int mnr;
    const int role = mp_role_r(d, jc, &mnr);
    if (role == 1 || role == 3) {
        for (int k = threadIdx.x + 1; k <= KMM1; k += RT_BS) {
            if (!mp_row_on(d, a, role, mnr, k)) continue;
            float *row = av + (size_t)(k - 1) * IMM1;
            float s = 0.0f;
            for (int i = 0; i < IMM1; ++i) s += row[i];
            s = s / (float)IMM1;
            for (int i = 0; i < IMM1; ++i) row[i] = s;
        }
        __syncthreads();
    }
    // negative feedback v = S / (1 + |S| / (blk DAMP)): dv/dS = 1/(1+q)^2,
    // dv/dblk = S q / (blk (1+q)^2); the blk term is summed per plane
    const DevCtl *ctl = a.tctl;
    const int damp_on = ctl->damp_on;
    const float DAMP = ctl->DAMP;
    const float blk = damp_on ? V.tBLK[A1(d.NROW, jc) - 1] : 1.0f;
    float pbf = 0.0f;             // FP32 per thread, FP64 across threads
    for (int c0 = threadIdx.x; c0 < nc; c0 += RT_U * RT_BS) {
        float S[RT_U];
        int o[RT_U];
#pragma unroll
        for (int u = 0; u < RT_U; ++u) {
            const int c = c0 + u * RT_BS;
            o[u] = -1;
            S[u] = 0.0f;
            if (c < nc) {
                o[u] = ix3(d, c % IMM1 + 1, jc, c / IMM1 + 1);
                if (damp_on) S[u] = V.tST[o[u]];
            }
        }
#pragma unroll
        for (int u = 0; u < RT_U; ++u) {
            if (o[u] < 0) continue;
            const float g = av[c0 + u * RT_BS];
            float out = g;
            if (damp_on) {
                const float q = fabsf(S[u]) / (blk * DAMP);
                const float r = 1.0f / (1.0f + q);
                out = g * r * r;
                pbf += g * S[u] * q / blk * r * r;
            }
            V.ST[o[u]] = out;
        }
    }
    double pb = (double)pbf;
    for (int o = 16; o > 0; o >>= 1) pb += __shfl_down_sync(0xffffffffu, pb, o);
    if ((threadIdx.x & 31) == 0) shd[threadIdx.x >> 5] = pb;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < RT_BS / 32; ++w) s += shd[w];
        V.pblk[jc - 1] = s;
    }
}

__global__ void __launch_bounds__(RT_BS) rk_ts_damp(const __grid_constant__ Dev d, const __grid_constant__ Adj a, int v0) {
    __shared__ double shd[RT_BS / 32];
    __shared__ float gchg[64], gblk[64];
    const AdjVar &V = a.v[v0 + blockIdx.y];
    const int IMM1 = d.IMM1, KMM1 = d.KMM1;
    const int j = blockIdx.x + 2;
    const int nc = IMM1 * KMM1;
    const DevCtl *ctl = a.tctl;
    const int NROWS = d.NROWS;
    float add = 0.0f;
    if (ctl->damp_on) {
        // dJ/dblk per row, then through the row mixing to dJ/dchg
        // one warp per row, its lanes over the J planes (a serial walk over
        // all planes by one thread per row was a chain of dependent loads)
        {
            const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
            for (int nr = w + 1; nr <= NROWS; nr += RT_BS / 32) {
                double s = 0.0;
                for (int jj = 2 + l; jj <= d.JM; jj += 32)
                    if (A1(d.NROW, jj) == nr) s += V.pblk[jj - 1];
                for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
                if (l == 0) {
                    gblk[nr - 1] = (float)s;
                    gchg[nr - 1] = 0.0f;
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            if (NROWS == 1) gchg[0] = gblk[0];
            if (NROWS == 2) {
                const float g = gblk[0] + gblk[1];
                gchg[0] = 0.5f * g;
                gchg[1] = 0.5f * g;
            }
            if (NROWS > 2) {
                for (int nr = 2; nr <= NROWS - 1; ++nr) {
                    const float g = gblk[nr - 1];
                    gchg[nr - 2] += 0.25f * g;
                    gchg[nr] += 0.25f * g;
                    gchg[nr - 1] += 0.5f * g;
                }
                gchg[NROWS - 2] += 0.5f * gblk[NROWS - 1];
                gchg[NROWS - 1] += 0.5f * gblk[NROWS - 1];
                gchg[0] += 0.5f * gblk[0];
                gchg[1] += 0.5f * gblk[0];
            }
        }
        __syncthreads();
        for (int nr = 1; nr <= NROWS; ++nr) {
            const int JST = A1(d.JSTART, nr) + 1, JEN = A1(d.JMIX, nr) - 1;
            if (j >= JST && j <= JEN) add = gchg[nr - 1] / (float)(IMM1 * KMM1 * (JEN - JST + 1));
        }
    }
    float psf = 0.0f;             // FP32 per thread, FP64 across threads
    for (int c0 = threadIdx.x; c0 < nc; c0 += RT_U * RT_BS) {
        float g[RT_U], ts[RT_U], rsp[RT_U];
        int o[RT_U];
#pragma unroll
        for (int u = 0; u < RT_U; ++u) {
            const int c = c0 + u * RT_BS;
            o[u] = -1;
            if (c < nc) {
                const int n = ix3(d, c % IMM1 + 1, j, c / IMM1 + 1);
                o[u] = n;
                g[u] = V.ST[n];
                ts[u] = add != 0.0f ? V.tST[n] : 0.0f;
                rsp[u] = d.RSTEP[n];
            }
        }
#pragma unroll
        for (int u = 0; u < RT_U; ++u) {
            if (o[u] < 0) continue;
            float gg = g[u];
            if (add != 0.0f) gg += (ts[u] < 0.0f ? -add : add);
            V.ST[o[u]] = gg;
            const float y = gg * rsp[u];
            V.Y[o[u]] = y;
            psf += y;
        }
    }
    __shared__ df shdf[RT_BS / 32];
    df ps = df_of(psf);
    for (int o = 16; o > 0; o >>= 1) ps = df_add(ps, df_shfl_down(ps, o));
    if ((threadIdx.x & 31) == 0) shdf[threadIdx.x >> 5] = ps;
    __syncthreads();
    if (threadIdx.x == 0) {
        df s = df_of(0.0f);
        for (int w = 0; w < RT_BS / 32; ++w) s = df_add(s, shdf[w]);
        V.psum[j - 1] = s;
    }
    // level-1 and level-2 partial sums of Y over this plane
    const int n1 = d.NIB1 * d.NKB1, n2 = d.NIB2 * d.NKB2;
    for (int t = threadIdx.x; t < n1 + n2; t += RT_BS) {
        const bool lv1 = t < n1;
        const int u = lv1 ? t : t - n1;
        const int nib = lv1 ? d.NIB1 : d.NIB2;
        const int ib = u % nib + 1, kb = u / nib + 1;
        const int i0 = lv1 ? A1(d.IB1_S, ib) : A1(d.IB2_S, ib), i1 = lv1 ? A1(d.IB1_E, ib) : A1(d.IB2_E, ib);
        const int k0 = lv1 ? A1(d.KB1_S, kb) : A1(d.KB2_S, kb), k1 = lv1 ? A1(d.KB1_E, kb) : A1(d.KB2_E, kb);
        float s = 0.0f;
        for (int k = k0; k <= k1; ++k)
            for (int i = i0; i <= i1; ++i) s += A3(V.Y, i, j, k);
        if (lv1) V.P1[(size_t)(j - 1) * n1 + u] = s;
        else V.P2[(size_t)(j - 1) * n2 + u] = s;
    }
}

__global__ void __launch_bounds__(RT_BS) rk_ts_cells(const __grid_constant__ Dev d, const __grid_constant__ Adj a, int v0) {
    extern __shared__ float sm[];
    __shared__ float s_sb;
    const AdjVar &V = a.v[v0 + blockIdx.y];
    const int IM = d.IM, IMM1 = d.IMM1, KMM1 = d.KMM1;
    const int j = blockIdx.x + 2;
    const int nc = IMM1 * KMM1;
    const int n1 = d.NIB1 * d.NKB1, n2 = d.NIB2 * d.NKB2;
    float *b1 = sm, *b2 = sm + n1, *st = sm + n1 + n2, *rs = st + nc;
    const int j1 = A1(d.JB1, j), j2 = A1(d.JB2, j), jsb = A1(d.JSBLK, j);
    const size_t m1 = (size_t)d.NIB1 * (d.NJB1 + 1), m2 = (size_t)d.NIB2 * (d.NJB2 + 1);
    for (int t = threadIdx.x; t < n1; t += RT_BS) {
        float s = 0.0f;
        if (j1 <= d.NJB1)
            for (int jj = A1(d.JB1_START, j1); jj <= A1(d.JB1_END, j1); ++jj) s += V.P1[(size_t)(jj - 1) * n1 + t];
        b1[t] = s;
    }
    for (int t = threadIdx.x; t < n2; t += RT_BS) {
        float s = 0.0f;
        if (j2 <= d.NJB2)
            for (int jj = A1(d.JB2_START, j2); jj <= A1(d.JB2_END, j2); ++jj) s += V.P2[(size_t)(jj - 1) * n2 + t];
        b2[t] = s;
    }
    if (threadIdx.x < 32) {
        const int a0 = A1(d.SB_START, jsb), b0 = A1(d.SB_END, jsb);
        df s = df_of(0.0f);
        for (int jj = a0 + (int)threadIdx.x; jj <= b0; jj += 32) s = df_add(s, V.psum[jj - 1]);
        for (int o = 16; o > 0; o >>= 1) s = df_add(s, df_shfl_down(s, o));
        if (threadIdx.x == 0) s_sb = df_val(s);
    }
    __syncthreads();
    const float SB = s_sb, SSB = A1(d.STEPSBK, jsb);
    // RT_U cells at a time: their block indices, then their operands, are
    // loaded together
    for (int c0 = threadIdx.x; c0 < nc; c0 += RT_U * RT_BS) {
        int i1[RT_U], i2[RT_U], k1[RT_U], k2[RT_U], nn[RT_U];
        float vs[RT_U], vp[RT_U], v1[RT_U], v2[RT_U];
#pragma unroll
        for (int u = 0; u < RT_U; ++u) {
            const int c = c0 + u * RT_BS;
            if (c >= nc) continue;
            const int i = c % IMM1 + 1, k = c / IMM1 + 1;
            nn[u] = ix3(d, i, j, k);
            i1[u] = A1(d.IB1, i); i2[u] = A1(d.IB2, i); k1[u] = A1(d.KB1, k); k2[u] = A1(d.KB2, k);
        }
#pragma unroll
        for (int u = 0; u < RT_U; ++u) {
            const int c = c0 + u * RT_BS;
            if (c >= nc) continue;
            const size_t s1 = (size_t)(i1[u] - 1) + (size_t)d.NIB1 * (j1 - 1) + m1 * (k1[u] - 1);
            const size_t s2 = (size_t)(i2[u] - 1) + (size_t)d.NIB2 * (j2 - 1) + m2 * (k2[u] - 1);
            vs[u] = V.ST[nn[u]];
            vp[u] = d.STEP[nn[u]];
            v1[u] = d.STEP1[s1];
            v2[u] = d.STEP2[s2];
        }
#pragma unroll
        for (int u = 0; u < RT_U; ++u) {
            const int c = c0 + u * RT_BS;
            if (c >= nc) continue;
            st[c] = vs[u] * vp[u] + b1[(k1[u] - 1) * d.NIB1 + (i1[u] - 1)] * v1[u] +
                    b2[(k2[u] - 1) * d.NIB2 + (i2[u] - 1)] * v2[u] + SB * SSB;
        }
    }
    __syncthreads();
    // mixing-plane pitchwise redistribution (1750): row <- (sum of row) FP(I)
    int mnr;
    const int role = mp_role_r(d, j, &mnr);
    if (role == 1 || role == 3) {
        for (int k = threadIdx.x + 1; k <= KMM1; k += RT_BS) {
            if (!mp_row_on(d, a, role, mnr, k)) continue;
            float *row = st + (size_t)(k - 1) * IMM1;
            float s = 0.0f;
            for (int i = 1; i <= IMM1; ++i) s += row[i - 1] * A1(d.FP, i);
            for (int i = 0; i < IMM1; ++i) row[i] = s;
        }
        __syncthreads();
    }
    // SCREE: STORE = F1 DELTA + F2 DIFF, DIFF = DELTA + F3 DIFF; then the flux sum
    const float RATPITCH = (float)A1(d.NBLADE, j - 1) / (float)A1(d.NBLADE, j);
    const int nr = A1(d.NROW, j);
    const int kts = A1(d.KTIPS, nr), kte = A1(d.KTIPE, nr);
    const bool lowx = d.FEXTRAP < 0.001f;
    const int jmx = role ? A1(d.JMIX, mnr) : 0;
    const float F1 = d.F1, F2 = d.F2, F3 = d.F3;
    for (int k = threadIdx.x; k < KMM1; k += RT_BS) rs[k] = 0.0f;
    __syncthreads();
    // the cell body; gdiff is the cell's DIFF adjoint, loaded with those of
    // the other cells of its group
    auto cell = [&](int c, int i, int k, int n, float gdiff) {
        const float gst = st[c];
        const float gdelta = F1 * gst + gdiff;
        V.DIFF[n] = F2 * gst + F3 * gdiff;
        if (gdelta == 0.0f) return;
        aadd(&V.XF[n], gdelta);
        aadd(&A3(V.XF, i, j - 1, k), -RATPITCH * gdelta);
        aadd(&V.RF[n], gdelta);
        aadd(&A3(V.RF, i, j, k + 1), -gdelta);
        const bool gap = kts > 0 && k >= kts && k <= kte - 1;
        // t0 = TF(i): the tip-gap mean of TF(1) and TF(IM) at i = 1
        if (gap && i == 1) {
            aadd(&A3(V.TF, 1, j, k), 0.5f * gdelta);
            aadd(&A3(V.TF, IM, j, k), 0.5f * gdelta);
        } else {
            aadd(&V.TF[n], gdelta);
        }
        // t1 = TF(i+1): the mean at i+1 = IM
        if (gap && i + 1 == IM) {
            aadd(&A3(V.TF, 1, j, k), -0.5f * gdelta);
            aadd(&A3(V.TF, IM, j, k), -0.5f * gdelta);
        } else {
            aadd(&A3(V.TF, i + 1, j, k), -gdelta);
        }
        // source: -src
        const float gsrc = -gdelta;
        bool plain = true;
        if (role && !lowx) {
            const float FLOWDIRN = -A3(a.tFLOWX, d.IMID, jmx, k);
            if (role == 1 && FLOWDIRN > 0.0f) {
                // src = SR - (XF(i,j-1) - lsum FP(i)) FEXTRAP, lsum = sum_i XF(i,j-1)
                aadd(&A3(V.XF, i, j - 1, k), -gsrc * d.FEXTRAP);
                atomicAdd(&rs[k - 1], gsrc * d.FEXTRAP * A1(d.FP, i));
            }
            if (role == 2) plain = false;
            if (role == 3 && !(FLOWDIRN > 0.0f)) {
                aadd(&V.XF[n], gsrc * d.FEXTRAP);
                atomicAdd(&rs[k - 1], -gsrc * d.FEXTRAP * A1(d.FP, i));
            }
        }
        if (plain) aadd(&V.SR[n], gsrc);
    };
    for (int c0 = threadIdx.x; c0 < nc; c0 += RT_U * RT_BS) {
        float gd[RT_U];
        int o[RT_U];
#pragma unroll
        for (int u = 0; u < RT_U; ++u) {
            const int c = c0 + u * RT_BS;
            o[u] = -1;
            if (c < nc) {
                o[u] = ix3(d, c % IMM1 + 1, j, c / IMM1 + 1);
                gd[u] = V.DIFF[o[u]];
            }
        }
#pragma unroll
        for (int u = 0; u < RT_U; ++u) {
            const int c = c0 + u * RT_BS;
            if (o[u] >= 0) cell(c, c % IMM1 + 1, c / IMM1 + 1, o[u], gd[u]);
        }
    }
    __syncthreads();
    if (role == 1 || role == 3) {
        const int jj = role == 1 ? j - 1 : j;
        for (int c = threadIdx.x; c < nc; c += RT_BS) {
            const int i = c % IMM1 + 1, k = c / IMM1 + 1;
            aadd(&A3(V.XF, i, jj, k), rs[k - 1]);
        }
    }
}

// objective seeds added at the start of each reverse step
__global__ void rk_seed(const Dev d, const Adj a) {
    const int IM = d.IM, KM = d.KM;
    const int np = IM * KM, nc = d.IMM1 * d.KMM1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int per = 5 * np + nc;
    if (t >= 2 * per || !*a.seed_on) return;
    const int p = t / per, r = t % per;
    const int j = a.seed_j[p];
    const float s = a.seed[t];
    if (s == 0.0f) return;
    if (r < 5 * np) {
        const int q = r / np, u = r % np;
        const int i = u % IM + 1, k = u / IM + 1;
        float *A[5] = {a.VX, a.VT, a.VR, a.HO, a.P};
        A3(A[q], i, j, k) += s;
    } else {
        const int u = r - 5 * np;
        const int i = u % d.IMM1 + 1, k = u / d.IMM1 + 1;
        A3(a.FLOWX, i, j, k) += s;
    }
}

// objective seeds of the EFICOOL mass averages on plane j (FP64 weights
// from the host): dJ/dspo, dJ/dsto, dJ/dbf
__global__ void rk_seed_plane(const Dev d, const Adj a, float *seed, int j,
                              double gspo, double gsto, double gbf, double spo, double sto, double bf) {
    const int IM = d.IM, KM = d.KM, IMM1 = d.IMM1, KMM1 = d.KMM1;
    const int np = IM * KM;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const double nb = (double)A1(d.NBLADE, j);
    const float TO1M = A1(d.TO1, d.KMID), PO1M = A1(d.PO1, d.KMID);
    auto tmp_of = [&](int n, float *dP, float *dHO, float *dE) {
        const float vx = a.tVX[n], vt = a.tVT[n], vr = a.tVR[n];
        const float EKE = 0.5f * (vx * vx + vt * vt + vr * vr);
        float TS = (a.tHO[n] - EKE) * d.RCP, TSTAG = a.tHO[n] * d.RCP;
        const bool cT = TSTAG < 0.1f * TO1M, cS = TS < 0.1f * TO1M;
        if (cT) TSTAG = 0.1f * TO1M;
        if (cS) TS = 0.1f * TO1M;
        float PSTAT = a.tP[n];
        const bool cP = PSTAT < 0.02f * PO1M;
        if (cP) PSTAT = 0.02f * PO1M;
        const float rat = powf(TSTAG / TS, d.RFGA);
        const float TMP = PSTAT * rat / PO1M;
        *dP = cP ? 0.0f : rat / PO1M;
        const float dTSTAG = cT ? 0.0f : TMP * d.RFGA / TSTAG * d.RCP;
        const float dTS = cS ? 0.0f : -TMP * d.RFGA / TS;
        *dHO = dTSTAG + dTS * d.RCP;
        *dE = -dTS * d.RCP;   // d/dEKE
        return TMP;
    };
    if (t < np) {
        // node (i, j, k): the cells of plane j around it weight its TMP, TEMP1 and P
        const int i = t % IM + 1, k = t / IM + 1;
        double w = 0.0;
        for (int kc = k - 1; kc <= k; ++kc)
            for (int ic = i - 1; ic <= i; ++ic) {
                if (ic < 1 || ic > IMM1 || kc < 1 || kc > KMM1) continue;
                w += 0.25 * (-(double)A3(a.tFLOWX, ic, j, kc) * nb) / bf;
            }
        const int n = ix3(d, i, j, k);
        float dP, dHO, dE;
        tmp_of(n, &dP, &dHO, &dE);
        const float TSTAG = a.tHO[n] * d.RCP;
        const float dT1 = (TSTAG < 0.1f * TO1M) ? 0.0f : d.RCP;
        const double gt = gspo * w, gT1 = gsto * w;
        const float vx = a.tVX[n], vt = a.tVT[n], vr = a.tVR[n];
        seed[0 * np + t] = (float)(gt * dE * vx);
        seed[1 * np + t] = (float)(gt * dE * vt);
        seed[2 * np + t] = (float)(gt * dE * vr);
        seed[3 * np + t] = (float)(gt * dHO + gT1 * dT1);
        seed[4 * np + t] = (float)(gt * dP);
    } else if (t < np + IMM1 * KMM1) {
        const int u = t - np;
        const int i = u % IMM1 + 1, k = u / IMM1 + 1;
        // spo = sum_c 0.25 DFLOW_c sum TMP / bf, DFLOW_c = -FLOWX_c NB
        float dP, dHO, dE;
        double stmp = 0.0, stt = 0.0;
        const int ii[4] = {i, i + 1, i + 1, i}, kk[4] = {k, k, k + 1, k + 1};
        for (int q = 0; q < 4; ++q) {
            const int n = ix3(d, ii[q], j, kk[q]);
            stmp += (double)tmp_of(n, &dP, &dHO, &dE);
            float TSTAG = a.tHO[n] * d.RCP;
            if (TSTAG < 0.1f * TO1M) TSTAG = 0.1f * TO1M;
            stt += (double)TSTAG;
        }
        const double dflow = -nb;   // d DFLOW / d FLOWX
        const double g = gspo * (0.25 * stmp - spo) / bf * dflow + gsto * (0.25 * stt - sto) / bf * dflow + gbf * dflow;
        seed[5 * np + u] = (float)g;
    }
}

}  // namespace

// =====================================================================
// host side
// =====================================================================
#define ACK(call)                                                                                    \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return api_fail(MGPU_E_CUDA, (std::string(#call) + ": " + cudaGetErrorString(e_)).c_str()); \
    } while (0)

// row means of |STORE| after the row mixing, as the negative feedback of the
// recorded step formed them (1501-1525): one CTA per variable
__global__ void rk_blk(const __grid_constant__ Dev d, const __grid_constant__ Adj a) {
    __shared__ double sh[RT_BS / 32];
    __shared__ float chg[64];
    const AdjVar &V = a.v[blockIdx.x];
    float *blk = const_cast<float *>(V.tBLK);
    const int IMM1 = d.IMM1, KMM1 = d.KMM1, NROWS = d.NROWS;
    for (int nr = 1; nr <= NROWS; ++nr) {
        const int JST = A1(d.JSTART, nr) + 1, JEN = A1(d.JMIX, nr) - 1;
        const int nc = IMM1 * KMM1 * (JEN - JST + 1);
        double s = 0.0;
        for (int c = threadIdx.x; c < nc; c += RT_BS) {
            const int i = c % IMM1 + 1, r = c / IMM1;
            const int k = r % KMM1 + 1, j = JST + r / KMM1;
            s += (double)fabsf(A3(V.tST, i, j, k));
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < RT_BS / 32; ++w) t += sh[w];
            chg[nr - 1] = (float)t / (float)nc;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (NROWS == 1) blk[0] = chg[0];
        if (NROWS == 2) {
            blk[1] = 0.5f * (chg[0] + chg[1]);
            blk[0] = blk[1];
        }
        if (NROWS > 2) {
            for (int nr = 2; nr <= NROWS - 1; ++nr) blk[nr - 1] = 0.25f * (chg[nr - 2] + chg[nr]) + 0.5f * chg[nr - 1];
            blk[NROWS - 1] = 0.5f * (chg[NROWS - 2] + chg[NROWS - 1]);
            blk[0] = 0.5f * (chg[0] + chg[1]);
        }
    }
}

// sum of squares of the five conserved-variable adjoints and of their change
__global__ void rk_norms(const __grid_constant__ Dev d, const __grid_constant__ Adj a, const float *prev, double *out) {
    __shared__ double sh[2][RT_BS / 32];
    const size_t N = (size_t)d.IM * d.JM * d.KM;
    double s = 0.0, c = 0.0;
    for (size_t t = (size_t)blockIdx.x * RT_BS + threadIdx.x; t < 5 * N; t += (size_t)gridDim.x * RT_BS) {
        const int v = (int)(t / N);
        const float x = a.v[v].D[t - (size_t)v * N];
        const float p = prev[t];
        s += (double)x * x;
        c += (double)(x - p) * (x - p);
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sh[0][threadIdx.x >> 5] = s;
        sh[1][threadIdx.x >> 5] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ts = 0.0, tc = 0.0;
        for (int w = 0; w < RT_BS / 32; ++w) {
            ts += sh[0][w];
            tc += sh[1][w];
        }
        atomicAdd(&out[0], ts);
        atomicAdd(&out[1], tc);
    }
}

// Krylov vector kernels over packed adjoint vectors of length len
// out[i] += V_i . w for i < nv (grid.y = i), FP64
// Dot products <V_i, w>.  Each thread sums its strided elements in FP32 (a
// few dozen terms), and the partial sums are added across threads in FP64.
// FP64 arithmetic is a small fraction of the FP32 rate on this GPU, so a
// conversion and an FP64 multiply-add per element would cost more than the
// memory traffic.
__global__ void rk_kdots(const float *V, int nv, const float *w, size_t len, double *out) {
    __shared__ double sh[RT_BS / 32];
    const int i = blockIdx.y;
    const float *v = V + (size_t)i * len;
    float sf = 0.0f;
    for (size_t t = (size_t)blockIdx.x * RT_BS + threadIdx.x; t < len; t += (size_t)gridDim.x * RT_BS)
        sf += v[t] * w[t];
    double s = (double)sf;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < RT_BS / 32; ++q) t += sh[q];
        atomicAdd(&out[i], t);
    }
}
// w += sign * sum_i c_i V_i, in FP32 (the basis vectors are FP32)
constexpr int KMAX = 256;
__global__ void rk_kcomb(const float *V, int nv, const double *c, float sign, float *w, size_t len) {
    __shared__ float cs[KMAX];
    for (int i = threadIdx.x; i < nv; i += blockDim.x) cs[i] = sign * (float)c[i];
    __syncthreads();
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < len; t += (size_t)gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int i = 0; i < nv; ++i) s += cs[i] * V[(size_t)i * len + t];
        w[t] += s;
    }
}
// y = a x
__global__ void rk_kscale(float a_, const float *x, float *y, size_t len) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < len; t += (size_t)gridDim.x * blockDim.x)
        y[t] = a_ * x[t];
}
// y = a x + b y
__global__ void rk_kaxpby(float a_, const float *x, float b_, float *y, size_t len) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < len; t += (size_t)gridDim.x * blockDim.x)
        y[t] = a_ * x[t] + b_ * y[t];
}

// =====================================================================
// SETUP's face areas and volumes (3030-4045) transposed: with the node
// coordinates X, R fixed they are linear in THETA, so dJ/dTHETA is the
// transposed map applied to dJ/d(AQX, AQR, ABX, ABR, ASX, ASR, VOLOR).
// One thread per node owns the faces whose corner (I, J, K) it is and
// scatters its THETA terms with atomics (once per gradient, not per step).
// On the planes after a mixing plane the areas read the downstream THETA
// extrapolated onto the mixing plane (3025):
//   TH(JMIX) = TH(JMIX+1) + DS(JMIX+1)/DS(JMIX+2) (TH(JMIX+1) - TH(JMIX+2)).
// =====================================================================
__device__ __forceinline__ void th_add(const Dev &d, float *gth, int i, int j, int k, float g) {
    if (g != 0.0f) atomicAdd(&gth[ix3(d, i, j, k)], g);
}
// an adjoint of THETA at plane jm = J-1 as the areas of plane J read it
__device__ __forceinline__ void thm_add(const Dev &d, float *gth, int i, int jm, int k, float g) {
    if (g == 0.0f) return;
    if (A1(d.INDMIX, jm) == 1) {
        const float fac = A2(d.DS, jm + 1, k) / A2(d.DS, jm + 2, k);
        th_add(d, gth, i, jm + 1, k, (1.0f + fac) * g);
        th_add(d, gth, i, jm + 2, k, -fac * g);
    } else {
        th_add(d, gth, i, jm, k, g);
    }
}

__global__ void rk_metrics(const Dev d, const Adj a, float *gth) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, (size_t)n, i, j, k);
    const int IM = d.IM, KM = d.KM, IMM1 = d.IMM1, KMM1 = d.KMM1, JM = d.JM;
    // VOLOR = -RAREA/8, RAREA = ABR(i) - ABR(i+1) + AQR(j) - AQR(j-1) + ASR(k) - ASR(k+1)
    auto gv = [&](int ii, int jj, int kk) -> float {
        if (ii < 1 || ii > IMM1 || jj < 2 || jj > JM || kk < 1 || kk > KMM1) return 0.0f;
        return A3(a.gVOLOR, ii, jj, kk);
    };
    // faces K = const, i <= IMM1, k <= KMM1 (AQX, AQR; K = KM and I = IM copy them)
    if (i <= IMM1 && k <= KMM1) {
        float gx = A3(a.gAQX, i, j, k), gr = A3(a.gAQR, i, j, k);
        if (k == KMM1) { gx += A3(a.gAQX, i, j, KM); gr += A3(a.gAQR, i, j, KM); }
        if (i == IMM1) { gx += A3(a.gAQX, IM, j, k); gr += A3(a.gAQR, IM, j, k); }
        if (i == IMM1 && k == KMM1) { gx += A3(a.gAQX, IM, j, KM); gr += A3(a.gAQR, IM, j, KM); }
        gr += -0.125f * gv(i, j, k) + 0.125f * gv(i, j + 1, k);
        const float R1 = A2(d.R, j, k + 1) - A2(d.R, j, k), X1 = A2(d.X, j, k + 1) - A2(d.X, j, k);
        // AQX = -(R1 T1 - R1 T2)/2, AQR = -(X1 T2 - X1 T1)/2
        const float gT1 = -0.5f * R1 * gx + 0.5f * X1 * gr, gT2 = 0.5f * R1 * gx - 0.5f * X1 * gr;
        const float rk1 = A2(d.R, j, k + 1), rk = A2(d.R, j, k);
        // T1 = R(j,k+1) (TH(i+1,j,k+1) - TH(i,j,k))
        // T2 = R(j,k+1) (TH(i,j,k+1) - TH(i,j,k)) - R(j,k) (TH(i+1,j,k) - TH(i,j,k))
        th_add(d, gth, i + 1, j, k + 1, rk1 * gT1);
        th_add(d, gth, i, j, k + 1, rk1 * gT2);
        th_add(d, gth, i + 1, j, k, -rk * gT2);
        th_add(d, gth, i, j, k, -rk1 * gT1 + (rk - rk1) * gT2);
    }
    // faces I = const, j >= 2, k <= KMM1 (ABX, ABR)
    if (j >= 2 && k <= KMM1) {
        const float gx = A3(a.gABX, i, j, k);
        const float gr = A3(a.gABR, i, j, k) - 0.125f * gv(i, j, k) + 0.125f * gv(i - 1, j, k);
        const float bx1 = A2(d.X, j - 1, k + 1) - A2(d.X, j, k), bx2 = A2(d.X, j, k + 1) - A2(d.X, j - 1, k);
        const float br1 = A2(d.R, j - 1, k + 1) - A2(d.R, j, k), br2 = A2(d.R, j, k + 1) - A2(d.R, j - 1, k);
        // ABX = -(br1 T2 - br2 T1)/2, ABR = -(bx2 T1 - bx1 T2)/2
        const float gT1 = 0.5f * br2 * gx - 0.5f * bx2 * gr, gT2 = -0.5f * br1 * gx + 0.5f * bx1 * gr;
        const float rm1kp = A2(d.R, j - 1, k + 1), rjkp = A2(d.R, j, k + 1), rm1k = A2(d.R, j - 1, k);
        // T1 = R(j-1,k+1) (THm(i,j-1,k+1) - TH(i,j,k))
        // T2 = R(j,k+1) (TH(i,j,k+1) - TH(i,j,k)) - R(j-1,k) (THm(i,j-1,k) - TH(i,j,k))
        thm_add(d, gth, i, j - 1, k + 1, rm1kp * gT1);
        th_add(d, gth, i, j, k + 1, rjkp * gT2);
        thm_add(d, gth, i, j - 1, k, -rm1k * gT2);
        th_add(d, gth, i, j, k, -rm1kp * gT1 + (rm1k - rjkp) * gT2);
    }
    // faces J = const, j >= 2, i <= IMM1 (ASX, ASR)
    if (j >= 2 && i <= IMM1) {
        const float gx = A3(a.gASX, i, j, k);
        const float gr = A3(a.gASR, i, j, k) - 0.125f * gv(i, j, k) + 0.125f * gv(i, j, k - 1);
        const float sx1 = A2(d.X, j - 1, k) - A2(d.X, j, k), sr1 = A2(d.R, j - 1, k) - A2(d.R, j, k);
        // ASX = (sr1 T2 - sr1 T1)/2, ASR = (sx1 T1 - sx1 T2)/2
        const float gT1 = -0.5f * sr1 * gx + 0.5f * sx1 * gr, gT2 = 0.5f * sr1 * gx - 0.5f * sx1 * gr;
        const float rm1 = A2(d.R, j - 1, k), rj = A2(d.R, j, k);
        // T1 = R(j-1,k) (THm(i,j-1,k) - TH(i,j,k)) - R(j,k) (TH(i+1,j,k) - TH(i,j,k))
        // T2 = R(j-1,k) (THm(i+1,j-1,k) - TH(i,j,k))
        thm_add(d, gth, i, j - 1, k, rm1 * gT1);
        th_add(d, gth, i + 1, j, k, -rj * gT1);
        thm_add(d, gth, i + 1, j - 1, k, rm1 * gT2);
        th_add(d, gth, i, j, k, (rj - rm1) * gT1 - rm1 * gT2);
    }
}

struct AdjState {
    mgpu_handle *h = nullptr;
    Adj a;
    std::vector<void *> allocs;
    DevCtl *tctl = nullptr;
    int *flag = nullptr;
    float *seed = nullptr;
    float *prev = nullptr;       // 5 N: the conserved-variable adjoints before the last iteration
    double *norms = nullptr;
    std::vector<double> sums;    // (4, JM) EFICOOL sums of the recorded step
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int objective = -1;
    double value = 0.0;
    bool ready = false;
    int iters = 0;
    int limiters = 0;            // bit 0: density, bit 1: Mach limiter active in the recorded step
    int *seed_on = nullptr;
    // restarted GMRES on (I - (dG/dU)^T) lambda = (dJ/dU)^T over the packed
    // state adjoint (the arrays of state_segments())
    float *kv = nullptr;         // (m + 1) basis vectors
    float *kw = nullptr, *kb = nullptr, *kx = nullptr;
    double *kdot = nullptr;      // (m + 2) FP64 dot products
    int kcap = 0;
    size_t klen = 0;
};

void adj_destroy(AdjState *s) {
    if (!s) return;
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    if (s->graph) cudaGraphDestroy(s->graph);
    for (void *p : s->allocs) cudaFree(p);
    void *kb[] = {s->kv, s->kw, s->kb, s->kx, s->kdot};
    for (void *p : kb)
        if (p) cudaFree(p);
    delete s;
}

namespace {

template <typename T>
int aalloc(AdjState *s, T **p, size_t count) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, (count ? count : 1) * sizeof(T));
    if (e != cudaSuccess) return api_fail(MGPU_E_NOMEM, "adjoint device allocation");
    s->allocs.push_back(q);
    cudaMemset(q, 0, (count ? count : 1) * sizeof(T));
    *p = (T *)q;
    return 0;
}

size_t smooth_bytes(const Dev &d) { return (size_t)3 * d.IM * d.KM * sizeof(float); }
size_t gather_bytes(const Dev &d) { return (size_t)d.IMM1 * d.KMM1 * sizeof(float); }
size_t cells_bytes(const Dev &d) {
    return ((size_t)d.NIB1 * d.NKB1 + (size_t)d.NIB2 * d.NKB2 + (size_t)d.IMM1 * d.KMM1 + d.KMM1) * sizeof(float);
}

int configure(const Dev &d) {
    struct {
        const void *f;
        size_t b;
    } k[] = {{(const void *)rk_ts_smooth, smooth_bytes(d)}, {(const void *)rk_ts_gather, gather_bytes(d)},
             {(const void *)rk_ts_cells, cells_bytes(d)}};
    for (auto &x : k) {
        if (x.b > 200 * 1024) return api_fail(MGPU_E_UNSUPPORTED, "J-plane too large for the adjoint kernels");
        ACK(raise_smem(x.f, x.b));
    }
    return 0;
}

void launch_tstep_rev(const Dev &d, const Adj &a, cudaStream_t s, int v0, int nv) {
    const size_t N = (size_t)d.IM * d.JM * d.KM;
    for (int v = v0; v < v0 + nv; ++v) cudaMemsetAsync(a.v[v].TM, 0, N * sizeof(float), s);
    const unsigned ja = (unsigned)d.JM, jp = (unsigned)(d.JM - 1);
    rk_ts_smooth<<<dim3(ja, nv), RT_BS, smooth_bytes(d), s>>>(d, a, v0);
    rk_ts_gather<<<dim3(ja, nv), RT_BS, gather_bytes(d), s>>>(d, a, v0);
    rk_ts_damp<<<dim3(jp, nv), RT_BS, 0, s>>>(d, a, v0);
    rk_ts_cells<<<dim3(jp, nv), RT_BS, cells_bytes(d), s>>>(d, a, v0);
}

// one reverse step: the adjoints of the state after a step (plus the
// objective seeds) -> the adjoints of the state before it
void enqueue_reverse(const Dev &d, const Adj &a, cudaStream_t s) {
    const size_t N = (size_t)d.IM * d.JM * d.KM;
    const unsigned gN = gridn(N, 256);
    const int per = 5 * d.IM * d.KM + d.IMM1 * d.KMM1;
    rk_seed<<<gridn((size_t)2 * per, 256), 256, 0, s>>>(d, a);
    if (d.IFMIX > 0 && d.RFMIX > 1.0e-3f && d.NRWSM1 > 0) rk_mixplan<<<d.NRWSM1 * d.KM, 64, 0, s>>>(d, a);
    rk_mach<<<gN, 256, 0, s>>>(d, a);
    rk_density<<<gridn((size_t)d.IM * d.KM, 128), 128, 0, s>>>(d, a);
    launch_tstep_rev(d, a, s, V_ROVX, 3);
    rk_flux_mom_coef<<<gN, 256, 0, s>>>(d, a);
    rk_flux_mom_gather<<<gN, 256, 0, s>>>(d, a);
    if (d.F_PDOWN != 0.0f) rk_peff<<<gN, 256, 0, s>>>(d, a);
    rk_bc_apply<<<gridn((size_t)d.IM * d.KM, 128), 128, 0, s>>>(d, a);
    launch_tstep_rev(d, a, s, V_RO, 2);
    rk_flux_energy_coef<<<gN, 256, 0, s>>>(d, a);
    rk_flux_energy_gather<<<gN, 256, 0, s>>>(d, a);
    rk_bc_sums<<<1, RBC_BS, 0, s>>>(d, a);
    rk_flux_mass_coef<<<gN, 256, 0, s>>>(d, a);
    rk_flux_mass_gather<<<gN, 256, 0, s>>>(d, a);
    rk_prim<<<gN, 256, 0, s>>>(d, a);
}

int unsupported(const Dev &d) {
    if (d.ITIMST != 3 || d.NRSMTH != 0) return api_fail(MGPU_E_UNSUPPORTED, "adjoint: SCREE without residual smoothing only");
    if (d.IPOUT != 0) return api_fail(MGPU_E_UNSUPPORTED, "adjoint: IPOUT = 0 only");
    if (d.IN_PRESS != 0 || d.IN_VTAN != 0 || d.IN_VR > 0)
        return api_fail(MGPU_E_UNSUPPORTED, "adjoint: IN_PRESS = 0, IN_VTAN = 0 and IN_VR <= 0 only");
    if (d.IN_FLOW != 0 || d.THROTTLE_EXIT > 0.001f || d.PLATE_LOSS > 0.001f || d.any_cusp2)
        return api_fail(MGPU_E_UNSUPPORTED, "adjoint: SETFLO, throttle, exit plate loss and IF_CUSP = 2 not differentiated");
    if (!(d.SFEXIT < 0.0001f) && d.NSFEXIT > 0) return api_fail(MGPU_E_UNSUPPORTED, "adjoint: exit smoothing not differentiated");
    if (d.KM > 512 || d.NROWS > 64) return api_fail(MGPU_E_UNSUPPORTED, "adjoint: KM <= 512 and NROWS <= 64");
    if (d.ILOS >= 200) return api_fail(MGPU_E_UNSUPPORTED, "adjoint: the Spalart-Allmaras model is not differentiated");
    if (d.IR <= 1 && d.JR <= 1 && d.KR <= 1) return api_fail(MGPU_E_UNSUPPORTED, "adjoint: runs without multigrid");
    return 0;
}

int allocate(AdjState *s, const Dev &d) {
    const size_t N = (size_t)d.IM * d.JM * d.KM, np = (size_t)d.IM * d.KM;
    Adj &a = s->a;
    memset(&a, 0, sizeof(a));
    int rc = 0;
    auto F = [&](float **p, size_t n) { if (!rc) rc = aalloc(s, p, n); };
    auto Fc = [&](const float **p, size_t n) {
        float *q = nullptr;
        if (!rc) rc = aalloc(s, &q, n);
        *p = q;
    };
    for (int v = 0; v < NVAR; ++v) {
        AdjVar &V = a.v[v];
        F(&V.D, N); F(&V.DIFF, N); F(&V.SR, N); F(&V.ST, N); F(&V.TM, N); F(&V.Y, N);
        if (v != V_RO) { F(&V.XF, N); F(&V.TF, N); F(&V.RF, N); }
        F(&V.P1, (size_t)d.JM * d.NIB1 * d.NKB1);
        F(&V.P2, (size_t)d.JM * d.NIB2 * d.NKB2);
        if (!rc) rc = aalloc(s, &V.psum, d.JM);
        if (!rc) rc = aalloc(s, &V.pblk, d.JM);
        Fc(&V.tST, N);
        Fc(&V.tBLK, d.NROWS);
    }
    F(&a.P, N); F(&a.HO, N); F(&a.VX, N); F(&a.VR, N); F(&a.VT, N); F(&a.ROVT, N); F(&a.PEFF, N);
    F(&a.FLOWX, N); F(&a.FLOWT, N); F(&a.FLOWR, N);
    a.v[V_RO].XF = a.FLOWX; a.v[V_RO].TF = a.FLOWT; a.v[V_RO].RF = a.FLOWR;
    F(&a.PD, d.KM); F(&a.PDK, d.KM); F(&a.PAVG, d.KM); F(&a.SSUM, d.KM);
    Fc(&a.tRO, N); Fc(&a.tROVX, N); Fc(&a.tROVR, N); Fc(&a.tRORVT, N); Fc(&a.tROE, N); Fc(&a.tPEFF0, N);
    Fc(&a.tHOJM, np); Fc(&a.tROVT1, np); Fc(&a.tP1, np);
    Fc(&a.tVX, N); Fc(&a.tVR, N); Fc(&a.tVT, N); Fc(&a.tROVT, N); Fc(&a.tP, N); Fc(&a.tHO, N); Fc(&a.tPEFF, N);
    Fc(&a.tFLOWX, N); Fc(&a.tFLOWT, N); Fc(&a.tFLOWR, N);
    Fc(&a.tBCBUF, (size_t)4 * d.KM); Fc(&a.tROIN, np);
    Fc(&a.tROL, N); Fc(&a.tROM, N); Fc(&a.tWT, N); Fc(&a.tDC0, N); Fc(&a.tDCA, N);
    Fc(&a.tVLIM, d.NROWS); Fc(&a.tROLIM, d.NROWS);
    {
        int *q = nullptr;
        if (!rc) rc = aalloc(s, &q, np);
        a.tDCOL = q;
    }
    F(&a.WT, N);
    F(&a.cf, (size_t)15 * N);
    Fc(&a.tMIX, (size_t)(d.NRWSM1 > 0 ? d.NRWSM1 : 1) * d.KM * mix_rec_size(d.IM));
    F(&a.gAQX, N); F(&a.gAQR, N); F(&a.gABX, N); F(&a.gABR, N); F(&a.gASX, N); F(&a.gASR, N); F(&a.gVOLOR, N);
    F(&a.gABT, (size_t)d.JM * d.KM);
    if (!rc) rc = aalloc(s, &s->tctl, 1);
    if (!rc) rc = aalloc(s, &s->flag, 1);
    const int per = 5 * d.IM * d.KM + d.IMM1 * d.KMM1;
    F(&s->seed, (size_t)2 * per);
    F(&s->prev, 5 * N);
    if (!rc) rc = aalloc(s, &s->norms, 2);
    if (!rc) rc = aalloc(s, &s->seed_on, 1);
    a.seed_on = s->seed_on;
    a.tctl = s->tctl;
    a.flag = s->flag;
    a.seed = s->seed;
    return rc;
}

// the adjoint arrays by name: the state adjoints (COMMON names) and PD
float *state_adj(AdjState *s, const Dev &d, const char *name, size_t *count) {
    const size_t N = (size_t)d.IM * d.JM * d.KM;
    Adj &a = s->a;
    struct {
        const char *n;
        float *p;
    } t[] = {{"RO", a.v[V_RO].D},        {"ROE", a.v[V_ROE].D},     {"ROVX", a.v[V_ROVX].D},
             {"RORVT", a.v[V_RORVT].D},  {"ROVR", a.v[V_ROVR].D},   {"DRO", a.v[V_RO].DIFF},
             {"DROE", a.v[V_ROE].DIFF},  {"DROVX", a.v[V_ROVX].DIFF}, {"DRORVT", a.v[V_RORVT].DIFF},
             {"DROVR", a.v[V_ROVR].DIFF}, {"P", a.P}, {"HO", a.HO}, {"ROVT", a.ROVT}, {"PEFF", a.PEFF},
             {"VX", a.VX}, {"VR", a.VR}, {"VT", a.VT}};
    for (auto &e : t)
        if (!strcmp(name, e.n)) {
            *count = N;
            return e.p;
        }
    if (!strcmp(name, "PD")) {
        *count = (size_t)d.KM;
        return a.PD;
    }
    return nullptr;
}

float *geom_adj(AdjState *s, const Dev &d, const char *name, size_t *count) {
    const size_t N = (size_t)d.IM * d.JM * d.KM;
    Adj &a = s->a;
    struct {
        const char *n;
        float *p;
    } t[] = {{"AQX", a.gAQX}, {"AQR", a.gAQR}, {"ABX", a.gABX}, {"ABR", a.gABR},
             {"ASX", a.gASX}, {"ASR", a.gASR}, {"VOLOR", a.gVOLOR}};
    for (auto &e : t)
        if (!strcmp(name, e.n)) {
            *count = N;
            return e.p;
        }
    if (!strcmp(name, "ABT")) {
        *count = (size_t)d.JM * d.KM;
        return a.gABT;
    }
    return nullptr;
}

// the state adjoint as segments of a packed vector
struct Seg {
    float *p;
    size_t n;
};
std::vector<Seg> state_segments(AdjState *s, const Dev &d) {
    const size_t N = (size_t)d.IM * d.JM * d.KM;
    Adj &a = s->a;
    std::vector<Seg> v;
    for (int q = 0; q < NVAR; ++q) v.push_back({a.v[q].D, N});
    for (int q = 0; q < NVAR; ++q) v.push_back({a.v[q].DIFF, N});
    v.push_back({a.PEFF, N});
    v.push_back({a.P, N});
    v.push_back({a.HO, N});
    v.push_back({a.ROVT, N});
    v.push_back({a.PD, (size_t)d.KM});
    return v;
}

int pack(AdjState *s, const Dev &d, float *dst, cudaStream_t st) {
    size_t o = 0;
    for (const Seg &g : state_segments(s, d)) {
        ACK(cudaMemcpyAsync(dst + o, g.p, g.n * sizeof(float), cudaMemcpyDeviceToDevice, st));
        o += g.n;
    }
    return 0;
}

int unpack(AdjState *s, const Dev &d, const float *src, cudaStream_t st) {
    size_t o = 0;
    for (const Seg &g : state_segments(s, d)) {
        ACK(cudaMemcpyAsync(g.p, src + o, g.n * sizeof(float), cudaMemcpyDeviceToDevice, st));
        o += g.n;
    }
    return 0;
}

int zero_adjoints(AdjState *s, const Dev &d, cudaStream_t st) {
    const size_t N = (size_t)d.IM * d.JM * d.KM;
    Adj &a = s->a;
    for (int v = 0; v < NVAR; ++v) {
        AdjVar &V = a.v[v];
        float *z[] = {V.D, V.DIFF, V.SR, V.ST, V.TM, V.Y, V.XF, V.TF, V.RF};
        for (float *p : z)
            if (p) ACK(cudaMemsetAsync(p, 0, N * sizeof(float), st));
    }
    float *z[] = {a.P, a.HO, a.VX, a.VR, a.VT, a.ROVT, a.PEFF, a.FLOWX, a.FLOWT, a.FLOWR, a.WT};
    for (float *p : z) ACK(cudaMemsetAsync(p, 0, N * sizeof(float), st));
    float *zk[] = {a.PD, a.PDK, a.PAVG, a.SSUM};
    for (float *p : zk) ACK(cudaMemsetAsync(p, 0, (size_t)d.KM * sizeof(float), st));
    return 0;
}

}  // namespace
}  // namespace mgpu

using namespace mgpu;

extern "C" {

int32_t mgpu_adjoint_prepare(mgpu_handle *h) {
    HandleView hv = handle_view(h);
    if (!h || !hv.committed) return api_fail(MGPU_E_STATE, "adjoint before commit");
    Dev &dh = handle_dev(h);
    int rc = unsupported(dh);
    if (rc) return rc;
    AdjState *&s = handle_adj(h);
    if (!s) {
        s = new AdjState();
        s->h = h;
        if ((rc = allocate(s, dh)) || (rc = configure(dh))) {
            adj_destroy(s);
            s = nullptr;
            return rc;
        }
    }
    const Dev &d = dh;
    cudaStream_t st = hv.stream;
    const size_t N = (size_t)d.IM * d.JM * d.KM, np = (size_t)d.IM * d.KM;
    const size_t fb = N * sizeof(float);
    Adj &a = s->a;
    // the state before the recorded step
    auto cp = [&](const float *dst, const float *src, size_t n) {
        return cudaMemcpyAsync((void *)dst, src, n * sizeof(float), cudaMemcpyDeviceToDevice, st);
    };
    ACK(cp(a.tRO, d.RO, N)); ACK(cp(a.tROVX, d.ROVX, N)); ACK(cp(a.tROVR, d.ROVR, N));
    ACK(cp(a.tRORVT, d.RORVT, N)); ACK(cp(a.tROE, d.ROE, N)); ACK(cp(a.tPEFF0, d.PEFF, N));
    ACK(cudaMemcpy2DAsync((void *)a.tHOJM, (size_t)d.IM * 4, d.HO + (size_t)d.IM * (d.JM - 1), (size_t)d.IM * d.JM * 4,
                          (size_t)d.IM * 4, d.KM, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpy2DAsync((void *)a.tROVT1, (size_t)d.IM * 4, d.ROVT, (size_t)d.IM * d.JM * 4, (size_t)d.IM * 4, d.KM,
                          cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpy2DAsync((void *)a.tP1, (size_t)d.IM * 4, d.P, (size_t)d.IM * d.JM * 4, (size_t)d.IM * 4, d.KM,
                          cudaMemcpyDeviceToDevice, st));
    // everything else the step changes, restored afterwards
    float *const keep[] = {d.DRO, d.DROE, d.DROVX, d.DROVR, d.DRORVT, d.P, d.HO, d.T_STATIC, d.VX, d.VR, d.VT,
                           d.WT, d.ROWT, d.ROVT};
    const int nkeep = (int)(sizeof(keep) / sizeof(keep[0]));
    float *save = nullptr, *savepd = nullptr;
    DevCtl *savectl = nullptr;
    ACK(cudaMallocAsync((void **)&save, nkeep * fb, st));
    ACK(cudaMallocAsync((void **)&savepd, (size_t)d.KM * 4, st));
    ACK(cudaMallocAsync((void **)&savectl, sizeof(DevCtl), st));
    for (int q = 0; q < nkeep; ++q) ACK(cudaMemcpyAsync(save + (size_t)q * N, keep[q], fb, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(savepd, d.PD, (size_t)d.KM * 4, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(savectl, d.ctl, sizeof(DevCtl), cudaMemcpyDeviceToDevice, st));
    // the recorded step: LOSS and STEPUP held
    Dev rec = d;
    rec.use_cond = 0;
    rec.FROZEN = 1;
    rec.ADJ_ROIN = const_cast<float *>(a.tROIN);
    rec.ADJ_MIX = const_cast<float *>(a.tMIX);
    rec.ADJ_FLAG = s->flag;
    rec.ADJ_RO_LIM = const_cast<float *>(a.tROL);
    rec.ADJ_RO_MACH = const_cast<float *>(a.tROM);
    ACK(cudaMemsetAsync(s->flag, 0, sizeof(int), st));
    Launch L{st, handle_sm_count(h)};
    launch_step_begin(rec, L);
    launch_prim(rec, L);
    enqueue_step_core(rec, L);
    ACK(cudaGetLastError());
    ACK(cp(a.tVX, d.VX, N)); ACK(cp(a.tVR, d.VR, N)); ACK(cp(a.tVT, d.VT, N)); ACK(cp(a.tROVT, d.ROVT, N));
    ACK(cp(a.tP, d.P, N)); ACK(cp(a.tHO, d.HO, N)); ACK(cp(a.tPEFF, d.PEFF, N));
    ACK(cp(a.tFLOWX, d.FLOWX, N)); ACK(cp(a.tFLOWT, d.FLOWT, N)); ACK(cp(a.tFLOWR, d.FLOWR, N));
    for (int v = 0; v < NVAR; ++v) ACK(cp(a.v[v].tST, d.var[v].ST, N));
    ACK(cp(a.tBCBUF, d.BCBUF, (size_t)4 * d.KM));
    ACK(cp(a.tWT, d.WT, N));
    ACK(cp(a.tVLIM, d.VLIMIT, (size_t)d.NROWS));
    ACK(cp(a.tROLIM, d.ROLIMIT, (size_t)d.NROWS));
    ACK(cudaMemcpyAsync(s->tctl, d.ctl, sizeof(DevCtl), cudaMemcpyDeviceToDevice, st));
    // the EFICOOL sums of the step's arrays (the objectives' forward values)
    double *dint = handle_int_buf(h);
    launch_integrals(rec, L, dint);
    rk_blk<<<NVAR, RT_BS, 0, st>>>(d, a);
    rk_density_prep<<<gridn(np, 128), 128, 0, st>>>(d, a);
    ACK(cudaGetLastError());
    s->sums.assign((size_t)4 * d.JM, 0.0);
    ACK(cudaMemcpyAsync(s->sums.data(), dint, s->sums.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    // restore the state
    ACK(cudaMemcpyAsync(d.RO, a.tRO, fb, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(d.ROVX, a.tROVX, fb, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(d.ROVR, a.tROVR, fb, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(d.RORVT, a.tRORVT, fb, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(d.ROE, a.tROE, fb, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(d.PEFF, a.tPEFF0, fb, cudaMemcpyDeviceToDevice, st));
    for (int q = 0; q < nkeep; ++q) ACK(cudaMemcpyAsync(keep[q], save + (size_t)q * N, fb, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(d.PD, savepd, (size_t)d.KM * 4, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(d.ctl, savectl, sizeof(DevCtl), cudaMemcpyDeviceToDevice, st));
    ACK(cudaFreeAsync(save, st));
    ACK(cudaFreeAsync(savepd, st));
    ACK(cudaFreeAsync(savectl, st));
    int flag = 0;
    ACK(cudaMemcpyAsync(&flag, s->flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    ACK(cudaStreamSynchronize(st));
    s->limiters = flag & 3;
    ACK(cudaMemsetAsync(s->flag, 0, sizeof(int), st));
    if ((rc = zero_adjoints(s, d, st))) return rc;
    ACK(cudaMemsetAsync(s->seed, 0, (size_t)2 * (5 * d.IM * d.KM + d.IMM1 * d.KMM1) * sizeof(float), st));
    s->a.seed_j[0] = 1;
    s->a.seed_j[1] = 2;
    s->objective = -1;
    s->value = 0.0;
    s->iters = 0;
    // the reverse step as a CUDA graph
    if (s->gexec) {
        cudaGraphExecDestroy(s->gexec);
        s->gexec = nullptr;
    }
    if (s->graph) {
        cudaGraphDestroy(s->graph);
        s->graph = nullptr;
    }
    {
        const int one = 1;
        ACK(cudaMemcpyAsync(s->seed_on, &one, sizeof(int), cudaMemcpyHostToDevice, st));
    }
    ACK(cudaStreamSynchronize(st));
    s->ready = true;
    return 0;
}

namespace {
int ensure_graph(AdjState *s, const Dev &d, cudaStream_t st) {
    if (s->gexec) return 0;
    ACK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    enqueue_reverse(d, s->a, st);
    cudaGraph_t g = nullptr;
    ACK(cudaStreamEndCapture(st, &g));
    s->graph = g;
    ACK(cudaGraphInstantiate(&s->gexec, g, 0));
    return 0;
}
AdjState *ready_state(mgpu_handle *h) {
    if (!h) return nullptr;
    AdjState *s = handle_adj(h);
    return (s && s->ready) ? s : nullptr;
}
}  // namespace

int32_t mgpu_adjoint_objective(mgpu_handle *h, int32_t which, double *value) {
    AdjState *s = ready_state(h);
    if (!s) return api_fail(MGPU_E_STATE, "adjoint objective before mgpu_adjoint_prepare");
    if (which < -1 || which > 2) return api_fail(MGPU_E_ARG, "objective: -1 none, 0 eta_tt, 1 mass flow in, 2 mass flow out");
    const Dev &d = handle_dev(h);
    cudaStream_t st = handle_view(h).stream;
    const int per = 5 * d.IM * d.KM + d.IMM1 * d.KMM1;
    ACK(cudaMemsetAsync(s->seed, 0, (size_t)2 * per * sizeof(float), st));
    const int J1 = d.NSTAGES == 1 ? 1 : 2, J2M1 = d.JM - 1;
    s->a.seed_j[0] = J1;
    s->a.seed_j[1] = J2M1;
    const std::vector<double> &v = s->sums;
    auto bf = [&](int j) { return v[(size_t)(j - 1)]; };
    auto spo = [&](int j) { return v[(size_t)d.JM + j - 1] / bf(j); };
    auto sto = [&](int j) { return v[(size_t)2 * d.JM + j - 1] / bf(j); };
    double J = 0.0, g[2][3] = {{0, 0, 0}, {0, 0, 0}};   // per plane: dJ/dspo, dJ/dsto, dJ/dbf
    if (which == 1) {
        J = bf(J1);
        g[0][2] = 1.0;
    } else if (which == 2) {
        J = bf(J2M1);
        g[1][2] = 1.0;
    } else if (which == 0) {
        const double FGA = (double)d.FGA;
        const double p1 = spo(J1), p2 = spo(J2M1), s1 = sto(J1), s2 = sto(J2M1);
        const double P = p2 / p1, D = s2 - s1, pf = std::pow(P, FGA), Dis = s1 * (pf - 1.0);
        const double dPf_dp2 = FGA * std::pow(P, FGA - 1.0) / p1, dPf_dp1 = -FGA * std::pow(P, FGA - 1.0) * p2 / (p1 * p1);
        if (D < 0.0) {          // turbine: eta = D / Dis
            J = D / Dis;
            g[1][1] = 1.0 / Dis;
            g[0][1] = -1.0 / Dis - D * (pf - 1.0) / (Dis * Dis);
            g[1][0] = -D / (Dis * Dis) * s1 * dPf_dp2;
            g[0][0] = -D / (Dis * Dis) * s1 * dPf_dp1;
        } else if (D > 0.0) {   // compressor: eta = Dis / D
            J = Dis / D;
            g[1][1] = -Dis / (D * D);
            g[0][1] = (pf - 1.0) / D + Dis / (D * D);
            g[1][0] = s1 * dPf_dp2 / D;
            g[0][0] = s1 * dPf_dp1 / D;
        } else {
            J = 1.0;
        }
    }
    if (which >= 0) {
        const int js[2] = {J1, J2M1};
        for (int p = 0; p < 2; ++p) {
            const int j = js[p];
            rk_seed_plane<<<gridn((size_t)per, 256), 256, 0, st>>>(d, s->a, s->seed + (size_t)p * per, j, g[p][0], g[p][1],
                                                                  g[p][2], spo(j), sto(j), bf(j));
        }
        ACK(cudaGetLastError());
    }
    // the seeds are kernel parameters of the captured graph (seed_j)
    if (s->gexec) {
        cudaGraphExecDestroy(s->gexec);
        s->gexec = nullptr;
        cudaGraphDestroy(s->graph);
        s->graph = nullptr;
    }
    ACK(cudaStreamSynchronize(st));
    s->objective = which;
    s->value = J;
    if (value) *value = J;
    return 0;
}

int32_t mgpu_adjoint_iterate(mgpu_handle *h, int32_t n, double *rel_change) {
    AdjState *s = ready_state(h);
    if (!s) return api_fail(MGPU_E_STATE, "adjoint iteration before mgpu_adjoint_prepare");
    if (n < 1) return api_fail(MGPU_E_ARG, "adjoint iteration count must be positive");
    const Dev &d = handle_dev(h);
    cudaStream_t st = handle_view(h).stream;
    int rc = ensure_graph(s, d, st);
    if (rc) return rc;
    const size_t N = (size_t)d.IM * d.JM * d.KM;
    for (int it = 0; it < n; ++it) {
        if (it == n - 1 && rel_change) {
            for (int v = 0; v < NVAR; ++v)
                ACK(cudaMemcpyAsync(s->prev + (size_t)v * N, s->a.v[v].D, N * sizeof(float), cudaMemcpyDeviceToDevice, st));
        }
        ACK(cudaGraphLaunch(s->gexec, st));
    }
    s->iters += n;
    int flag = 0;
    ACK(cudaMemcpyAsync(&flag, s->flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (rel_change) {
        ACK(cudaMemsetAsync(s->norms, 0, 2 * sizeof(double), st));
        rk_norms<<<4 * handle_sm_count(h), RT_BS, 0, st>>>(d, s->a, s->prev, s->norms);
        double nm[2];
        ACK(cudaMemcpyAsync(nm, s->norms, sizeof(nm), cudaMemcpyDeviceToHost, st));
        ACK(cudaStreamSynchronize(st));
        *rel_change = nm[0] > 0.0 ? std::sqrt(nm[1] / nm[0]) : 0.0;
    } else {
        ACK(cudaStreamSynchronize(st));
    }
    if (flag & 1) return api_fail(MGPU_E_UNSUPPORTED, "adjoint: supersonic relative flow at a mixing plane (Prandtl-Meyer sweep) is not differentiated");
    return 0;
}

int32_t mgpu_adjoint_solve(mgpu_handle *h, int32_t max_iters, double tol, int32_t *iters, double *rel_change) {
    AdjState *s = ready_state(h);
    if (!s) return api_fail(MGPU_E_STATE, "adjoint solve before mgpu_adjoint_prepare");
    if (max_iters < 1 || !(tol > 0.0)) return api_fail(MGPU_E_ARG, "adjoint solve: max_iters >= 1, tol > 0");
    int done = 0;
    double rel = 1.0;
    const int chunk = 50;
    int rc = 0;
    while (done < max_iters) {
        const int n = max_iters - done < chunk ? max_iters - done : chunk;
        if ((rc = mgpu_adjoint_iterate(h, n, &rel))) break;
        done += n;
        if (rel < tol) break;
    }
    if (iters) *iters = done;
    if (rel_change) *rel_change = rel;
    if (rc) return rc;
    return rel < tol ? 0 : 1;
}

int32_t mgpu_adjoint_solve_krylov(mgpu_handle *h, int32_t inner, int32_t restart, int32_t max_steps, double tol,
                                  double stall, int32_t *steps, double *rel_residual) {
    AdjState *s = ready_state(h);
    if (!s) return api_fail(MGPU_E_STATE, "adjoint solve before mgpu_adjoint_prepare");
    if (inner < 1 || restart < 2 || restart > 200 || max_steps < 1 || !(tol > 0.0) || !(stall >= 0.0 && stall < 1.0))
        return api_fail(MGPU_E_ARG,
                        "Krylov solve: inner >= 1, 2 <= restart <= 200, max_steps >= 1, tol > 0, 0 <= stall < 1");
    const Dev &d = handle_dev(h);
    cudaStream_t st = handle_view(h).stream;
    int rc = ensure_graph(s, d, st);
    if (rc) return rc;
    size_t len = 0;
    for (const Seg &g : state_segments(s, d)) len += g.n;
    if (s->kcap < restart + 1 || s->klen != len) {
        if (s->kv) cudaFree(s->kv);
        if (s->kw) cudaFree(s->kw);
        if (s->kb) cudaFree(s->kb);
        if (s->kx) cudaFree(s->kx);
        if (s->kdot) cudaFree(s->kdot);
        s->kv = s->kw = s->kb = s->kx = nullptr;
        s->kdot = nullptr;
        ACK(cudaMalloc(&s->kv, (size_t)(restart + 1) * len * sizeof(float)));
        ACK(cudaMalloc(&s->kw, len * sizeof(float)));
        ACK(cudaMalloc(&s->kb, len * sizeof(float)));
        ACK(cudaMalloc(&s->kx, len * sizeof(float)));
        ACK(cudaMalloc(&s->kdot, (size_t)(restart + 2) * sizeof(double)));
        s->kcap = restart + 1;
        s->klen = len;
    }
    const int sm = handle_sm_count(h);
    const unsigned gb = (unsigned)(4 * sm);
    auto seeds = [&](int on) { return cudaMemsetAsync(s->seed_on, on ? 1 : 0, sizeof(int), st); };
    auto dots = [&](const float *V, int nv, const float *w, std::vector<double> &out) -> int {
        ACK(cudaMemsetAsync(s->kdot, 0, (size_t)nv * sizeof(double), st));
        rk_kdots<<<dim3(gb, nv), RT_BS, 0, st>>>(V, nv, w, len, s->kdot);
        out.assign((size_t)nv, 0.0);
        ACK(cudaMemcpyAsync(out.data(), s->kdot, (size_t)nv * sizeof(double), cudaMemcpyDeviceToHost, st));
        ACK(cudaStreamSynchronize(st));
        return 0;
    };
    auto comb = [&](const float *V, const std::vector<double> &c, float sign, float *w) -> int {
        ACK(cudaMemcpyAsync(s->kdot, c.data(), c.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        rk_kcomb<<<gb, RT_BS, 0, st>>>(V, (int)c.size(), s->kdot, sign, w, len);
        return 0;
    };
    // The operator is the inner-step map: out = x - ((dG/dU)^T)^inner x, and
    // the right-hand side b = sum_{i < inner} ((dG/dU)^T)^i (dJ/dU)^T, the
    // inner steps from lambda = 0; the fixed point is the adjoint's.
    int nprod = 0;
    auto apply = [&](const float *x, float *out) -> int {
        int r = unpack(s, d, x, st);
        if (r) return r;
        ACK(seeds(0));
        for (int q = 0; q < inner; ++q) ACK(cudaGraphLaunch(s->gexec, st));
        r = pack(s, d, out, st);
        if (r) return r;
        rk_kaxpby<<<gb, RT_BS, 0, st>>>(1.0f, x, -1.0f, out, len);
        nprod += inner;
        return 0;
    };
    if ((rc = pack(s, d, s->kx, st))) return rc;          // initial guess: the current adjoint
    ACK(cudaMemsetAsync(s->kw, 0, len * sizeof(float), st));
    if ((rc = unpack(s, d, s->kw, st))) return rc;
    ACK(seeds(1));
    for (int q = 0; q < inner; ++q) ACK(cudaGraphLaunch(s->gexec, st));
    nprod += inner;
    if ((rc = pack(s, d, s->kb, st))) return rc;
    std::vector<double> dd;
    if ((rc = dots(s->kb, 1, s->kb, dd))) return rc;
    const double bnorm = std::sqrt(dd[0]);
    double rel = 0.0;
    const int m = restart;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
    bool done = bnorm == 0.0;
    double cycle_rel = -1.0;     // residual estimate at the end of the last restart cycle
    while (!done && nprod < max_steps) {
        // r = b - A x into v_0
        float *v0 = s->kv;
        if ((rc = apply(s->kx, v0))) return rc;
        rk_kaxpby<<<gb, RT_BS, 0, st>>>(1.0f, s->kb, -1.0f, v0, len);
        if ((rc = dots(v0, 1, v0, dd))) return rc;
        const double beta = std::sqrt(dd[0]);
        rel = beta / bnorm;
        if (rel < tol) break;
        rk_kscale<<<gb, RT_BS, 0, st>>>((float)(1.0 / beta), v0, v0, len);
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int jdone = 0;
        for (int j = 0; j < m && nprod < max_steps; ++j) {
            float *vj = s->kv + (size_t)j * len, *w = s->kw;
            if ((rc = apply(vj, w))) return rc;
            std::vector<double> h1, h2;
            if ((rc = dots(s->kv, j + 1, w, h1))) return rc;     // classical Gram-Schmidt, twice
            if ((rc = comb(s->kv, h1, -1.0f, w))) return rc;
            if ((rc = dots(s->kv, j + 1, w, h2))) return rc;
            if ((rc = comb(s->kv, h2, -1.0f, w))) return rc;
            if ((rc = dots(w, 1, w, dd))) return rc;
            const double hn = std::sqrt(dd[0]);
            for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = h1[i] + h2[i];
            H[(size_t)(j + 1) * m + j] = hn;
            if (hn > 0.0) rk_kscale<<<gb, RT_BS, 0, st>>>((float)(1.0 / hn), w, s->kv + (size_t)(j + 1) * len, len);
            // Givens rotations of the Hessenberg column
            for (int i = 0; i < j; ++i) {
                const double a0 = H[(size_t)i * m + j], a1 = H[(size_t)(i + 1) * m + j];
                H[(size_t)i * m + j] = cs[i] * a0 + sn[i] * a1;
                H[(size_t)(i + 1) * m + j] = -sn[i] * a0 + cs[i] * a1;
            }
            const double a0 = H[(size_t)j * m + j], a1 = H[(size_t)(j + 1) * m + j];
            const double r_ = std::sqrt(a0 * a0 + a1 * a1);
            cs[j] = r_ > 0.0 ? a0 / r_ : 1.0;
            sn[j] = r_ > 0.0 ? a1 / r_ : 0.0;
            H[(size_t)j * m + j] = r_;
            H[(size_t)(j + 1) * m + j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            jdone = j + 1;
            rel = std::fabs(g[j + 1]) / bnorm;
            if (rel < tol || hn == 0.0) break;
        }
        // x += V y, H y = g
        for (int i = jdone - 1; i >= 0; --i) {
            double t = g[i];
            for (int k = i + 1; k < jdone; ++k) t -= H[(size_t)i * m + k] * y[k];
            y[i] = t / H[(size_t)i * m + i];
        }
        std::vector<double> yy(y.begin(), y.begin() + jdone);
        if ((rc = comb(s->kv, yy, 1.0f, s->kx))) return rc;
        if (rel < tol) done = true;
        // stagnation: this cycle lowered the residual by less than stall of it
        if (stall > 0.0 && cycle_rel > 0.0 && cycle_rel - rel < stall * cycle_rel) done = true;
        cycle_rel = rel;
    }
    if ((rc = unpack(s, d, s->kx, st))) return rc;
    ACK(seeds(1));
    ACK(cudaStreamSynchronize(st));
    s->iters += nprod;
    if (steps) *steps = nprod;
    if (rel_residual) *rel_residual = rel;
    return rel < tol ? 0 : 1;
}

int32_t mgpu_adjoint_gradient(mgpu_handle *h) {
    AdjState *s = ready_state(h);
    if (!s) return api_fail(MGPU_E_STATE, "adjoint gradient before mgpu_adjoint_prepare");
    const Dev &d = handle_dev(h);
    cudaStream_t st = handle_view(h).stream;
    const size_t N = (size_t)d.IM * d.JM * d.KM;
    Adj &a = s->a;
    float *g[] = {a.gAQX, a.gAQR, a.gABX, a.gABR, a.gASX, a.gASR, a.gVOLOR};
    for (float *p : g) ACK(cudaMemsetAsync(p, 0, N * sizeof(float), st));
    ACK(cudaMemsetAsync(a.gABT, 0, (size_t)d.JM * d.KM * sizeof(float), st));
    Adj ag = a;
    ag.geom = 1;
    enqueue_reverse(d, ag, st);
    ACK(cudaGetLastError());
    ACK(cudaStreamSynchronize(st));
    return 0;
}

int32_t mgpu_adjoint_gradient_theta(mgpu_handle *h, float *djdtheta, int64_t nbytes) {
    AdjState *s = ready_state(h);
    if (!s || !djdtheta) return api_fail(MGPU_E_STATE, "adjoint THETA gradient before mgpu_adjoint_prepare");
    const Dev &d = handle_dev(h);
    const size_t N = (size_t)d.IM * d.JM * d.KM;
    if ((int64_t)(N * sizeof(float)) != nbytes) return api_fail(MGPU_E_ARG, "THETA gradient size mismatch");
    cudaStream_t st = handle_view(h).stream;
    float *gth = nullptr;
    ACK(cudaMallocAsync((void **)&gth, N * sizeof(float), st));
    ACK(cudaMemsetAsync(gth, 0, N * sizeof(float), st));
    rk_metrics<<<gridn(N, 256), 256, 0, st>>>(d, s->a, gth);
    ACK(cudaGetLastError());
    ACK(cudaMemcpyAsync(djdtheta, gth, N * sizeof(float), cudaMemcpyDeviceToHost, st));
    ACK(cudaFreeAsync(gth, st));
    ACK(cudaStreamSynchronize(st));
    return 0;
}

int32_t mgpu_adjoint_get(mgpu_handle *h, const char *name, float *out, int64_t nbytes) {
    AdjState *s = ready_state(h);
    if (!s || !name || !out) return api_fail(MGPU_E_STATE, "adjoint get before mgpu_adjoint_prepare");
    const Dev &d = handle_dev(h);
    size_t cnt = 0;
    float *p = state_adj(s, d, name, &cnt);
    if (!p && !strncmp(name, "d", 1)) p = geom_adj(s, d, name + 1, &cnt);
    if (!p) return api_fail(MGPU_E_ARG, (std::string("unknown adjoint array ") + name).c_str());
    if ((int64_t)(cnt * sizeof(float)) != nbytes) return api_fail(MGPU_E_ARG, "adjoint array size mismatch");
    cudaStream_t st = handle_view(h).stream;
    ACK(cudaMemcpyAsync(out, p, cnt * sizeof(float), cudaMemcpyDeviceToHost, st));
    ACK(cudaStreamSynchronize(st));
    return 0;
}

int32_t mgpu_adjoint_set(mgpu_handle *h, const char *name, const float *in, int64_t nbytes) {
    AdjState *s = ready_state(h);
    if (!s || !name || !in) return api_fail(MGPU_E_STATE, "adjoint set before mgpu_adjoint_prepare");
    const Dev &d = handle_dev(h);
    size_t cnt = 0;
    float *p = state_adj(s, d, name, &cnt);
    if (!p) return api_fail(MGPU_E_ARG, (std::string("unknown adjoint state array ") + name).c_str());
    if ((int64_t)(cnt * sizeof(float)) != nbytes) return api_fail(MGPU_E_ARG, "adjoint array size mismatch");
    cudaStream_t st = handle_view(h).stream;
    ACK(cudaMemcpyAsync(p, in, cnt * sizeof(float), cudaMemcpyHostToDevice, st));
    ACK(cudaStreamSynchronize(st));
    return 0;
}

}  // extern "C"
