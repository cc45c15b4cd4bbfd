// mgpu_noalloc.cu -- mgpu_integrals_noalloc: the EFICOOL integrals of
// mgpu_integrals_compute through a path that allocates nothing.
//
// mgpu_integrals_compute stages its node quantities in the handle's
// node-sized work arrays (TEMP1, TMP), its per-station sums in a buffer the
// handle allocated, and its host-side arithmetic in heap vectors.  Here one
// kernel forms the stagnation quantities at the four corners of each face
// on the fly and writes the four mass-weighted sums of each J station into
// a fixed static device array; a one-thread kernel turns the two stations'
// sums into the efficiencies beside them, and the host copies those six
// numbers into the caller's struct.  Per face and per station the
// arithmetic is the same expressions in the same order as
// mgpu_integrals_compute's, so the two agree to the last bits of the FP64
// efficiency formula (device pow against the host's).
//
// The scratch is a file-scope __device__ array: one copy per device in each
// process, its address looked up once per device with cudaGetSymbolAddress.
#include <cstdio>
#include <mutex>

#include "mgpu_internal.cuh"

// The scratch: 4 sums per J station (mass flow, flow-weighted PO/PO1, TO,
// P), then 8 result slots -- 131,136 bytes.  No slot needs to start at
// zero: each call writes every slot it later reads.
static __device__ __align__(256) double g_int_scratch[4 * MGPU_NOALLOC_MAX_JM + 8];

namespace mgpu {
namespace {

constexpr int NA_BS = 256;
constexpr int NA_MAX_DEVICES = 64;

std::mutex g_setup_mu;
double *g_scratch_addr[NA_MAX_DEVICES] = {};

// Stagnation temperature and stagnation-pressure ratio at one node: the
// node loop of EFICOOL (multall-open-18.3.f:10687-10739), with the same
// floors as mgpu_integrals_compute.
__device__ __forceinline__ void stag_node(const Dev &d, size_t n, float TO1M, float PO1M, float &tstag,
                                          float &pratio) {
    float vx = d.VX[n], vt = d.VT[n], vr = d.VR[n];
    float EKE = 0.5f * (vx * vx + vt * vt + vr * vr);
    float TS = (d.HO[n] - EKE) * d.RCP;
    float TSTAG = d.HO[n] * d.RCP;
    if (TSTAG < 0.1f * TO1M) TSTAG = 0.1f * TO1M;
    if (TS < 0.1f * TO1M) TS = 0.1f * TO1M;
    float PSTAT = d.P[n];
    if (PSTAT < 0.02f * PO1M) PSTAT = 0.02f * PO1M;
    float PSTAG = PSTAT * powf(TSTAG / TS, d.RFGA);
    tstag = TSTAG;
    pratio = PSTAG / PO1M;
}

// One CTA per J station: the SUMFLX mass averages (multall-open-18.3.f:
// 7873-7912) summed in the order of mgpu_integrals_compute's reduction.
__global__ void __launch_bounds__(NA_BS) k_int_sum_direct(Dev d, double *sums) {
    int j = blockIdx.x + 1;
    int ncell = d.IMM1 * d.KMM1;
    float TO1M = A1(d.TO1, d.KMID), PO1M = A1(d.PO1, d.KMID);
    double bf = 0, spo = 0, sto = 0, sps = 0;
    double nb = (double)A1(d.NBLADE, j);
    for (int c = threadIdx.x; c < ncell; c += NA_BS) {
        int i = c % d.IMM1 + 1, k = c / d.IMM1 + 1;
        size_t n00 = ix3(d, i, j, k), n10 = ix3(d, i + 1, j, k), n11 = ix3(d, i + 1, j, k + 1),
               n01 = ix3(d, i, j, k + 1);
        float t00, t10, t11, t01, r00, r10, r11, r01;
        stag_node(d, n00, TO1M, PO1M, t00, r00);
        stag_node(d, n10, TO1M, PO1M, t10, r10);
        stag_node(d, n11, TO1M, PO1M, t11, r11);
        stag_node(d, n01, TO1M, PO1M, t01, r01);
        double DFLOW = -(double)A3(d.FLOWX, i, j, k) * nb;
        double DFLOW4 = 0.25 * DFLOW;
        bf += DFLOW;
        spo += DFLOW4 * ((double)r00 + r10 + r11 + r01);
        sto += DFLOW4 * ((double)t00 + t10 + t11 + t01);
        sps += DFLOW4 * ((double)d.P[n00] + d.P[n10] + d.P[n11] + d.P[n01]);
    }
    __shared__ double sh[4][NA_BS / 32];
    double v[4] = {bf, spo, sto, sps};
    for (int q = 0; q < 4; ++q) {
        double x = v[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) sh[q][threadIdx.x >> 5] = x;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0.0;
        for (int w = 0; w < NA_BS / 32; ++w) t += sh[threadIdx.x][w];
        sums[(size_t)threadIdx.x * d.JM + (j - 1)] = t;
    }
}

// Whole-machine efficiencies (multall-open-18.3.f:11269-11394) from the
// inlet station J1 (1 for one stage, else 2) and the exit station JM-1.
__global__ void k_int_eta(Dev d, double *sums) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int JM = d.JM;
    int J1 = d.NSTAGES == 1 ? 1 : 2, J2M1 = JM - 1;
    double bf1 = sums[J1 - 1], bf2 = sums[J2M1 - 1];
    double PO1M = (double)A1(d.PO1, d.KMID);
    double FGA = (double)d.FGA;
    double POIN = sums[(size_t)JM + J1 - 1] / bf1 * PO1M;
    double PO2 = sums[(size_t)JM + J2M1 - 1] / bf2 * PO1M;
    double TO_IN = sums[(size_t)2 * JM + J1 - 1] / bf1;
    double TO_OUT = sums[(size_t)2 * JM + J2M1 - 1] / bf2;
    double PSOUT = sums[(size_t)3 * JM + J2M1 - 1] / bf2;
    double TORAT = TO_OUT / TO_IN, DELTO = TO_OUT - TO_IN, PORAT = PO2 / POIN, PSRAT = PSOUT / POIN;
    if (PORAT < 0.01) PORAT = 0.01;
    double TO2IS = pow(PORAT, FGA) * TO_IN, TSTAT2_IS = pow(PSRAT, FGA) * TO_IN;
    double DELTOIS = TO2IS - TO_IN, DELT_TOT_STAT = TSTAT2_IS - TO_IN;
    double ETAIS = 1.0, ETATS = 1.0;
    if (DELTO > 0.0) { ETAIS = DELTOIS / DELTO; ETATS = DELT_TOT_STAT / DELTO; }
    if (DELTO < 0.0) { ETAIS = DELTO / DELTOIS; ETATS = DELTO / DELT_TOT_STAT; }
    double *r = sums + (size_t)4 * JM;
    r[0] = bf1;
    r[1] = bf2;
    r[2] = ETAIS;
    r[3] = ETATS;
    r[4] = PORAT;
    r[5] = TORAT;
}

// Looks up (once per device, with that device current) the address of the
// static scratch, and loads the two kernels of this path, so that no later
// call loads a module.
int scratch_for_device(int dev, double **p) {
    char msg[160];
    if (dev < 0 || dev >= NA_MAX_DEVICES) {
        snprintf(msg, sizeof msg, "mgpu_integrals_noalloc: device %d beyond the %d supported", dev, NA_MAX_DEVICES);
        return api_fail(MGPU_E_ARG, msg);
    }
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void *a = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&a, g_int_scratch);
        if (e != cudaSuccess || a == nullptr) {
            snprintf(msg, sizeof msg, "mgpu_integrals_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return api_fail(MGPU_E_CUDA, msg);
        }
        // load both kernels now: under lazy module loading a kernel is
        // otherwise loaded at its first launch, which may take device memory
        cudaFuncAttributes fa;
        e = cudaFuncGetAttributes(&fa, k_int_sum_direct);
        if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_int_eta);
        if (e != cudaSuccess) {
            snprintf(msg, sizeof msg, "mgpu_integrals_noalloc: loading the kernels: %s", cudaGetErrorString(e));
            return api_fail(MGPU_E_CUDA, msg);
        }
        g_scratch_addr[dev] = (double *)a;
    }
    *p = g_scratch_addr[dev];
    return 0;
}

}  // namespace
}  // namespace mgpu

using namespace mgpu;

int32_t mgpu_integrals_noalloc(mgpu_handle *h, mgpu_integrals *out) {
    char msg[160];
    if (!h) return api_fail(MGPU_E_ARG, "mgpu_integrals_noalloc: null handle");
    HandleView v = handle_view(h);
    const Dev &d = *v.d;
    if (d.JM > MGPU_NOALLOC_MAX_JM) {
        snprintf(msg, sizeof msg, "mgpu_integrals_noalloc: JM=%d exceeds the fixed scratch (MGPU_NOALLOC_MAX_JM=%d)",
                 d.JM, MGPU_NOALLOC_MAX_JM);
        return api_fail(MGPU_E_ARG, msg);
    }
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) {
        snprintf(msg, sizeof msg, "mgpu_integrals_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
        return api_fail(MGPU_E_CUDA, msg);
    }
    if (cur != v.device) {
        snprintf(msg, sizeof msg, "mgpu_integrals_noalloc: device %d is current, the handle lives on device %d", cur,
                 v.device);
        return api_fail(MGPU_E_STATE, msg);
    }
    double *scratch = nullptr;
    int rc = scratch_for_device(v.device, &scratch);
    if (rc) return rc;
    if (!out) return 0;  // set-up only
    if (!v.committed) return api_fail(MGPU_E_STATE, "mgpu_integrals_noalloc: integrals before commit");
    if (d.JM < 2) return api_fail(MGPU_E_ARG, "mgpu_integrals_noalloc: JM < 2");

    k_int_sum_direct<<<d.JM, NA_BS, 0, v.stream>>>(d, scratch);
    k_int_eta<<<1, 32, 0, v.stream>>>(d, scratch);
    double res[6];
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(res, scratch + (size_t)4 * d.JM, sizeof res, cudaMemcpyDeviceToHost, v.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
    if (e != cudaSuccess) {
        snprintf(msg, sizeof msg, "mgpu_integrals_noalloc: %s", cudaGetErrorString(e));
        return api_fail(MGPU_E_CUDA, msg);
    }
    out->mass_flow_in = res[0];
    out->mass_flow_out = res[1];
    out->eta_tt = res[2];
    out->eta_ts = res[3];
    out->po_ratio = res[4];
    out->to_ratio = res[5];
    out->j1 = d.NSTAGES == 1 ? 1 : 2;
    out->j2m1 = d.JM - 1;
    return 0;
}
