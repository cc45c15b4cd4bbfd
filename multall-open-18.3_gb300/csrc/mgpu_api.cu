// mgpu_api.cu -- the C ABI of include/mgpu.h.
//
// A handle owns one flow problem on the current CUDA device: every COMMON
// array of the loop in HBM, the loop's work arrays, one stream and, after
// the first step, a CUDA graph holding the whole launch sequence of one
// LOOP iteration.  Arrays are bound by COMMON name (the table in
// include/mgpu_common_table.h).  No exception crosses the ABI: every entry
// point catches, records the message for mgpu_last_error() and returns a
// negative status.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "mgpu_internal.cuh"

using namespace mgpu;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return fail(MGPU_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

enum Shape { SH_IJK, SH_JK, SH_IK, SH_IJ, SH_J, SH_I, SH_K, SH_ROW, SH_MG1, SH_MG2, SH_SB };
enum Role { RO_GEOM, RO_OPT, RO_STATE, RO_OUT };

struct ArrayInfo {
    const char *name;
    bool is_int;
    Shape shape;
    Role role;
};

#define T_IS_INT_INT32 true
#define T_IS_INT_FLOAT32 false
const ArrayInfo kArrays[] = {
#define MGPU_AINFO(n, t, s, r) {#n, T_IS_INT_##t, SH_##s, RO_##r},
    MGPU_ARRAYS(MGPU_AINFO)
};
const int kNumArrays = sizeof(kArrays) / sizeof(kArrays[0]);

}  // namespace

struct mgpu_handle {
    Dev d;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;     // captures the bodies of conditional graph nodes
    cudaStream_t aux = nullptr;      // a parallel branch of the step graph (k_bc_sums)
    cudaStream_t aux2 = nullptr;     // another (the Spalart-Allmaras transport)
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_sa0 = nullptr, ev_sa1 = nullptr, ev_sa2 = nullptr;
    int device = 0;
    int sm_count = 0;
    bool committed = false;
    bool bound[sizeof(kArrays) / sizeof(kArrays[0])] = {};
    void *dptr[sizeof(kArrays) / sizeof(kArrays[0])] = {};
    size_t dbytes[sizeof(kArrays) / sizeof(kArrays[0])] = {};
    std::vector<void *> allocs;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    size_t graph_nodes = 0;
    size_t loss_nodes = 0, tail_nodes = 0;   // kernels in the conditional bodies
    double *d_int = nullptr;     // integrals output (4 x JM)
    void *flush_buf = nullptr;   // > L2, rewritten between timed iterations
    size_t flush_bytes = 0;
    DevCtl *h_ctl = nullptr;     // pinned mirror of the control block
    AdjState *adj = nullptr;     // discrete adjoint, after mgpu_adjoint_prepare
};

// A batch: one CUDA graph whose branches are the step graphs of several
// handles, forked from and joined back to the batch's own stream.
struct mgpu_batch {
    std::vector<mgpu_handle *> hs;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> joins;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    size_t graph_nodes = 0;
    void *flush_buf = nullptr;
    size_t flush_bytes = 0;
};

namespace {

size_t shape_count(const mgpu_handle *h, Shape s) {
    const Dev &d = h->d;
    switch (s) {
    case SH_IJK: return (size_t)d.IM * d.JM * d.KM;
    case SH_JK: return (size_t)d.JM * d.KM;
    case SH_IK: return (size_t)d.IM * d.KM;
    case SH_IJ: return (size_t)d.IM * d.JM;
    case SH_J: return d.JM;
    case SH_I: return d.IM;
    case SH_K: return d.KM;
    case SH_ROW: return d.NROWS;
    case SH_MG1: return (size_t)d.NIB1 * (d.NJB1 + 1) * d.NKB1;
    case SH_MG2: return (size_t)d.NIB2 * (d.NJB2 + 1) * d.NKB2;
    case SH_SB: return d.NSBLK;
    }
    return 0;
}

int find_array(const char *name) {
    for (int a = 0; a < kNumArrays; ++a)
        if (!strcmp(kArrays[a].name, name)) return a;
    return -1;
}

void **dev_slot(Dev &d, const char *name) {
#define MGPU_SLOT(n, t, s, r) if (!strcmp(name, #n)) return (void **)&d.n;
    MGPU_ARRAYS(MGPU_SLOT)
    return nullptr;
}

template <typename T>
int dalloc(mgpu_handle *h, T **p, size_t count) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 16);
    if (e != cudaSuccess) return fail(MGPU_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    e = cudaMemset(q, 0, count * sizeof(T) + 16);
    if (e != cudaSuccess) return fail(MGPU_E_CUDA, std::string("cudaMemset: ") + cudaGetErrorString(e));
    h->allocs.push_back(q);
    *p = (T *)q;
    return 0;
}

template <typename T>
int upload(mgpu_handle *h, T *dst, const std::vector<T> &src) {
    CK(cudaMemcpy(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
    return 0;
}

template <typename T>
int download(mgpu_handle *h, std::vector<T> &dst, const T *src, size_t n) {
    dst.resize(n);
    CK(cudaMemcpy(dst.data(), src, n * sizeof(T), cudaMemcpyDeviceToHost));
    return 0;
}

// the tables LOSS builds on its first call (multall-open-18.3.f:8123-8189)
void loss_tables(const Dev &d, const std::vector<float> &FP, const std::vector<float> &FR,
                 const std::vector<float> &X, const std::vector<float> &R, const std::vector<int> &NBLADE,
                 const std::vector<int> &JLE, const std::vector<int> &JTE, const std::vector<float> *XL,
                 std::vector<float> &FILAM, std::vector<float> &FITURB, std::vector<float> &FIWAKE,
                 std::vector<float> &FIUP, std::vector<float> &FKLAM, std::vector<float> &FKTURB) {
    const int IM = d.IM, KM = d.KM, IMM1 = d.IMM1, KMM1 = d.KMM1, JM = d.JM, KMID = d.KMID;
    FILAM.assign((size_t)d.NROWS * IM, 0.f);
    FITURB = FIWAKE = FIUP = FILAM;
    FKLAM.assign((size_t)d.NROWS * KM, 0.f);
    FKTURB = FKLAM;
    auto fp = [&](int i) { return FP[i - 1]; };
    auto fr = [&](int k) { return FR[k - 1]; };
    auto x2 = [&](int j, int k) { return X[(size_t)(j - 1) + (size_t)JM * (k - 1)]; };
    auto r2 = [&](int j, int k) { return R[(size_t)(j - 1) + (size_t)JM * (k - 1)]; };
    for (int nrw = 1; nrw <= d.NROWS; ++nrw) {
        float XI1 = XL[0][nrw - 1], XIM = XL[1][nrw - 1], XK1 = XL[2][nrw - 1], XKM = XL[3][nrw - 1];
        float XDWN = XL[4][nrw - 1], XUP = XL[5][nrw - 1];
        auto at = [&](std::vector<float> &v, int i) -> float & { return v[(size_t)(nrw - 1) * IM + i - 1]; };
        auto atk = [&](std::vector<float> &v, int k) -> float & { return v[(size_t)(nrw - 1) * KM + k - 1]; };
        float SUMF = 0.0f;
        for (int i = 2; i <= IMM1; ++i) {
            SUMF = SUMF + fp(i - 1);
            float XLIM = XI1 * (1.0f - SUMF) + XIM * SUMF;
            float FPITCH = SUMF * (1.0f - SUMF);
            if (FPITCH > XLIM) FPITCH = XLIM;
            float DF = fp(i) + fp(i - 1);
            at(FILAM, i) = fp(i) / DF;
            at(FITURB, i) = 0.16f * FPITCH * FPITCH / (DF * DF);
            at(FIWAKE, i) = 0.16f * XDWN * XDWN / (DF * DF);
            at(FIUP, i) = 0.16f * XUP * XUP / (DF * DF);
        }
        float DF = fp(1) + fp(IMM1);
        at(FILAM, 1) = fp(1) / DF;
        at(FIWAKE, 1) = 0.16f * XDWN * XDWN / (DF * DF);
        at(FIUP, 1) = 0.16f * XUP * XUP / (DF * DF);
        at(FITURB, 1) = at(FITURB, 2);
        at(FILAM, IM) = fp(IMM1) / DF;
        at(FIWAKE, IM) = 0.16f * XDWN * XDWN / (DF * DF);
        at(FIUP, IM) = 0.16f * XUP * XUP / (DF * DF);
        at(FITURB, IM) = at(FITURB, IMM1);
        float AVGSPAN = 0.0f;
        int JMID = (int)(0.5f * (float)(JLE[nrw - 1] + JTE[nrw - 1]));
        for (int k = 2; k <= KM; ++k) {
            float XDIF = x2(JMID, k) - x2(JMID, k - 1);
            float RDIF = r2(JMID, k) - r2(JMID, k - 1);
            AVGSPAN = AVGSPAN + sqrtf(XDIF * XDIF + RDIF * RDIF);
        }
        float AVGPIT = 2.0f * 3.1415926f * r2(JMID, KMID) / (float)NBLADE[JMID - 1];
        float XLIMH = XK1 * AVGPIT / AVGSPAN;
        float XLIMT = XKM * AVGPIT / AVGSPAN;
        SUMF = 0.0f;
        for (int k = 2; k <= KMM1; ++k) {
            SUMF = SUMF + fr(k - 1);
            float XLIM = XLIMH * (1.0f - SUMF) + XLIMT * SUMF;
            float FCSPAN = SUMF * (1.0f - SUMF);
            if (FCSPAN > XLIM) FCSPAN = XLIM;
            float DFk = fr(k) + fr(k - 1);
            atk(FKLAM, k) = fr(k) / DFk;
            atk(FKTURB, k) = 0.16f * FCSPAN * FCSPAN / (DFk * DFk);
        }
    }
}

// contiguous extent of each block of a 1-based map over [lo, hi]
int extents(const std::vector<int> &map, int lo, int hi, int nblk, std::vector<int> &s, std::vector<int> &e,
            const char *what) {
    s.assign(nblk, 1 << 30);
    e.assign(nblk, -1);
    for (int x = lo; x <= hi; ++x) {
        int b = map[x - 1];
        if (b < 1 || b > nblk) continue;
        if (e[b - 1] >= 0 && e[b - 1] != x - 1)
            return fail(MGPU_E_ARG, std::string("non-contiguous multigrid block in ") + what);
        if (s[b - 1] > x) s[b - 1] = x;
        e[b - 1] = x;
    }
    for (int b = 0; b < nblk; ++b)
        if (e[b] < 0) {
            s[b] = 1;
            e[b] = 0;
        }
    return 0;
}

// keeps the GPU busy for ~cycles clocks so that a burst of launches queued
// behind it runs back to back (used only when profiling); always ends
__global__ void k_delay(long long cycles) {
    long long t0 = clock64();
    while (clock64() - t0 < cycles) {
    }
}

// the launch sequence of one LOOP iteration
// The reference updates RO, ROE, ROVX, RORVT, ROVR one after the other,
// each TSTEP reading only its own fluxes and the start-of-step primitives;
// the only coupling is the inlet/exit condition, which reads the new RO and
// ROE and resets the momenta at J=1 before their update.  So the step runs
// two batched TSTEPs, [RO, ROE] and [ROVX, RORVT, ROVR], with the boundary
// conditions between them; every value is the same as in the serial order.
// join: when the step is captured as a graph, k_bc_sums already runs on a
// branch forked after k_prim (capture_step) and join marks its end
// A second parallel branch of the step graph for the Spalart-Allmaras
// model: the transported viscosity's fluxes and TSTEP read the mass fluxes,
// the cell-average density and the model's own arrays, none of which the
// inlet/exit conditions, the momentum fluxes or TSTEP of the momenta write,
// and these read nothing it writes.  Its inlet value (4679-4689) follows the
// conditions; the limiters, which may change the density it reads there,
// wait for it.
struct SaBranch {
    cudaStream_t s = nullptr;
    cudaEvent_t start = nullptr, bc = nullptr, done = nullptr;
};

void enqueue_core(const Dev &d, Launch L, cudaEvent_t join = nullptr, const SaBranch *sa = nullptr) {
    Launch L0 = L;        // follows the LOSS conditional node: plain stream order
    L0.pdl = false;
    launch_flux_mass_energy(d, L0);
    launch_tstep(d, L, V_RO, 2);
    if (d.ILOS >= 100) launch_roavg_cell(d, L);     // 4255-4267, after TSTEP(RO)
    const bool sab = sa && sa->s && d.ILOS >= 200;
    if (sab) {
        cudaEventRecord(sa->start, L.s);
        cudaStreamWaitEvent(sa->s, sa->start, 0);
        launch_sa_transport(d, Launch{sa->s, L.sm_count, nullptr});   // 4279-4347
    } else if (d.ILOS >= 200) {
        launch_sa_transport(d, L);                  // 4279-4347, after the cell-average density
    }
    if (join) {
        cudaStreamWaitEvent(L.s, join, 0);
        launch_bc_apply(d, L0);
    } else {
        launch_bc_sums(d, L);
        launch_bc_apply(d, L);
    }
    if (sab) {
        cudaEventRecord(sa->bc, L.s);
        cudaStreamWaitEvent(sa->s, sa->bc, 0);
        launch_sa_inlet(d, Launch{sa->s, L.sm_count, nullptr});       // 4679-4689
        cudaEventRecord(sa->done, sa->s);
    } else if (d.ILOS >= 200) {
        launch_sa_inlet(d, L);
    }
    if (d.IN_FLOW != 0) launch_setflo(d, L);
    launch_flux_mom(d, L);          // also PEFF and the density limiter's column flags
    launch_tstep(d, L, V_ROVX, 3);
    if (sab) {
        cudaStreamWaitEvent(L.s, sa->done, 0);
        launch_limiters(d, L0);
    } else {
        launch_limiters(d, L);
    }
    launch_mixplan(d, L);
    if (d.any_cusp2) launch_cusp(d, L);
}

void enqueue_tail(const Dev &d, Launch L) {
    launch_tail(d, L);
    launch_stepup(d, L, 0.25f, true);
}

// kernel by kernel, every kernel present (LOSS and tail kernels return
// early when their flag is off); used for profiling
int enqueue_step(mgpu_handle *h, Prof *prof = nullptr) {
    const Dev &d = h->d;
    Launch L{h->stream, h->sm_count, prof};
    launch_step_begin(d, L);
    launch_prim(d, L);
    launch_loss(d, L, false);
    enqueue_core(d, L);
    enqueue_tail(d, L);
    CK(cudaGetLastError());
    return 0;
}

// appends an IF conditional node to the graph being captured on h->stream
// and captures its body (fn) on the side stream; *nbody = the body's nodes
template <typename F>
int add_conditional(mgpu_handle *h, cudaGraphConditionalHandle hnd, size_t *nbody, F fn) {
    cudaStreamCaptureStatus st;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    CK(cudaStreamGetCaptureInfo(h->stream, &st, nullptr, &cg, &deps, nullptr, &ndeps));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = hnd;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, cg, deps, nullptr, ndeps, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    CK(cudaStreamBeginCaptureToGraph(h->side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    fn(Launch{h->side, h->sm_count, nullptr});
    cudaGraph_t out = nullptr;
    CK(cudaStreamEndCapture(h->side, &out));
    CK(cudaGraphGetNodes(body, nullptr, nbody));
    CK(cudaStreamUpdateCaptureDependencies(h->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    return 0;
}

// Records one LOOP iteration of h on h->stream, which must be capturing
// (alone, or as one branch of a batch graph): the LOSS and tail kernels sit
// in conditional bodies that the step-control kernel switches on only on
// the steps that need them.
int capture_step(mgpu_handle *h) {
    cudaStreamCaptureStatus st;
    cudaGraph_t cg = nullptr;
    CK(cudaStreamGetCaptureInfo(h->stream, &st, nullptr, &cg, nullptr, nullptr, nullptr));
    cudaGraphConditionalHandle hl = 0, ht = 0;
    // every handle of a graph belongs to one conditional node: an inviscid
    // problem (ILOS = 0), which has no LOSS node, creates no LOSS handle
    if (h->d.ILOS != 0) CK(cudaGraphConditionalHandleCreate(&hl, cg, 0, cudaGraphCondAssignDefault));
    CK(cudaGraphConditionalHandleCreate(&ht, cg, 0, cudaGraphCondAssignDefault));
    Dev dg = h->d;
    dg.use_cond = 1;
    dg.cond_loss = (unsigned long long)hl;
    dg.cond_tail = (unsigned long long)ht;
    Launch L{h->stream, h->sm_count, nullptr};
    launch_step_begin(dg, L);
    L.pdl = true;          // kernel-to-kernel edges of the step are programmatic
    launch_prim(dg, L);
    // the exit-pressure sums depend on nothing the next kernels write, so they
    // run beside LOSS, the mass/energy fluxes and TSTEP(RO, ROE)
    CK(cudaEventRecord(h->ev_fork, h->stream));
    CK(cudaStreamWaitEvent(h->aux, h->ev_fork, 0));
    launch_bc_sums(dg, Launch{h->aux, h->sm_count, nullptr});
    CK(cudaEventRecord(h->ev_join, h->aux));
    // an inviscid problem (ILOS = 0) has no LOSS node
    int rc = dg.ILOS == 0 ? 0 : add_conditional(h, hl, &h->loss_nodes, [&](Launch L2) { launch_loss(dg, L2, false); });
    SaBranch sab{h->aux2, h->ev_sa0, h->ev_sa1, h->ev_sa2};
    if (!rc) enqueue_core(dg, L, h->ev_join, &sab);
    if (!rc) rc = add_conditional(h, ht, &h->tail_nodes, [&](Launch L2) { enqueue_tail(dg, L2); });
    return rc;
}

// one LOOP iteration of h as a CUDA graph
int build_graph(mgpu_handle *h) {
    if (h->gexec) return 0;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rc = capture_step(h);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return fail(MGPU_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    h->graph = g;
    CK(cudaGraphGetNodes(g, nullptr, &h->graph_nodes));
    CK(cudaGraphInstantiate(&h->gexec, g, 0));
    return 0;
}

void fill_monitors(const DevCtl &c, mgpu_monitors *m) {
    memset(m, 0, sizeof(*m));
    m->nstep = c.nstep;
    m->tail_ran = c.do_tail;
    m->ifend = c.ifend;
    m->health = c.health;
    m->emax = c.EMAX;
    m->imax = c.IMAXE;
    m->jmax = c.JMAXE;
    m->kmax = c.KMAXE;
    m->eavg = c.EAVG;
    m->econt = c.ECONT;
    m->jcont = c.JCONT;
    m->vref = c.VREF;
    m->vmax = c.VMAX;
    m->ivmax = c.IVMAX;
    m->jvmax = c.JVMAX;
    m->kvmax = c.KVMAX;
    m->flow_in = c.flow_in;
    m->flow_out = c.flow_out;
}

int read_ctl(mgpu_handle *h) {
    CK(cudaMemcpyAsync(h->h_ctl, h->d.ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

}  // namespace

namespace mgpu {

HandleView handle_view(const mgpu_handle *h) { return HandleView{&h->d, h->stream, h->device, h->committed}; }

int api_fail(int code, const char *msg) { return fail(code, msg); }

void enqueue_step_core(const Dev &d, Launch L) { enqueue_core(d, L); }
AdjState *&handle_adj(mgpu_handle *h) { return h->adj; }
Dev &handle_dev(mgpu_handle *h) { return h->d; }
int handle_sm_count(const mgpu_handle *h) { return h->sm_count; }
double *handle_int_buf(mgpu_handle *h) { return h->d_int; }
const void *handle_array(const mgpu_handle *h, const char *name, size_t *bytes) {
    int a = find_array(name);
    if (a < 0 || !h->dptr[a]) return nullptr;
    if (bytes) *bytes = h->dbytes[a];
    return h->dptr[a];
}

}  // namespace mgpu

extern "C" {

int32_t mgpu_abi_version(void) { return MGPU_ABI_VERSION; }

int32_t mgpu_last_error(char *buf, int32_t len) {
    if (!buf || len <= 0) return MGPU_E_ARG;
    snprintf(buf, (size_t)len, "%s", g_err.c_str());
    return 0;
}

int32_t mgpu_device_count(void) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) return fail(MGPU_E_CUDA, cudaGetErrorString(e));
    return n;
}

int32_t mgpu_create(int32_t im, int32_t jm, int32_t km, int32_t nrows, mgpu_handle **out) {
    if (!out) return fail(MGPU_E_ARG, "null handle pointer");
    *out = nullptr;
    if (im < 5 || jm < 10 || km < 5 || nrows < 1 || nrows > 64)
        return fail(MGPU_E_ARG, "dimensions out of range (IM,KM >= 5, JM >= 10, 1 <= NROWS <= 64)");
    if (im > 160 || km > 160) return fail(MGPU_E_UNSUPPORTED, "IM and KM above 160 are not covered");
    if ((int64_t)im * jm * km > (int64_t)1 << 30)
        return fail(MGPU_E_UNSUPPORTED, "more than 2^30 nodes are not covered (32-bit node indices)");
    mgpu_handle *h = new (std::nothrow) mgpu_handle();
    if (!h) return fail(MGPU_E_NOMEM, "host allocation");
    Dev &d = h->d;
    memset(&d, 0, sizeof(d));
    d.IM = im; d.JM = jm; d.KM = km; d.NROWS = nrows;
    d.IMM1 = im - 1; d.JMM1 = jm - 1; d.KMM1 = km - 1;
    d.IMM2 = im - 2; d.JMM2 = jm - 2; d.KMM2 = km - 2;
    d.IMID = (int)(0.5f * im);
    d.KMID = (int)(0.5f * km);
    d.NRWSM1 = nrows - 1;
    d.ts_bs[0] = d.ts_bs[1] = 256;
#define MGPU_DEF_I(n, v) d.n = v;
    MGPU_INT_SCALARS(MGPU_DEF_I)
#define MGPU_DEF_R(n, v) d.n = v;
    MGPU_REAL_SCALARS(MGPU_DEF_R)
    int rc = 0;
    auto bail = [&](int code) {
        mgpu_destroy(h);
        return code;
    };
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) return bail(fail(MGPU_E_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e)));
    cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->device);
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(fail(MGPU_E_CUDA, cudaGetErrorString(e)));
    e = cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(fail(MGPU_E_CUDA, cudaGetErrorString(e)));
    e = cudaStreamCreateWithFlags(&h->aux, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->aux2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_sa0, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_sa1, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_sa2, cudaEventDisableTiming);
    if (e != cudaSuccess) return bail(fail(MGPU_E_CUDA, cudaGetErrorString(e)));
    // arrays whose size is known now
    for (int a = 0; a < kNumArrays; ++a) {
        Shape s = kArrays[a].shape;
        if (s == SH_MG1 || s == SH_MG2 || s == SH_SB) continue;
        size_t cnt = shape_count(h, s);
        void **slot = dev_slot(d, kArrays[a].name);
        if (kArrays[a].is_int) rc = dalloc(h, (int32_t **)slot, cnt);
        else rc = dalloc(h, (float **)slot, cnt);
        if (rc) return bail(rc);
        h->dptr[a] = *slot;
        h->dbytes[a] = cnt * 4;
    }
    size_t N = (size_t)im * jm * km;
    float **work[] = {&d.FLOWX, &d.FLOWT, &d.FLOWR, &d.ZERO, &d.TEMP1};
    for (float **w : work)
        if ((rc = dalloc(h, w, N))) return bail(rc);
    // per-variable TSTEP operands; RO's face fluxes are the mass fluxes
    float *vd[NVAR] = {d.RO, d.ROE, d.ROVX, d.RORVT, d.ROVR};
    float *vdiff[NVAR] = {d.DRO, d.DROE, d.DROVX, d.DRORVT, d.DROVR};
    for (int v = 0; v < NVAR; ++v) {
        VarSet &V = d.var[v];
        V.D = vd[v];
        V.DIFF = vdiff[v];
        if (v == V_RO) {
            V.XF = d.FLOWX;
            V.TF = d.FLOWT;
            V.RF = d.FLOWR;
            V.SR = d.ZERO;
        } else {
            float **fl[] = {&V.XF, &V.TF, &V.RF, &V.SR};
            for (float **w : fl)
                if ((rc = dalloc(h, w, N))) return bail(rc);
        }
        if ((rc = dalloc(h, &V.ST, N)) || (rc = dalloc(h, &V.TM, N)) || (rc = dalloc(h, &V.psum, jm)) ||
            (rc = dalloc(h, &V.pabs, jm)) || (rc = dalloc(h, &V.AVG_BLK, nrows)))
            return bail(rc);
    }
    d.STORE = d.var[V_RO].ST;
    d.TMP = d.var[V_RO].TM;
    if ((rc = dalloc(h, &d.PLIM, km))) return bail(rc);
    float **rowt[] = {&d.FILAM, &d.FITURB, &d.FIWAKE, &d.FIUP};
    for (float **w : rowt)
        if ((rc = dalloc(h, w, (size_t)nrows * im))) return bail(rc);
    if ((rc = dalloc(h, &d.FKLAM, (size_t)nrows * km))) return bail(rc);
    if ((rc = dalloc(h, &d.FKTURB, (size_t)nrows * km))) return bail(rc);
    if ((rc = dalloc(h, &d.VLIMIT, nrows))) return bail(rc);
    if ((rc = dalloc(h, &d.ROLIMIT, nrows))) return bail(rc);
    if ((rc = dalloc(h, &d.BLADE_FLOW, jm))) return bail(rc);
    if ((rc = dalloc(h, &d.DFLAG, (size_t)im * km))) return bail(rc);
    if ((rc = dalloc(h, &d.BCBUF, (size_t)4 * km))) return bail(rc);
    if ((rc = dalloc(h, &d.FLOWJ, jm))) return bail(rc);
    d.nparts = (int)((N + 255) / 256) + 1;
    if ((rc = dalloc(h, &d.part_sum, d.nparts))) return bail(rc);
    if ((rc = dalloc(h, &d.part_key, d.nparts))) return bail(rc);
    if ((rc = dalloc(h, &d.part_cnt, d.nparts))) return bail(rc);
    if ((rc = dalloc(h, &d.ctl, 1))) return bail(rc);
    if ((rc = dalloc(h, &h->d_int, (size_t)4 * jm))) return bail(rc);
    e = cudaMallocHost((void **)&h->h_ctl, sizeof(DevCtl));
    if (e != cudaSuccess) return bail(fail(MGPU_E_NOMEM, cudaGetErrorString(e)));
    *out = h;
    return 0;
}

void mgpu_destroy(mgpu_handle *h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->adj) adj_destroy(h->adj);
    if (h->flush_buf) cudaFree(h->flush_buf);
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    if (h->graph) cudaGraphDestroy(h->graph);
    for (void *p : h->allocs) cudaFree(p);
    if (h->h_ctl) cudaFreeHost(h->h_ctl);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->aux) cudaStreamDestroy(h->aux);
    if (h->aux2) cudaStreamDestroy(h->aux2);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    for (cudaEvent_t ev : {h->ev_sa0, h->ev_sa1, h->ev_sa2})
        if (ev) cudaEventDestroy(ev);
    delete h;
}

int32_t mgpu_set_int(mgpu_handle *h, const char *name, int32_t value) {
    if (!h || !name) return fail(MGPU_E_ARG, "null argument");
    if (h->committed) return fail(MGPU_E_STATE, "scalars are fixed after commit");
#define MGPU_SETI(n, v) if (!strcmp(name, #n)) { h->d.n = value; return 0; }
    MGPU_INT_SCALARS(MGPU_SETI)
    return fail(MGPU_E_ARG, std::string("unknown integer scalar ") + name);
}

int32_t mgpu_set_real(mgpu_handle *h, const char *name, float value) {
    if (!h || !name) return fail(MGPU_E_ARG, "null argument");
    if (h->committed) return fail(MGPU_E_STATE, "scalars are fixed after commit");
#define MGPU_SETR(n, v) if (!strcmp(name, #n)) { h->d.n = value; return 0; }
    MGPU_REAL_SCALARS(MGPU_SETR)
    return fail(MGPU_E_ARG, std::string("unknown real scalar ") + name);
}

int32_t mgpu_get_real(mgpu_handle *h, const char *name, float *value) {
    if (!h || !name || !value) return fail(MGPU_E_ARG, "null argument");
    if (h->committed && (!strcmp(name, "VISLAM") || !strcmp(name, "FTCOND") || !strcmp(name, "SFT") ||
                         !strcmp(name, "SFX") || !strcmp(name, "DAMP") || !strcmp(name, "FMIXUP") ||
                         !strcmp(name, "PDOWN_HUB") || !strcmp(name, "PDOWN_TIP") || !strcmp(name, "THROTTLE_PRES"))) {
        int rc = read_ctl(h);
        if (rc) return rc;
        const DevCtl &c = *h->h_ctl;
        if (!strcmp(name, "VISLAM")) *value = c.VISLAM;
        else if (!strcmp(name, "FTCOND")) *value = c.FTCOND;
        else if (!strcmp(name, "SFT")) *value = c.SFT;
        else if (!strcmp(name, "SFX")) *value = c.SFX;
        else if (!strcmp(name, "DAMP")) *value = c.DAMP;
        else if (!strcmp(name, "PDOWN_HUB")) *value = c.PDOWN_HUB;
        else if (!strcmp(name, "PDOWN_TIP")) *value = c.PDOWN_TIP;
        else if (!strcmp(name, "THROTTLE_PRES")) *value = c.THROTTLE_PRES;
        else *value = c.FMIXUP;
        return 0;
    }
    if (!strcmp(name, "PREFF")) { *value = h->d.PREFF; return 0; }
#define MGPU_GETR(n, v) if (!strcmp(name, #n)) { *value = h->d.n; return 0; }
    MGPU_REAL_SCALARS(MGPU_GETR)
    return fail(MGPU_E_ARG, std::string("unknown real scalar ") + name);
}

int32_t mgpu_get_int(mgpu_handle *h, const char *name, int32_t *value) {
    if (!h || !name || !value) return fail(MGPU_E_ARG, "null argument");
    if (!strcmp(name, "NSTEP") && h->committed) {
        int rc = read_ctl(h);
        if (rc) return rc;
        *value = h->h_ctl->nstep;
        return 0;
    }
#define MGPU_GETI(n, v) if (!strcmp(name, #n)) { *value = h->d.n; return 0; }
    MGPU_INT_SCALARS(MGPU_GETI)
    return fail(MGPU_E_ARG, std::string("unknown integer scalar ") + name);
}

int32_t mgpu_set_array(mgpu_handle *h, const char *name, const void *host, int64_t nbytes) {
    if (!h || !name || !host) return fail(MGPU_E_ARG, "null argument");
    int a = find_array(name);
    if (a < 0) return fail(MGPU_E_ARG, std::string("unknown array ") + name);
    if (kArrays[a].role == RO_OUT) return fail(MGPU_E_ARG, std::string("array is output only: ") + name);
    if (h->committed && kArrays[a].role != RO_STATE)
        return fail(MGPU_E_STATE, std::string("geometry is fixed after commit: ") + name);
    Shape s = kArrays[a].shape;
    if ((s == SH_MG1 || s == SH_MG2 || s == SH_SB) && !h->dptr[a]) {
        Dev &d = h->d;
        if ((s == SH_MG1 && (d.NIB1 <= 0 || d.NJB1 <= 0 || d.NKB1 <= 0)) ||
            (s == SH_MG2 && (d.NIB2 <= 0 || d.NJB2 <= 0 || d.NKB2 <= 0)) || (s == SH_SB && d.NSBLK <= 0))
            return fail(MGPU_E_STATE, std::string("set the multigrid block counts before ") + name);
        size_t cnt = shape_count(h, s);
        void **slot = dev_slot(d, name);
        int rc = dalloc(h, (float **)slot, cnt);
        if (rc) return rc;
        h->dptr[a] = *slot;
        h->dbytes[a] = cnt * 4;
    }
    size_t want = shape_count(h, s) * 4;
    if ((size_t)nbytes != want)
        return fail(MGPU_E_ARG, std::string("size mismatch for ") + name + ": expected " + std::to_string(want) +
                                    " bytes, got " + std::to_string(nbytes));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(h->dptr[a], host, want, cudaMemcpyHostToDevice));
    h->bound[a] = true;
    return 0;
}

int32_t mgpu_get_array(mgpu_handle *h, const char *name, void *host, int64_t nbytes) {
    if (!h || !name || !host) return fail(MGPU_E_ARG, "null argument");
    int a = find_array(name);
    const void *src = nullptr;
    size_t want = 0;
    if (a >= 0) {
        src = h->dptr[a];
        want = shape_count(h, kArrays[a].shape) * 4;
        if (!src) return fail(MGPU_E_STATE, std::string("array not allocated: ") + name);
    } else {
        size_t N = (size_t)h->d.IM * h->d.JM * h->d.KM;
        if (!strcmp(name, "FLOWX")) src = h->d.FLOWX;
        else if (!strcmp(name, "STORE")) src = h->d.STORE;
        else return fail(MGPU_E_ARG, std::string("unknown array ") + name);
        want = N * 4;
    }
    if ((size_t)nbytes != want) return fail(MGPU_E_ARG, std::string("size mismatch for ") + name);
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(host, src, want, cudaMemcpyDeviceToHost));
    return 0;
}

int32_t mgpu_setup_metrics(mgpu_handle *h) {
    if (!h) return fail(MGPU_E_ARG, "null handle");
    if (h->committed) return fail(MGPU_E_STATE, "setup_metrics after commit: the geometry is fixed by then");
    for (const char *n : {"X", "R", "RTHETA", "INDMIX", "WRAD"})
        if (!h->bound[find_array(n)]) return fail(MGPU_E_STATE, std::string("setup_metrics needs ") + n);
    const Dev &d = h->d;
    const size_t N = (size_t)d.IM * d.JM * d.KM;
    float *work = nullptr;
    CK(cudaMalloc(&work, 3 * N * sizeof(float)));
    auto P = [&](const char *n) { return (float *)h->dptr[find_array(n)]; };
    MetricArgs<float> a{P("X"), P("R"), P("RTHETA"), (const int *)h->dptr[find_array("INDMIX")], P("WRAD"),
                        work, work + N, work + 2 * N, P("AQX"), P("AQR"), P("ABX"), P("ABR"), P("VOL"), P("ASX"),
                        P("ASR"), P("VOLOR"), P("ABT"), P("WRABT")};
    cudaError_t e = launch_setup_metrics(d.IM, d.JM, d.KM, a, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(work);
    if (e != cudaSuccess) return fail(MGPU_E_CUDA, std::string("setup_metrics: ") + cudaGetErrorString(e));
    for (const char *n : {"AQX", "AQR", "ABX", "ABR", "VOL", "ASX", "ASR", "VOLOR", "ABT", "WRABT"})
        h->bound[find_array(n)] = true;
    return 0;
}

int32_t mgpu_setup_geometry(mgpu_handle *h, int32_t nsecs, const float *sections, const float *fthick,
                            const float *fractip) {
    if (!h || !sections || !fthick || !fractip) return fail(MGPU_E_ARG, "null argument");
    if (h->committed) return fail(MGPU_E_STATE, "setup_geometry after commit: the geometry is fixed by then");
    if (nsecs < 2 || nsecs > 32) return fail(MGPU_E_ARG, "setup_geometry: 2 to 32 blade sections");
    for (const char *n : {"FR", "FP", "NROW", "NBLADE", "INDMIX", "JSTART", "JLE", "JTE", "JMIX", "KTIPS", "KTIPE", "KS1",
                          "KS2", "WRAD"})
        if (!h->bound[find_array(n)]) return fail(MGPU_E_STATE, std::string("setup_geometry needs ") + n);
    const Dev &d = h->d;
    const size_t JK = (size_t)d.JM * d.KM, ns = (size_t)nsecs;
    const size_t n_sec = 4 * ns * d.JM, n_fth = (size_t)d.NROWS * d.KM, n_frt = 2 * (size_t)d.NROWS;
    float *buf = nullptr;
    const size_t total = n_sec + n_fth + n_frt + ns * d.JM + d.JM + JK;
    CK(cudaMalloc(&buf, total * sizeof(float)));
    float *dsec = buf, *dfth = dsec + n_sec, *dfrt = dfth + n_fth, *dsm = dfrt + n_frt, *dsh = dsm + ns * d.JM,
          *drtu = dsh + d.JM;
    cudaError_t e = cudaMemcpyAsync(dsec, sections, n_sec * sizeof(float), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dfth, fthick, n_fth * sizeof(float), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dfrt, fractip, n_frt * sizeof(float), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        auto F = [&](const char *n) { return (float *)h->dptr[find_array(n)]; };
        auto I = [&](const char *n) { return (const int *)h->dptr[find_array(n)]; };
        GeoArgs g{d.IM, d.JM, d.KM, nsecs, d.KMID, dsec, F("FR"), F("FP"), I("NROW"), I("NBLADE"), I("INDMIX"),
                  I("JSTART"), I("JLE"), I("JTE"), I("JMIX"), I("KTIPS"), I("KTIPE"), I("KS1"), I("KS2"), dfrt, dfth,
                  dsm, dsh, F("X"), F("R"), drtu, F("RT_THICK"), F("RTHETA")};
        e = launch_setup_geometry(g, h->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(buf);
    if (e != cudaSuccess) return fail(MGPU_E_CUDA, std::string("setup_geometry: ") + cudaGetErrorString(e));
    for (const char *n : {"X", "R", "RT_THICK", "RTHETA"}) h->bound[find_array(n)] = true;
    return mgpu_setup_metrics(h);
}

int32_t mgpu_setup_metrics64(mgpu_handle *h, const double *x, const double *r, const double *rtheta, double *out,
                             int64_t n_out) {
    if (!h || !x || !r || !rtheta || !out) return fail(MGPU_E_ARG, "null argument");
    for (const char *n : {"INDMIX", "WRAD"})
        if (!h->bound[find_array(n)]) return fail(MGPU_E_STATE, std::string("setup_metrics64 needs ") + n);
    const Dev &d = h->d;
    const size_t N = (size_t)d.IM * d.JM * d.KM, JK = (size_t)d.JM * d.KM;
    if (n_out != (int64_t)(8 * N + 2 * JK))
        return fail(MGPU_E_ARG, "setup_metrics64: out holds 8*IM*JM*KM + 2*JM*KM doubles");
    double *buf = nullptr;
    const size_t total = 2 * JK + N + 3 * N + 8 * N + 2 * JK;
    CK(cudaMalloc(&buf, total * sizeof(double)));
    double *dx = buf, *dr = dx + JK, *drt = dr + JK, *work = drt + N, *o = work + 3 * N;
    cudaError_t e = cudaMemcpyAsync(dx, x, JK * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dr, r, JK * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(drt, rtheta, N * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(o, 0, (8 * N + 2 * JK) * sizeof(double), h->stream);
    if (e == cudaSuccess) {
        MetricArgs<double> a{dx, dr, drt, (const int *)h->dptr[find_array("INDMIX")],
                             (const float *)h->dptr[find_array("WRAD")], work, work + N, work + 2 * N,
                             o, o + N, o + 2 * N, o + 3 * N, o + 4 * N, o + 5 * N, o + 6 * N, o + 7 * N,
                             o + 8 * N, o + 8 * N + JK};
        e = launch_setup_metrics(d.IM, d.JM, d.KM, a, h->stream);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, o, (8 * N + 2 * JK) * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(buf);
    if (e != cudaSuccess) return fail(MGPU_E_CUDA, std::string("setup_metrics64: ") + cudaGetErrorString(e));
    return 0;
}

int32_t mgpu_commit(mgpu_handle *h) {
    if (!h) return fail(MGPU_E_ARG, "null handle");
    if (h->committed) return fail(MGPU_E_STATE, "already committed");
    Dev &d = h->d;
    for (int a = 0; a < kNumArrays; ++a)
        if (kArrays[a].role != RO_OUT && kArrays[a].role != RO_OPT && !h->bound[a])
            return fail(MGPU_E_ARG, std::string("array not bound: ") + kArrays[a].name);
#define MGPU_CHKI(n, v) if (d.n == MGPU_REQUIRED_INT) return fail(MGPU_E_ARG, "integer not set: " #n);
    MGPU_INT_SCALARS(MGPU_CHKI)
#define MGPU_CHKR(n, v) if (d.n == MGPU_REQUIRED_REAL) return fail(MGPU_E_ARG, "real not set: " #n);
    MGPU_REAL_SCALARS(MGPU_CHKR)
    if (d.ITIMST != 3) return fail(MGPU_E_UNSUPPORTED, "ITIMST other than 3 (incompressible 5/6) not covered");
    // new_loss: NEW_LOSS (ILOS 100-199) or SPAL_LOSS (200-299), which share
    // the per-cell strain-rate work, the mixing lengths and the wall terms
    const bool new_loss = d.ILOS >= 100 && d.ILOS < 300;
    const bool sa = d.ILOS >= 200 && d.ILOS < 300;
    if (d.ILOS != 0 && d.ILOS != 10 && !new_loss)
        return fail(MGPU_E_UNSUPPORTED, "only ILOS=0 (inviscid), 10 (LOSS), 100-199 (NEW_LOSS) and 200-299 "
                                        "(Spalart-Allmaras, SPAL_LOSS) are covered");
    if (new_loss) {
        for (const char *n : {"XLENGTH", "FST_RAT", "ROAVG_CELL"})
            if (!h->bound[find_array(n)]) return fail(MGPU_E_ARG, std::string("ILOS >= 100 needs ") + n);
        if (!(d.VORT_MAX > 0.0f)) return fail(MGPU_E_ARG, "ILOS >= 100 needs VORT_MAX > 0 (SETUP 7322-7328)");
    }
    if (d.IFGAS != 0) return fail(MGPU_E_UNSUPPORTED, "real-gas IFGAS=1 not covered");
    if (d.IFCOOL || d.IFBLEED || d.IFSHROUD) return fail(MGPU_E_UNSUPPORTED, "cooling/bleed/shroud not covered");
    if (d.IF_REPEAT != 0) return fail(MGPU_E_UNSUPPORTED, "IF_REPEAT not covered");
    if (d.THROTTLE_EXIT > 0.001f && d.THROTTLE_MAS == 0.0f) return fail(MGPU_E_ARG, "THROTTLE_MAS must be set with THROTTLE_EXIT");
    if (d.YPLUSWALL < -10.0f && d.JM > 1700)
        return fail(MGPU_E_UNSUPPORTED, "YPLUSWALL<-10 with JM > 1700 is not covered (SET_PWALLGRAD column buffer)");
    if (d.IPOUT == 3 || d.IPOUT < -1) return fail(MGPU_E_UNSUPPORTED, "IPOUT not covered");
    if (d.NCHANGE <= 0 || d.NMIXUP <= 0 || d.NLOS <= 0) return fail(MGPU_E_ARG, "NCHANGE, NMIXUP, NLOS must be positive");
    if (d.KM > 512) return fail(MGPU_E_UNSUPPORTED, "KM above 512");
    size_t smem = (size_t)2 * d.IM * d.KM * sizeof(float);
    if (smem > 200 * 1024) return fail(MGPU_E_UNSUPPORTED, "J-plane does not fit shared memory");

    // host copies of the inputs the derived tables need
    int rc = 0;
    auto geti = [&](const char *n, std::vector<int> &v) -> int {
        int a = find_array(n);
        return download(h, v, (const int *)h->dptr[a], shape_count(h, kArrays[a].shape));
    };
    auto getf = [&](const char *n, std::vector<float> &v) -> int {
        int a = find_array(n);
        return download(h, v, (const float *)h->dptr[a], shape_count(h, kArrays[a].shape));
    };
    std::vector<int> JLED, IF_CUSP, JB1, JB2, JSBLK, IB1, IB2, KB1, KB2, NBLADE, JLE, JTE, NROW, JSTART, JMIX, INDMIX;
    std::vector<float> FP, FR, X, R, PO1, TO1, P, RO, XL[6];
    if ((rc = geti("JLED", JLED)) || (rc = geti("IF_CUSP", IF_CUSP)) || (rc = geti("JB1", JB1)) || (rc = geti("JB2", JB2)) ||
        (rc = geti("JSBLK", JSBLK)) || (rc = geti("IB1", IB1)) || (rc = geti("IB2", IB2)) || (rc = geti("KB1", KB1)) ||
        (rc = geti("KB2", KB2)) || (rc = geti("NBLADE", NBLADE)) || (rc = geti("JLE", JLE)) || (rc = geti("JTE", JTE)) ||
        (rc = geti("NROW", NROW)) || (rc = geti("JSTART", JSTART)) || (rc = geti("JMIX", JMIX)) ||
        (rc = geti("INDMIX", INDMIX)))
        return rc;
    if ((rc = getf("FP", FP)) || (rc = getf("FR", FR)) || (rc = getf("X", X)) || (rc = getf("R", R)) ||
        (rc = getf("PO1", PO1)) || (rc = getf("TO1", TO1)) || (rc = getf("P", P)) || (rc = getf("RO", RO)) ||
        (rc = getf("XLLIM_I1", XL[0])) || (rc = getf("XLLIM_IM", XL[1])) || (rc = getf("XLLIM_K1", XL[2])) ||
        (rc = getf("XLLIM_KM", XL[3])) || (rc = getf("XLLIM_DWN", XL[4])) || (rc = getf("XLLIM_UP", XL[5])))
        return rc;
    if (new_loss && !d.NLS && (rc = dalloc(h, &d.NLS, new_loss_work_floats(d)))) return rc;
    if (sa) {
        // the reader's defaults FSTURB = 1, TURBVIS_DAMP = 0.5 (2052-2053)
        if (!h->bound[find_array("FSTURB")] && (rc = upload(h, d.FSTURB, std::vector<float>(d.NROWS, 1.0f))))
            return rc;
        if (!h->bound[find_array("TURBVIS_DAMP")] &&
            (rc = upload(h, d.TURBVIS_DAMP, std::vector<float>(d.NROWS, 0.5f))))
            return rc;
        if (!d.SAW && (rc = dalloc(h, &d.SAW, sa_work_floats(d)))) return rc;
        // the sixth TSTEP variable: TRANS_DYN_VIS with its history DEL_DYNVIS
        VarSet &V = d.var[V_SA];
        const size_t N = (size_t)d.IM * d.JM * d.KM;
        V.D = d.TRANS_DYN_VIS;
        V.DIFF = d.DEL_DYNVIS;
        if (!V.XF) {
            float **fl[] = {&V.XF, &V.TF, &V.RF, &V.SR, &V.ST, &V.TM};
            for (float **w : fl)
                if ((rc = dalloc(h, w, N))) return rc;
            if ((rc = dalloc(h, &V.psum, d.JM)) || (rc = dalloc(h, &V.pabs, d.JM)) ||
                (rc = dalloc(h, &V.AVG_BLK, d.NROWS)))
                return rc;
        }
    }
    d.any_cusp2 = 0;
    for (int nr = 0; nr < d.NROWS; ++nr) {
        if (IF_CUSP[nr] > 2) return fail(MGPU_E_UNSUPPORTED, "IF_CUSP above 2 not covered");
        if (IF_CUSP[nr] == 2) d.any_cusp2 = 1;
    }
    if (d.any_cusp2) {
        for (const char *n : {"NUP_I1", "NUP_IM", "N_WAKE", "SEP_THIK", "SEP_DRAG", "RT_THICK", "RTHETA"})
            if (!h->bound[find_array(n)]) return fail(MGPU_E_ARG, std::string("IF_CUSP=2 needs ") + n);
        if (d.IM < 7) return fail(MGPU_E_ARG, "IF_CUSP=2 needs IM >= 7");
        std::vector<int> NUP1, NUPM, NW;
        if ((rc = geti("NUP_I1", NUP1)) || (rc = geti("NUP_IM", NUPM)) || (rc = geti("N_WAKE", NW))) return rc;
        for (int nr = 0; nr < d.NROWS; ++nr) {
            if (IF_CUSP[nr] != 2) continue;
            // every forced point stays inside the row, so the rows are independent
            int js1 = JTE[nr] - NUP1[nr], jsm = JTE[nr] - NUPM[nr];
            if (js1 < JSTART[nr] + 1 || jsm < JSTART[nr] + 1 || JTE[nr] + NW[nr] > JMIX[nr] || NW[nr] < 0)
                return fail(MGPU_E_ARG, "IF_CUSP=2: NUP_I1, NUP_IM, N_WAKE reach outside the row");
        }
    }
    for (int nr = 0; nr < d.NROWS; ++nr) {
        if (JSTART[nr] < 1 || JMIX[nr] > d.JM || JMIX[nr] - JSTART[nr] < 8)
            return fail(MGPU_E_ARG, "row J ranges (JSTART/JMIX) out of range");
        if (nr < d.NROWS - 1 && JMIX[nr] + 4 > d.JM) return fail(MGPU_E_ARG, "mixing plane too close to the exit");
    }
    for (int j = 1; j <= d.JM; ++j)
        if (NROW[j - 1] < 1 || NROW[j - 1] > d.NROWS) return fail(MGPU_E_ARG, "NROW out of range");
    for (int nr = 0; nr < d.NROWS; ++nr)
        if (JLED[nr] < 3 || JLED[nr] >= JMIX[nr] || JLE[nr] < 1 || JTE[nr] > d.JM || JTE[nr] <= JLE[nr])
            return fail(MGPU_E_ARG, "leading/trailing edge indices out of range");
    if (INDMIX[d.JM - 1] != 0) return fail(MGPU_E_ARG, "INDMIX(JM) must be 0");

    d.RFTHROTL1 = 1.0f - d.RFTHROTL;
    // gas constants, SETUP 6459-6468
    d.GA1 = d.GA - 1.0f;
    d.FGA = d.GA1 / d.GA;
    d.RFGA = 1.0f / d.FGA;
    d.RCP = 1.0f / d.CP;
    d.CV = d.CP / d.GA;
    d.RCV = 1.0f / d.CV;
    d.RGAS = d.CP - d.CV;
    // LOOP prologue, 3677-3709
    auto P3 = [&](const std::vector<float> &v, int i, int j, int k) {
        return v[(size_t)(i - 1) + (size_t)d.IM * ((size_t)(j - 1) + (size_t)d.JM * (k - 1))];
    };
    d.RO_REF = PO1[d.KMID - 1] / (d.RGAS * TO1[d.KMID - 1]);
    float ROMIN = fminf(P3(RO, d.IMID, 1, d.KMID), P3(RO, d.IMID, d.JM, d.KMID));
    d.ROLIM = 0.25f * ROMIN;
    d.RIJKM = 2.0f / (float)(d.IM * d.JM * d.KM);
    std::vector<float> PLIM(d.KM);
    for (int k = 1; k <= d.KM; ++k) PLIM[k - 1] = 0.9f * PO1[k - 1] + 0.1f * P3(P, 1, 1, k);
    if ((rc = upload(h, d.PLIM, PLIM))) return rc;
    d.PREFF = 0.5f * (P3(P, d.IMID, 1, d.KMID) + P3(P, d.IMID, d.JM, d.KMID));
    d.SFXIN = d.SFXIN * d.CFL / 0.5f;
    d.SFTIN = d.SFTIN * d.CFL / 0.5f;
    d.RFIN1 = 1.0f - d.RFIN;
    d.RFIN2 = 2.0f * d.RFIN;
    d.TCOOL_MIN = 1.0E6f;
    // the LOSS tables
    std::vector<float> FILAM, FITURB, FIWAKE, FIUP, FKLAM, FKTURB;
    loss_tables(d, FP, FR, X, R, NBLADE, JLE, JTE, XL, FILAM, FITURB, FIWAKE, FIUP, FKLAM, FKTURB);
    if ((rc = upload(h, d.FILAM, FILAM)) || (rc = upload(h, d.FITURB, FITURB)) || (rc = upload(h, d.FIWAKE, FIWAKE)) ||
        (rc = upload(h, d.FIUP, FIUP)) || (rc = upload(h, d.FKLAM, FKLAM)) || (rc = upload(h, d.FKTURB, FKTURB)))
        return rc;
    // multigrid block extents
    std::vector<int> s, e;
    struct Ext {
        const std::vector<int> *map;
        int lo, hi, n;
        int **ds, **de;
        const char *what;
    } ext[] = {
        {&JB1, 2, d.JM, d.NJB1, &d.JB1_START, &d.JB1_END, "JB1"},
        {&JB2, 2, d.JM, d.NJB2, &d.JB2_START, &d.JB2_END, "JB2"},
        {&IB1, 1, d.IMM1, d.NIB1, &d.IB1_S, &d.IB1_E, "IB1"},
        {&IB2, 1, d.IMM1, d.NIB2, &d.IB2_S, &d.IB2_E, "IB2"},
        {&KB1, 1, d.KMM1, d.NKB1, &d.KB1_S, &d.KB1_E, "KB1"},
        {&KB2, 1, d.KMM1, d.NKB2, &d.KB2_S, &d.KB2_E, "KB2"},
        {&JSBLK, 2, d.JM, d.NSBLK, &d.SB_START, &d.SB_END, "JSBLK"},
    };
    for (auto &x : ext) {
        if ((rc = extents(*x.map, x.lo, x.hi, x.n, s, e, x.what))) return rc;
        if ((rc = dalloc(h, x.ds, x.n)) || (rc = dalloc(h, x.de, x.n))) return rc;
        if ((rc = upload(h, *x.ds, s)) || (rc = upload(h, *x.de, e))) return rc;
    }
    // level-2 blocks nested in level-1 blocks (IRBB, KRBB multiples of IR,
    // KR): the cells kernel then forms the level-2 partials from the level-1 ones
    {
        auto nested = [&](const std::vector<int> &m1, const std::vector<int> &m2, int n) {
            for (int x = 1; x <= n; ++x) {
                const bool start2 = x == 1 || m2[x - 1] != m2[x - 2], end2 = x == n || m2[x - 1] != m2[x];
                const bool start1 = x == 1 || m1[x - 1] != m1[x - 2], end1 = x == n || m1[x - 1] != m1[x];
                if ((start2 && !start1) || (end2 && !end1)) return false;
            }
            return true;
        };
        d.mg_nested = nested(IB1, IB2, d.IMM1) && nested(KB1, KB2, d.KMM1) ? 1 : 0;
    }
    for (int j = 2; j <= d.JM; ++j) {
        if (JB1[j - 1] < 1 || JB1[j - 1] > d.NJB1 + 1 || JB2[j - 1] < 1 || JB2[j - 1] > d.NJB2 + 1 ||
            JSBLK[j - 1] < 1 || JSBLK[j - 1] > d.NSBLK)
            return fail(MGPU_E_ARG, "multigrid J map out of range");
    }
    for (int v = 0; v < (sa ? NVAR + 1 : NVAR); ++v) {
        VarSet &V = d.var[v];
        if ((rc = dalloc(h, &V.B1CHG, shape_count(h, SH_MG1))) || (rc = dalloc(h, &V.B2CHG, shape_count(h, SH_MG2))) ||
            (rc = dalloc(h, &V.SBSUM, d.NSBLK)) || (rc = dalloc(h, &V.P1, (size_t)d.JM * d.NIB1 * d.NKB1)) ||
            (rc = dalloc(h, &V.P2, (size_t)d.JM * d.NIB2 * d.NKB2)))
            return rc;
    }
    if (d.REDUCE_ORDER < 0 || d.REDUCE_ORDER > 2) return fail(MGPU_E_ARG, "REDUCE_ORDER must be 0, 1 or 2");
    if (d.TS_THREADS != 0 && d.TS_THREADS != 128 && d.TS_THREADS != 192 && d.TS_THREADS != 256 &&
        d.TS_THREADS != 512)
        return fail(MGPU_E_ARG, "TS_THREADS must be 0, 128, 192, 256 or 512");
    if (d.TS_PAIR != 0 && d.TS_PAIR != 1) return fail(MGPU_E_ARG, "TS_PAIR must be 0 or 1");
    d.ts_bs[0] = d.ts_bs[1] = d.TS_THREADS ? d.TS_THREADS : 256;
    // the control block
    DevCtl c;
    memset(&c, 0, sizeof(c));
    c.EAVG = 1.0E06f;
    c.ECONT = 1.0f;
    c.EMAX = 1.0E06f;
    c.FMIXUP = 1.0f;
    c.VISLAM = d.VISLAM;
    c.FTCOND = d.FTCOND;
    c.PDOWN_HUB = d.PDOWN_HUB;
    c.PDOWN_TIP = d.PDOWN_TIP;
    c.THROTTLE_PRES = d.THROTTLE_PRES;
    c.CHECK_FLOW_JM = 0.0f;
    c.nstep = d.NSTEP;
    CK(cudaMemcpy(d.ctl, &c, sizeof(c), cudaMemcpyHostToDevice));
    CK(configure_kernels(d));
    CK(cudaDeviceSynchronize());
    h->committed = true;
    return 0;
}

int32_t mgpu_stepup(mgpu_handle *h, float relax) {
    if (!h || !h->committed) return fail(MGPU_E_STATE, "stepup before commit");
    Launch L{h->stream, h->sm_count};
    launch_stepup(h->d, L, relax, false);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int32_t mgpu_loss_init(mgpu_handle *h) {
    if (!h || !h->committed) return fail(MGPU_E_STATE, "loss_init before commit");
    Launch L{h->stream, h->sm_count};
    launch_loss(h->d, L, true);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int32_t mgpu_step(mgpu_handle *h, int32_t force_end, mgpu_monitors *mon) {
    if (!h || !h->committed) return fail(MGPU_E_STATE, "step before commit");
    int rc = build_graph(h);
    if (rc) return rc;
    int fe = force_end ? 1 : 0;
    CK(cudaMemcpyAsync(&h->d.ctl->force_end, &fe, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    CK(cudaGraphLaunch(h->gexec, h->stream));
    if ((rc = read_ctl(h))) return rc;
    const DevCtl &c = *h->h_ctl;
    if (mon) fill_monitors(c, mon);
    if (c.do_tail && c.health) return fail(MGPU_E_NONFINITE, "non-finite or non-positive density in the flow field");
    return 0;
}

int32_t mgpu_run(mgpu_handle *h, int32_t nsteps, mgpu_monitors *mon) {
    if (!h || !h->committed) return fail(MGPU_E_STATE, "run before commit");
    if (nsteps < 0) return fail(MGPU_E_ARG, "negative step count");
    int rc = build_graph(h);
    if (rc) return rc;
    // The end test at the top of step n (3762-3764) reads NSTEP and the
    // monitors EMAX, EAVG and ECONT, which only a tail (every fifth step, or
    // the final one) rewrites.  So no step after a tail up to and including
    // the next tail can be the final one unless that tail met the test or
    // NSTEPS_MAX falls among them: such a run of steps is launched back to
    // back, then the control block is read, and the run stops right after
    // the final step, where LOOP stops (5444-5451).
    if ((rc = read_ctl(h))) return rc;
    int done = 0;
    for (;;) {
        const DevCtl &c = *h->h_ctl;
        if (mon) fill_monitors(c, mon);
        // a field already flagged by the last tail (of this call, or of an
        // earlier mgpu_step / mgpu_run) is not marched further
        if ((done > 0 || c.nstep > 0) && c.health)
            return fail(MGPU_E_NONFINITE, "non-finite or non-positive density in the flow field");
        if (c.ifend) return 1;
        if (done >= nsteps) return 0;
        const int n0 = c.nstep;
        int n = 1;                              // a met test makes the next step the final one
        if (!c.converged) {
            n = (n0 / 5 + 1) * 5 - n0;          // up to the next tail
            if (h->d.NSTEPS_MAX > n0 && h->d.NSTEPS_MAX - n0 < n) n = h->d.NSTEPS_MAX - n0;
        }
        if (n > nsteps - done) n = nsteps - done;
        for (int s = 0; s < n; ++s) CK(cudaGraphLaunch(h->gexec, h->stream));
        done += n;
        if ((rc = read_ctl(h))) return rc;
    }
}

int32_t mgpu_step_io_bytes(int32_t *h2d, int32_t *d2h) {
    if (!h2d || !d2h) return fail(MGPU_E_ARG, "null argument");
    *h2d = (int32_t)sizeof(int);
    *d2h = (int32_t)sizeof(DevCtl);
    return 0;
}

int32_t mgpu_sync(mgpu_handle *h) {
    if (!h) return fail(MGPU_E_ARG, "null handle");
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int32_t mgpu_integrals_compute(mgpu_handle *h, mgpu_integrals *out) {
    if (!h || !h->committed || !out) return fail(MGPU_E_STATE, "integrals before commit");
    const Dev &d = h->d;
    Launch L{h->stream, h->sm_count};
    launch_integrals(d, L, h->d_int);
    CK(cudaGetLastError());
    std::vector<double> v((size_t)4 * d.JM);
    CK(cudaMemcpyAsync(v.data(), h->d_int, v.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    // whole-machine efficiency (11269-11394): for one stage the inlet
    // station is J=1, otherwise J=2; the exit station is JM-1
    int J1 = d.NSTAGES == 1 ? 1 : 2, J2M1 = d.JM - 1;
    auto bf = [&](int j) { return v[(size_t)(j - 1)]; };
    auto spo = [&](int j) { return v[(size_t)d.JM + j - 1] / bf(j); };
    auto sto = [&](int j) { return v[(size_t)2 * d.JM + j - 1] / bf(j); };
    auto sps = [&](int j) { return v[(size_t)3 * d.JM + j - 1] / bf(j); };
    double PO1M = 0.0;
    {
        std::vector<float> po1;
        int a = find_array("PO1");
        int rc = download(h, po1, (const float *)h->dptr[a], d.KM);
        if (rc) return rc;
        PO1M = po1[d.KMID - 1];
    }
    double FGA = (double)d.FGA;
    double POIN = spo(J1) * PO1M, PO2 = spo(J2M1) * PO1M, PSOUT = sps(J2M1);
    double TO_IN = sto(J1), TO_OUT = sto(J2M1);
    double TORAT = TO_OUT / TO_IN, DELTO = TO_OUT - TO_IN, PORAT = PO2 / POIN, PSRAT = PSOUT / POIN;
    if (PORAT < 0.01) PORAT = 0.01;
    double TO2IS = pow(PORAT, FGA) * TO_IN, TSTAT2_IS = pow(PSRAT, FGA) * TO_IN;
    double DELTOIS = TO2IS - TO_IN, DELT_TOT_STAT = TSTAT2_IS - TO_IN;
    double ETAIS = 1.0, ETATS = 1.0;
    if (DELTO > 0.0) { ETAIS = DELTOIS / DELTO; ETATS = DELT_TOT_STAT / DELTO; }
    if (DELTO < 0.0) { ETAIS = DELTO / DELTOIS; ETATS = DELTO / DELT_TOT_STAT; }
    out->mass_flow_in = bf(J1);
    out->mass_flow_out = bf(J2M1);
    out->eta_tt = ETAIS;
    out->eta_ts = ETATS;
    out->po_ratio = PORAT;
    out->to_ratio = TORAT;
    out->j1 = J1;
    out->j2m1 = J2M1;
    return 0;
}

int32_t mgpu_stage_performance(mgpu_handle *h, int32_t nstg, mgpu_stage *out) {
    if (!h || !h->committed || !out) return fail(MGPU_E_STATE, "stage performance before commit");
    const Dev &d = h->d;
    const int NSTAGES = d.NSTAGES, NROWS = d.NROWS;
    const int NSTGP1 = NSTAGES == 1 ? 1 : NSTAGES + 1;
    if (nstg < 1 || nstg > NSTGP1) return fail(MGPU_E_ARG, "stage number out of range");
    const int an = find_array("NSTAGE");
    if (!h->bound[an]) return fail(MGPU_E_STATE, "bind the row array NSTAGE for the stage table");
    std::vector<int> NSTAGE, JSTART, JMIX, NROW;
    std::vector<float> P, FP, PO1;
    auto geti = [&](const char *n, std::vector<int> &v) {
        int a = find_array(n);
        return download(h, v, (const int *)h->dptr[a], shape_count(h, kArrays[a].shape));
    };
    auto getf = [&](const char *n, std::vector<float> &v) {
        int a = find_array(n);
        return download(h, v, (const float *)h->dptr[a], shape_count(h, kArrays[a].shape));
    };
    int rc = 0;
    if ((rc = geti("NSTAGE", NSTAGE)) || (rc = geti("JSTART", JSTART)) || (rc = geti("JMIX", JMIX)) ||
        (rc = geti("NROW", NROW)) || (rc = getf("P", P)) || (rc = getf("FP", FP)) || (rc = getf("PO1", PO1)))
        return rc;
    // the stages' stations, as the reader sets them (1522-1536)
    std::vector<int> JSTG_START(NSTAGES + 2, 0), JSTG_END(NSTAGES + 2, 0);
    JSTG_START[1] = 1;
    for (int n = 1; n <= NROWS; ++n) {
        const int s0 = NSTAGE[n - 1], s1 = n < NROWS ? NSTAGE[n] : NSTAGES + 1;
        if (s0 < 1 || s0 > NSTAGES) return fail(MGPU_E_ARG, "NSTAGE out of 1..NSTAGES");
        if (s0 != s1) {
            JSTG_END[s0] = JMIX[n - 1];
            if (s1 <= NSTAGES) JSTG_START[s1] = JSTART[n];
        }
    }
    // 11269-11293
    int J1, J2, J2M1, JMS;
    const bool whole = NSTGP1 > 1 && nstg == NSTGP1;
    if (!whole) {
        J1 = JSTG_START[nstg];
        J2 = JSTG_END[nstg] + 1;
        J2M1 = nstg == NSTAGES ? d.JM - 1 : J2;
        JMS = JMIX[NROW[J1] - 1];          // NROW(J1+1)
    } else {
        J1 = 2;
        J2 = d.JM;
        J2M1 = d.JM - 1;
        JMS = (J1 + J2) / 2;
    }
    if (J1 < 1 || J2M1 > d.JM || J1 >= J2M1) return fail(MGPU_E_ARG, "stage stations out of range");
    Launch L{h->stream, h->sm_count};
    launch_integrals(d, L, h->d_int);
    CK(cudaGetLastError());
    std::vector<double> v((size_t)4 * d.JM);
    CK(cudaMemcpyAsync(v.data(), h->d_int, v.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    auto bf = [&](int j) { return v[(size_t)(j - 1)]; };
    auto spo = [&](int j) { return v[(size_t)d.JM + j - 1] / bf(j); };
    auto sto = [&](int j) { return v[(size_t)2 * d.JM + j - 1] / bf(j); };
    auto sps = [&](int j) { return v[(size_t)3 * d.JM + j - 1] / bf(j); };
    const double PO1M = PO1[d.KMID - 1], FGA = (double)d.FGA;
    out->j1 = J1;
    out->j2m1 = J2M1;
    out->jmix = JMS;
    out->has_reaction = !whole;
    out->reac_hub = out->reac_mid = out->reac_tip = 0.0;
    if (!whole) {
        // pitchwise static pressures, REAL*4 in I order (11300-11349)
        const int KMID2 = d.KM / 2;
        auto pline = [&](int j, int k) {
            float s = 0.0f;
            for (int i = 1; i <= d.IMM1; ++i) {
                const size_t a = (size_t)(i - 1) + (size_t)d.IM * ((size_t)(j - 1) + (size_t)d.JM * (size_t)(k - 1));
                s = s + 0.5f * (P[a] + P[a + 1]) * FP[i - 1];
            }
            return s;
        };
        const int ks[3] = {1, KMID2, d.KM};
        float rr[3];
        const float pmid_in = pline(J1, KMID2), pmid_out = pline(J2M1, KMID2);
        for (int q = 0; q < 3; ++q) {
            const float pin = pline(J1, ks[q]), pm = pline(JMS, ks[q]), po = pline(J2M1, ks[q]);
            rr[q] = (pm - po) / (pin - po);
            if (pmid_out > pmid_in) rr[q] = 1.0f - rr[q];    // a compressor
        }
        out->reac_hub = rr[0];
        out->reac_mid = rr[1];
        out->reac_tip = rr[2];
    }
    // 11366-11394
    const double POIN = spo(J1) * PO1M, PO2 = spo(J2M1) * PO1M, PSOUT = sps(J2M1);
    const double TO_IN = sto(J1), TO_OUT = sto(J2M1);
    const double TORAT = TO_OUT / TO_IN, DELTO = TO_OUT - TO_IN, PSRAT = PSOUT / POIN;
    double PORAT = PO2 / POIN;
    if (PORAT < 0.01) PORAT = 0.01;
    const double TO2IS = pow(PORAT, FGA) * TO_IN, TSTAT2_IS = pow(PSRAT, FGA) * TO_IN;
    const double DELTOIS = TO2IS - TO_IN, DELT_TOT_STAT = TSTAT2_IS - TO_IN;
    double ETAIS = 1.0, ETATS = 1.0;
    if (DELTO > 0.0) { ETAIS = DELTOIS / DELTO; ETATS = DELT_TOT_STAT / DELTO; }
    if (DELTO < 0.0) { ETAIS = DELTO / DELTOIS; ETATS = DELTO / DELT_TOT_STAT; }
    double EPOLY = log(TORAT) / log(PORAT) / FGA;
    if (TORAT > 1.0) EPOLY = 1.0 / EPOLY;
    out->mass_flow_in = bf(J1);
    out->mass_flow_out = bf(J2M1);
    out->po_ratio = PORAT;
    out->to_ratio = TORAT;
    out->delta_to = DELTO;
    out->eta_tt = ETAIS;
    out->eta_ts = ETATS;
    out->eta_poly = EPOLY;
    return 0;
}

int32_t mgpu_autotune(mgpu_handle *h, int32_t *chosen, double *ms) {
    if (!h || !h->committed) return fail(MGPU_E_STATE, "autotune before commit");
    Dev &d = h->d;
    const size_t N = (size_t)d.IM * d.JM * d.KM, fb = N * sizeof(float);
    // the candidates run TSTEP on the handle's arrays; the variables and their
    // histories are put back after each
    float *save = nullptr;
    CK(cudaMallocAsync((void **)&save, 2 * NVAR * fb, h->stream));
    for (int v = 0; v < NVAR; ++v) {
        CK(cudaMemcpyAsync(save + (size_t)(2 * v) * N, d.var[v].D, fb, cudaMemcpyDeviceToDevice, h->stream));
        CK(cudaMemcpyAsync(save + (size_t)(2 * v + 1) * N, d.var[v].DIFF, fb, cudaMemcpyDeviceToDevice, h->stream));
    }
    constexpr int NC = 4;
    const int cand[NC] = {128, 192, 256, 512};
    // each timed pass starts from a cold L2, as it does inside a step (the
    // passes run back to back would find their arrays in L2)
    if (!h->flush_buf) {
        int l2 = 0;
        CK(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, h->device));
        h->flush_bytes = (size_t)(l2 > 0 ? l2 : 128 << 20) * 2;
        CK(cudaMalloc(&h->flush_buf, h->flush_bytes));
    }
    double t[2][NC] = {};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int best[2] = {2, 2};
    // each pass on its own: the pass of RO and ROE (2 x (JM-1) CTAs) and the
    // pass of the momenta (3 x (JM-1)) fill the SMs differently
    for (int p = 0; p < 2; ++p) {
        const int v0 = p ? V_ROVX : V_RO, nv = p ? 3 : 2;
        for (int c = 0; c < NC; ++c) {
            Dev dt = d;
            dt.ts_bs[p] = cand[c];
            dt.use_cond = 0;
            Launch L{h->stream, h->sm_count};
            for (int r = 0; r < 2; ++r) launch_tstep(dt, L, v0, nv);
            const int reps = 10;
            double sum = 0.0;
            for (int r = 0; r < reps; ++r) {
                CK(cudaMemsetAsync(h->flush_buf, r & 0xff, h->flush_bytes, h->stream));
                CK(cudaEventRecord(e0, h->stream));
                launch_tstep(dt, L, v0, nv);
                CK(cudaEventRecord(e1, h->stream));
                CK(cudaGetLastError());
                CK(cudaEventSynchronize(e1));
                float f = 0.0f;
                CK(cudaEventElapsedTime(&f, e0, e1));
                sum += (double)f;
            }
            t[p][c] = sum / reps;
            for (int v = v0; v < v0 + nv; ++v) {
                CK(cudaMemcpyAsync(d.var[v].D, save + (size_t)(2 * v) * N, fb, cudaMemcpyDeviceToDevice, h->stream));
                CK(cudaMemcpyAsync(d.var[v].DIFF, save + (size_t)(2 * v + 1) * N, fb, cudaMemcpyDeviceToDevice,
                                   h->stream));
            }
        }
        // the fastest candidate, once all are timed
        for (int c = 0; c < NC; ++c)
            if (t[p][c] < t[p][best[p]]) best[p] = c;
    }
    CK(cudaFreeAsync(save, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (d.ts_bs[0] != cand[best[0]] || d.ts_bs[1] != cand[best[1]]) {
        d.ts_bs[0] = cand[best[0]];
        d.ts_bs[1] = cand[best[1]];
        if (h->gexec) {
            cudaGraphExecDestroy(h->gexec);
            h->gexec = nullptr;
        }
        if (h->graph) {
            cudaGraphDestroy(h->graph);
            h->graph = nullptr;
        }
    }
    if (chosen) {
        chosen[0] = cand[best[0]];
        chosen[1] = cand[best[1]];
    }
    if (ms)
        for (int p = 0; p < 2; ++p)
            for (int c = 0; c < NC; ++c) ms[p * NC + c] = t[p][c];
    return 0;
}

int32_t mgpu_bench_steps(mgpu_handle *h, int32_t nsteps, int32_t flush_l2, double *total_ms) {
    if (!h || !h->committed || !total_ms || nsteps < 0) return fail(MGPU_E_ARG, "bad arguments to mgpu_bench_steps");
    int rc = build_graph(h);
    if (rc) return rc;
    if (flush_l2 && !h->flush_buf) {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, h->device);
        h->flush_bytes = (size_t)(l2 > 0 ? l2 : 128 << 20) * 2;
        CK(cudaMalloc(&h->flush_buf, h->flush_bytes));
    }
    std::vector<cudaEvent_t> ev((size_t)2 * nsteps);
    for (auto &e : ev) CK(cudaEventCreate(&e));
    for (int s = 0; s < nsteps; ++s) {
        if (flush_l2) CK(cudaMemsetAsync(h->flush_buf, s & 0xff, h->flush_bytes, h->stream));
        CK(cudaEventRecord(ev[2 * s], h->stream));
        CK(cudaGraphLaunch(h->gexec, h->stream));
        CK(cudaEventRecord(ev[2 * s + 1], h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    double tot = 0.0;
    for (int s = 0; s < nsteps; ++s) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ev[2 * s], ev[2 * s + 1]));
        tot += ms;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    *total_ms = tot;
    if ((rc = read_ctl(h))) return rc;
    if (h->h_ctl->health) return fail(MGPU_E_NONFINITE, "non-finite or non-positive density in the flow field");
    return 0;
}

int32_t mgpu_profile_steps(mgpu_handle *h, int32_t nsteps, mgpu_kernel_time *out, int32_t max_entries,
                           int32_t *n_out) {
    if (!h || !h->committed || !out || !n_out || nsteps < 0) return fail(MGPU_E_ARG, "bad arguments to mgpu_profile_steps");
    std::map<std::string, std::pair<int, double>> acc;
    std::vector<std::string> order;
    for (int s = 0; s < nsteps; ++s) {
        Prof *p = new (std::nothrow) Prof();
        if (!p) return fail(MGPU_E_NOMEM, "host allocation");
        for (int e = 0; e < Prof::MAXEV; ++e) cudaEventCreate(&p->ev[e]);
        Launch L0{h->stream, h->sm_count, p};
        k_delay<<<1, 1, 0, h->stream>>>(40000000LL);   // ~20 ms at 2 GHz
        mark(L0, "start");
        int rc = enqueue_step(h, p);
        cudaError_t ce = cudaStreamSynchronize(h->stream);
        if (!rc && ce == cudaSuccess) {
            for (int e = 1; e < p->n; ++e) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, p->ev[e - 1], p->ev[e]);
                std::string nm = p->name[e];
                if (!acc.count(nm)) order.push_back(nm);
                acc[nm].first += 1;
                acc[nm].second += ms;
            }
        }
        for (int e = 0; e < Prof::MAXEV; ++e) cudaEventDestroy(p->ev[e]);
        delete p;
        if (rc) return rc;
        if (ce != cudaSuccess) return fail(MGPU_E_CUDA, cudaGetErrorString(ce));
    }
    int n = 0;
    for (const auto &nm : order) {
        if (n >= max_entries) break;
        snprintf(out[n].name, sizeof(out[n].name), "%s", nm.c_str());
        out[n].launches = acc[nm].first;
        out[n].total_ms = acc[nm].second;
        ++n;
    }
    *n_out = n;
    return 0;
}

void mgpu_batch_destroy(mgpu_batch *b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->flush_buf) cudaFree(b->flush_buf);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (cudaEvent_t e : b->joins)
        if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int32_t mgpu_batch_create(mgpu_handle *const *handles, int32_t n, mgpu_batch **out) {
    if (!handles || !out || n < 1) return fail(MGPU_E_ARG, "mgpu_batch_create: need n >= 1 handles and an out pointer");
    *out = nullptr;
    int cur = -1;
    CK(cudaGetDevice(&cur));
    for (int i = 0; i < n; ++i) {
        mgpu_handle *h = handles[i];
        if (!h || !h->committed) return fail(MGPU_E_STATE, "mgpu_batch_create: every handle must be committed");
        if (h->device != cur) return fail(MGPU_E_STATE, "mgpu_batch_create: every handle must live on the current device");
        for (int q = 0; q < i; ++q)
            if (handles[q] == h) return fail(MGPU_E_ARG, "mgpu_batch_create: a handle appears twice");
    }
    mgpu_batch *b = new (std::nothrow) mgpu_batch();
    if (!b) return fail(MGPU_E_NOMEM, "host allocation");
    b->hs.assign(handles, handles + n);
    b->device = cur;
    b->joins.assign((size_t)n, nullptr);
    auto bail = [&](int code) {
        mgpu_batch_destroy(b);
        return code;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    for (int i = 0; i < n && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&b->joins[i], cudaEventDisableTiming);
    if (e != cudaSuccess) return bail(fail(MGPU_E_CUDA, std::string("mgpu_batch_create: ") + cudaGetErrorString(e)));
    e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return bail(fail(MGPU_E_CUDA, std::string("batch capture: ") + cudaGetErrorString(e)));
    int rc = 0;
    e = cudaEventRecord(b->fork, b->stream);
    for (int i = 0; i < n && !rc && e == cudaSuccess; ++i) {
        mgpu_handle *h = b->hs[i];
        e = cudaStreamWaitEvent(h->stream, b->fork, 0);
        if (e != cudaSuccess) break;
        rc = capture_step(h);
        if (rc) break;
        e = cudaEventRecord(b->joins[i], h->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->joins[i], 0);
    }
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (rc || e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (rc) return bail(rc);
        return bail(fail(MGPU_E_CUDA, std::string("batch capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2)));
    }
    b->graph = g;
    e = cudaGraphGetNodes(g, nullptr, &b->graph_nodes);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->gexec, g, 0);
    if (e != cudaSuccess) return bail(fail(MGPU_E_CUDA, std::string("batch graph: ") + cudaGetErrorString(e)));
    *out = b;
    return 0;
}

namespace {
// the control blocks of every instance, read back on the batch stream
int batch_read(mgpu_batch *b, mgpu_monitors *mons, int *ended) {
    for (mgpu_handle *h : b->hs)
        CK(cudaMemcpyAsync(h->h_ctl, h->d.ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    int nend = 0;
    for (size_t i = 0; i < b->hs.size(); ++i) {
        const DevCtl &c = *b->hs[i]->h_ctl;
        if (mons) fill_monitors(c, &mons[i]);
        if (c.health) {
            char msg[96];
            snprintf(msg, sizeof msg, "batch instance %zu: non-finite or non-positive density", i);
            return fail(MGPU_E_NONFINITE, msg);
        }
        if (c.converged || c.ifend) ++nend;
    }
    *ended = nend;
    return 0;
}
}  // namespace

int32_t mgpu_batch_run(mgpu_batch *b, int32_t nsteps, mgpu_monitors *mons) {
    if (!b || nsteps < 0) return fail(MGPU_E_ARG, "bad arguments to mgpu_batch_run");
    const int chunk = 50;
    int done = 0, ended = 0, rc = 0;
    while (done < nsteps) {
        int m = nsteps - done < chunk ? nsteps - done : chunk;
        for (int s = 0; s < m; ++s) CK(cudaGraphLaunch(b->gexec, b->stream));
        done += m;
        if ((rc = batch_read(b, mons, &ended))) return rc;
    }
    if (nsteps == 0 && (rc = batch_read(b, mons, &ended))) return rc;
    return ended;
}

int32_t mgpu_batch_bench_steps(mgpu_batch *b, int32_t nsteps, int32_t flush_l2, double *total_ms) {
    if (!b || !total_ms || nsteps < 0) return fail(MGPU_E_ARG, "bad arguments to mgpu_batch_bench_steps");
    if (flush_l2 && !b->flush_buf) {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, b->device);
        b->flush_bytes = (size_t)(l2 > 0 ? l2 : 128 << 20) * 2;
        CK(cudaMalloc(&b->flush_buf, b->flush_bytes));
    }
    std::vector<cudaEvent_t> ev((size_t)2 * nsteps);
    for (auto &e : ev) CK(cudaEventCreate(&e));
    for (int s = 0; s < nsteps; ++s) {
        if (flush_l2) CK(cudaMemsetAsync(b->flush_buf, s & 0xff, b->flush_bytes, b->stream));
        CK(cudaEventRecord(ev[2 * s], b->stream));
        CK(cudaGraphLaunch(b->gexec, b->stream));
        CK(cudaEventRecord(ev[2 * s + 1], b->stream));
    }
    CK(cudaStreamSynchronize(b->stream));
    double tot = 0.0;
    for (int s = 0; s < nsteps; ++s) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ev[2 * s], ev[2 * s + 1]));
        tot += ms;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    *total_ms = tot;
    int ended = 0;
    return batch_read(b, nullptr, &ended);
}

int32_t mgpu_kernels_per_step(mgpu_handle *h, int32_t which) {
    if (!h || !h->committed) return fail(MGPU_E_STATE, "kernels_per_step before commit");
    if (which < 0 || which > 3) return fail(MGPU_E_ARG, "kernels_per_step: which must be 0..3");
    int rc = build_graph(h);
    if (rc) return rc;
    size_t n = h->graph_nodes - 2;   // every top-level node but the two conditionals is a kernel
    if (which & 1) n += h->loss_nodes;
    if (which & 2) n += h->tail_nodes;
    return (int32_t)n;
}

}  // extern "C"
