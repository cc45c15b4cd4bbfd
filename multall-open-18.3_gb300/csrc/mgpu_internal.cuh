// mgpu_internal.cuh -- device-side description of one Multall flow problem.
//
// Every COMMON array of the loop lives in HBM in the reference's packed
// Fortran order (I fastest, then J, then K), so one node (I,J,K) is
// element (I-1) + IM*((J-1) + JM*(K-1)) and a warp reads 32 consecutive
// pitchwise points.  Kernels take the whole description by value (`Dev`,
// ~2.3 KB of kernel parameters: pointers, dimensions and the constant
// REAL scalars); the values that change from step to step (smoothing ramp,
// NSTEP, the 5-step flags, the monitors) live in a small device struct
// `DevCtl` that the first kernel of each step updates, so a step is a fixed
// launch sequence that can be captured once in a CUDA graph.
//
// Indices in kernel code are the reference's 1-based ones.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/mgpu.h"
#include "../../include/mgpu_common_table.h"

namespace mgpu {

#define MGPU_T_INT32 int32_t
#define MGPU_T_FLOAT32 float

// Reduction slots written by the step and read back by the host.
struct DevMon {
    double vrms;            // sum of |W|^2 (VRMS)
    unsigned long long vmax_key;
    double eavg_sum;
    unsigned long long emax_key;
    int health;
    int pad;
};

// State that changes from step to step; one per problem, in device memory.
struct DevCtl {
    int nstep;        // NSTEP
    int ifend;        // IFEND after the convergence test of this step
    int force_end;    // host request: make this the final step
    int do_tail;      // every-5-step tail runs on this step
    int do_loss;      // LOSS runs on this step
    int damp_on;      // negative feedback active (2 <= DAMP <= 100)
    int converged;    // the reference's convergence test met at a tail
    int pad0;
    float SFT, SFX, DAMP, FMIXUP;
    float SFT1, SFTH, SFX1, SFXH, SFX14, SFXB, SFXB1, SFXBH, SFXHM1;
    float VISLAM, FTCOND;
    float EMAX, EAVG, ECONT, VMAX, VREF;
    int IMAXE, JMAXE, KMAXE, JCONT, IVMAX, JVMAX, KVMAX;
    int health;
    double flow_in, flow_out;
    DevMon mon;
    // exit pressures that the throttle condition moves from step to step
    // (4488-4505), and CHECK_FLOW(JM) of the last tail
    float PDOWN_HUB, PDOWN_TIP, THROTTLE_PRES, CHECK_FLOW_JM;
};

// A double-float value hi + lo (its arithmetic is below, beside racc).
struct df {
    float hi, lo;
};

// One conserved variable's TSTEP operands and work arrays.  The five
// variables (RO, ROE, ROVX, RORVT, ROVR) each have their own face fluxes and
// cell-change arrays, so the TSTEP kernels can update several variables in
// one launch (blockIdx.y selects the variable): RO and ROE together, then
// the three momenta after the inlet/exit conditions.
struct VarSet {
    float *D, *DIFF;             // the variable and its SCREE history (COMMON)
    float *XF, *TF, *RF, *SR;    // XFLUX, TFLUX, RFLUX, SOURCE of this variable
    float *ST;                   // STORE: cell changes
    float *TM;                   // TMP: node values before SMOOTH_VAR
    df *psum, *pabs;             // (JM) per-J-plane sums of STORE and |STORE| (double-float)
    float *P1, *P2;              // (JM, NIB1*NKB1) / (JM, NIB2*NKB2) per-plane block partials
    float *B1CHG, *B2CHG;        // MG1 / MG2 block sums, reference order
    float *SBSUM;                // (NSBLK) superblock sums, reference order
    float *AVG_BLK;              // (NROWS) row means of |STORE|, reference order
};
constexpr int NVAR = 5;
enum { V_RO = 0, V_ROE = 1, V_ROVX = 2, V_RORVT = 3, V_ROVR = 4 };
// the Spalart-Allmaras transported viscosity (ILOS >= 200): a sixth TSTEP
// variable, cell-centred, after the five conserved ones
constexpr int V_SA = 5;

struct Dev {
    // dimensions
    int IM, JM, KM, NROWS;
    int IMM1, JMM1, KMM1, IMM2, JMM2, KMM2, IMID, KMID, NRWSM1;
    // COMMON integer and real scalars (include/mgpu_common_table.h)
#define MGPU_DEV_I(n, d) int n;
    MGPU_INT_SCALARS(MGPU_DEV_I)
#define MGPU_DEV_R(n, d) float n;
    MGPU_REAL_SCALARS(MGPU_DEV_R)
    // gas constants and loop constants (SETUP 6459-6468, LOOP 3677-3709)
    float GA1, FGA, RFGA, RCP, CV, RCV, RGAS;
    float RO_REF, ROLIM, RIJKM, PREFF, RFIN1, RFIN2, TCOOL_MIN;
    float RFTHROTL1;                   // 1 - RFTHROTL (reader 559)
    int any_cusp2;                     // some row has IF_CUSP = 2
    // COMMON arrays on the device
#define MGPU_DEV_A(n, t, s, r) MGPU_T_##t *n;
    MGPU_ARRAYS(MGPU_DEV_A)
    // loop work arrays (COMMON scratch of the reference).  STORE and TMP
    // alias var[V_RO].ST / .TM (scratch of the tail, STEPUP and integrals);
    // RO's face fluxes are the mass fluxes FLOWX/FLOWT/FLOWR and its SOURCE
    // is the all-zero ZERO array.
    float *FLOWX, *FLOWT, *FLOWR, *ZERO;
    float *STORE, *TMP, *TEMP1;
    VarSet var[NVAR + 1];
    float *PLIM;                       // (KM)
    float *FILAM, *FITURB, *FIWAKE, *FIUP, *FKLAM, *FKTURB;   // (NROWS, IM|KM)
    float *VLIMIT, *ROLIMIT;           // (NROWS)
    int *DFLAG;                        // (IM*KM) density-limiter column flags
    float *BCBUF;                      // (4, KM) PAVG2, PAVG3, PAVGOUT, and the PD each K's exit update uses
    float *FLOWJ;                      // (JM) SETFLO's FLOW(J)
    float *NLS;                        // NEW_LOSS work: 9 strain-rate arrays, then the wall-face terms
    // Spalart-Allmaras work (ILOS >= 200): ABS_VORT, DYN_VIS_ML, GRAD_TVIS,
    // TVISGRADX/R/T (node arrays), then REYNOLDS(NROWS) and three scalars
    float *SAW;
    // recording hooks of the adjoint's linearisation step (null otherwise):
    // RO(I,1,K) as the inlet condition reads it, the mixing-plane inputs of
    // each (row interface, K), and bit flags for a limiter that changed a value
    float *ADJ_ROIN;
    float *ADJ_MIX;
    int *ADJ_FLAG;
    float *ADJ_RO_LIM;     // RO as the density limiter finds it
    float *ADJ_RO_MACH;    // RO as the Mach limiter finds it
    double *BLADE_FLOW;                // (JM)
    // per-block reduction partials of the 5-step tail
    double *part_sum;
    unsigned long long *part_key;
    int *part_cnt;
    int nparts;
    // multigrid block extents (host-derived from JB1/JB2)
    int *JB1_START, *JB1_END, *JB2_START, *JB2_END;    // (NJBn)
    int *IB1_S, *IB1_E, *IB2_S, *IB2_E;                 // (NIBn) I extent of each block
    int *KB1_S, *KB1_E, *KB2_S, *KB2_E;                 // (NKBn) K extent of each block
    int *SB_START, *SB_END;                             // (NSBLK)
    int mg_nested;                     // every level-2 block is a union of level-1 blocks (in I and in K)
    DevCtl *ctl;
    // graph conditionals selecting the LOSS and 5-step tail bodies (set by
    // the step-control kernel when the step runs from the CUDA graph)
    int use_cond;
    unsigned long long cond_loss, cond_tail;
    int ts_bs[2];                      // threads per J-plane CTA of TSTEP (128, 192, 256 or 512; mgpu_autotune)
                                       // for the pass of 2 variables (RO, ROE) and the pass of 3 (momenta)
};

// Element offsets in 32-bit int: mgpu_create keeps IM*JM*KM below 2^30,
// and signed arithmetic lets the compiler share one node's offset among its
// neighbours (i+1, j-1, k+1 ... differ by constants).
__host__ __device__ inline int ix3(const Dev &d, int i, int j, int k) {
    return (i - 1) + d.IM * ((j - 1) + d.JM * (k - 1));
}
__host__ __device__ inline int ix2(const Dev &d, int j, int k) { return (j - 1) + d.JM * (k - 1); }
__host__ __device__ inline int ixik(const Dev &d, int i, int k) { return (i - 1) + d.IM * (k - 1); }
__host__ __device__ inline int ixij(const Dev &d, int i, int j) { return (i - 1) + d.IM * (j - 1); }

// 1-based accessors used by the kernels, e.g. A3(d.RO, i, j, k)
#define A3(p, i, j, k) (p)[ix3(d, (i), (j), (k))]
#define A2(p, j, k) (p)[ix2(d, (j), (k))]
#define AIK(p, i, k) (p)[ixik(d, (i), (k))]
#define AIJ(p, i, j) (p)[ixij(d, (i), (j))]
#define A1(p, x) (p)[(x) - 1]

// Decomposes a linear node index n (I fastest) into 1-based (i, j, k).
// mgpu_create keeps IM*JM*KM below 2^31, so 32-bit division suffices.
__device__ inline void node_ijk(const Dev &d, size_t n, int &i, int &j, int &k) {
    const unsigned u = (unsigned)n, im = (unsigned)d.IM, jm = (unsigned)d.JM;
    const unsigned q = u / im, q2 = q / jm;
    i = (int)(u - q * im) + 1;
    j = (int)(q - q2 * jm) + 1;
    k = (int)q2 + 1;
}

// One addition of a long parallel reduction (the tree sums of the multigrid
// levels, row means, monitors and mixing-plane averages).  REDUCE_ORDER 0,
// the default precision split, adds in FP64.  REDUCE_ORDER 2, the plain FP32
// path, rounds every partial sum to REAL*4: the same tree, with FP32 adds
// (a float sum of two floats, held exactly in a double).  REDUCE_ORDER 1
// forms these sums elsewhere, sequentially in the reference's order.
__device__ __forceinline__ double racc(int order, double s, double x) {
    return order == 2 ? (double)((float)s + (float)x) : s + x;
}

// A double-float: the unevaluated sum hi + lo of two FP32 values with |lo|
// at most half an ulp of hi, a 48-bit significand.  The TSTEP kernels'
// long sums of the default precision split accumulate in it rather than in
// FP64: GB300 issues very few FP64 instructions per clock, and the FP64 tree
// sums that every CTA forms in its prologue or epilogue queued behind one
// another on each SM's FP64 pipe.  An addition is two of Knuth's TwoSum and
// two of Dekker's Fast2Sum (the accurate double-double addition), all in
// FP32; these error-free transformations need every sum rounded on its own,
// which the library's --fmad=false build guarantees (they hold no products).
__device__ __forceinline__ df df_of(float x) { return df{x, 0.0f}; }
__device__ __forceinline__ float df_val(df a) { return a.hi + a.lo; }
__device__ __forceinline__ df df_add(df a, df b) {
    float s = a.hi + b.hi;
    float bv = s - a.hi;
    float e = (a.hi - (s - bv)) + (b.hi - bv);          // a.hi + b.hi = s + e exactly
    float t = a.lo + b.lo;
    float tv = t - a.lo;
    float f = (a.lo - (t - tv)) + (b.lo - tv);          // a.lo + b.lo = t + f exactly
    e = e + t;
    float s2 = s + e;
    e = e - (s2 - s);
    e = e + f;
    float s3 = s2 + e;
    return df{s3, e - (s3 - s2)};
}
__device__ __forceinline__ df df_shfl_down(df v, int o) {
    return df{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
}
__device__ __forceinline__ df df_shfl_xor(df v, int o) {
    return df{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}
// One addition of a long sum: double-float for REDUCE_ORDER 0, FP32 (every
// partial sum rounded to REAL*4) for REDUCE_ORDER 2, the plain FP32 path.
__device__ __forceinline__ df dacc(int order, df s, df x) {
    return order == 2 ? df{s.hi + x.hi, 0.0f} : df_add(s, x);
}

// Order-preserving key for "largest value, earliest index wins": the value
// must be >= 0 (squares, absolute values); NaN counts as smallest.
__device__ inline unsigned long long max_key(float v, size_t lin) {
    if (!(v >= 0.0f)) return 0ull;
    return ((unsigned long long)__float_as_uint(v) << 32) | (unsigned long long)(0xFFFFFFFFu - (unsigned)lin);
}

// ---------------------------------------------------------------------
// kernel launch wrappers (defined in the .cu files); each enqueues on s
// ---------------------------------------------------------------------
// Optional per-kernel event trace (mgpu_profile_steps): each launch wrapper
// calls mark() after a launch, so consecutive events bracket one kernel.
struct Prof {
    static constexpr int MAXEV = 4096;
    cudaEvent_t ev[MAXEV];
    const char *name[MAXEV];
    int n = 0;
};

struct Launch {
    cudaStream_t s;
    int sm_count;
    Prof *prof = nullptr;
    // programmatic dependent launch: the kernel may be scheduled while its
    // predecessor in the stream drains; every kernel calls pdl_wait() before
    // it touches memory, which returns once the predecessor has completed
    // and its writes are visible
    bool pdl = false;
};

// No kernel triggers its dependent early (griddepcontrol.launch_dependents):
// the dependent's CTAs would then hold SM slots while they wait, and in a
// batch graph those slots belong to the other instances' kernels (the
// 64-instance batch ran 13 % slower with an early trigger; one stage gained
// nothing measurable).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline void launchk(const Launch &L, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = L.s;
    cudaLaunchAttribute at[1];
    if (L.pdl) {
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
    }
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

inline void mark(const Launch &L, const char *name) {
    if (L.prof && L.prof->n < Prof::MAXEV) {
        cudaEventRecord(L.prof->ev[L.prof->n], L.s);
        L.prof->name[L.prof->n] = name;
        L.prof->n++;
    }
}

void launch_step_begin(const Dev &d, Launch L);
void launch_prim(const Dev &d, Launch L);
void launch_loss(const Dev &d, Launch L, bool init_call);
void launch_new_loss(const Dev &d, Launch L, bool init_call);
// pieces NEW_LOSS and SPAL_LOSS share: the laminar viscosity for the first
// quarter of the steps, SET_PWALLGRAD, and the wall shear stresses, face
// stresses and force update (mgpu_loss.cu)
void launch_loss_prologue(const Dev &d, Launch L, bool init_call);
void launch_pwallgrad(const Dev &d, Launch L, bool init_call);
void launch_viscous_walls_and_forces(const Dev &d, Launch L, bool init_call);
void launch_roavg_cell(const Dev &d, Launch L);
size_t new_loss_work_floats(const Dev &d);
// mass fluxes FLOWX/FLOWT/FLOWR, ROWT, WT and the energy fluxes of ROE
void launch_flux_mass_energy(const Dev &d, Launch L);
// inlet/exit conditions: the pitchwise sums and PD(K) (one CTA), then the
// boundary states; the sums read only values final before TSTEP(RO, ROE)
void launch_bc_sums(const Dev &d, Launch L);
void launch_bc_apply(const Dev &d, Launch L);
void launch_setflo(const Dev &d, Launch L);       // IN_FLOW != 0
void launch_cusp(const Dev &d, Launch L);         // IF_CUSP = 2 rows
// XMOM, RVT and RMOM fluxes; also PEFF (4321) and the density limiter's
// column flags
void launch_flux_mom(const Dev &d, Launch L);
// TSTEP for the nv variables v0 .. v0+nv-1 of d.var
void launch_tstep(const Dev &d, Launch L, int v0, int nv);
void launch_limiters(const Dev &d, Launch L);
void launch_mixplan(const Dev &d, Launch L);
// node arrays at the start of the Spalart-Allmaras work buffer (SAW); then
// REYNOLDS(1..64) and the scalars VORTICITY_FAC, PGRAD_FAC and the inlet
// density RO(IMID,1,KMID) before the inlet condition
__host__ __device__ inline size_t sa_work_node_floats(const Dev &d) { return (size_t)6 * d.IM * d.JM * d.KM; }
// Spalart-Allmaras (mgpu_sa.cu): the transported viscosity's step after
// TSTEP(RO) and the cell-average density, its inlet value after the inlet
// condition, and SPAL_LOSS
void launch_sa_transport(const Dev &d, Launch L);
void launch_sa_inlet(const Dev &d, Launch L);
void launch_spal_loss(const Dev &d, Launch L, bool init_call);
size_t sa_work_floats(const Dev &d);
// TSTEP's flux sum, SCREE, multigrid and residual smoothing of STORE for the
// nv variables from v0 (the stages TSTEP shares with the transported
// viscosity), mgpu_tstep.cu
void launch_tstep_cells_prolong(const Dev &d, Launch L, int v0, int nv);
void launch_tail(const Dev &d, Launch L);
void launch_stepup(const Dev &d, Launch L, float relax, bool gated);
void launch_integrals(const Dev &d, Launch L, double *out8);

// Raises a kernel's dynamic shared-memory limit to `bytes` (at least the
// 48 KB default) and never lowers it: the limit belongs to the function, not
// to a handle, so handles of different sizes (a batch) must not shrink one
// another's.
inline cudaError_t raise_smem(const void *f, size_t bytes) {
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, f);
    if (e != cudaSuccess) return e;
    const int want = (int)(bytes > 48 * 1024 ? bytes : 48 * 1024);
    if (a.maxDynamicSharedSizeBytes >= want) return cudaSuccess;
    return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, want);
}

// sets per-kernel attributes (dynamic shared memory of the J-plane kernels
// and of the LOSS kernels)
cudaError_t configure_kernels(const Dev &d);
cudaError_t configure_loss_kernels(const Dev &d);
cudaError_t configure_flux_kernels(const Dev &d);

// one LOOP iteration without the LOSS and tail bodies, eager launches on
// L.s (mgpu_api.cu)
void enqueue_step_core(const Dev &d, Launch L);

// floats recorded per (row interface, K) by k_mixplan for the adjoint: the
// five conserved variables at (IMID, JP1), then per I those at JP2 and JP3
__host__ __device__ inline int mix_rec_size(int im) { return 5 + 10 * im; }

// SETUP's face areas and volumes (mgpu_metrics.cu), in float or double:
// from X, R (J,K), RTHETA (I,J,K), INDMIX and WRAD (J) to the face areas,
// volumes, ABT and WRABT; THETA, TEMP1 and TEMP2 are work arrays of IJK size.
template <typename T>
struct MetricArgs {
    const T *X, *R, *RTHETA;
    const int *INDMIX;
    const float *WRAD;
    T *THETA, *TEMP1, *TEMP2;
    T *AQX, *AQR, *ABX, *ABR, *VOL, *ASX, *ASR, *VOLOR;
    T *ABT, *WRABT;
};
template <typename T>
cudaError_t launch_setup_metrics(int IM, int JM, int KM, const MetricArgs<T> &a, cudaStream_t s);

// SETUP's grid from a deck's NS blade sections (mgpu_metrics.cu).
struct GeoArgs {
    int IM, JM, KM, NS, KMID;
    const float *sec;                 // (4, NS, JM): XSURF, RSURF, RT_UPP, RT_THICK
    const float *FR, *FP;             // normalised spacings
    const int *NROW, *NBLADE, *INDMIX;
    const int *JSTART, *JLE, *JTE, *JMIX, *KTIPS, *KTIPE, *KS1, *KS2;
    const float *FRACTIP, *FTHICK;    // (NROWS, 2), (NROWS, KM)
    float *SMERID, *SH;               // work: (NS, JM), (JM)
    float *X, *R, *RTU, *RTT;         // (J, K)
    float *RTHETA;                    // (I, J, K)
};
cudaError_t launch_setup_geometry(const GeoArgs &g, cudaStream_t s);

// Read-only view of a handle, for entry points defined outside mgpu_api.cu.
struct HandleView {
    const Dev *d;
    cudaStream_t stream;
    int device;
    bool committed;
};
HandleView handle_view(const mgpu_handle *h);
// The discrete adjoint (mgpu_adjoint.cu) keeps its state beside the handle.
struct AdjState;
void adj_destroy(AdjState *a);
AdjState *&handle_adj(mgpu_handle *h);
Dev &handle_dev(mgpu_handle *h);
int handle_sm_count(const mgpu_handle *h);
double *handle_int_buf(mgpu_handle *h);        // (4, JM) FP64 integrals scratch
const void *handle_array(const mgpu_handle *h, const char *name, size_t *bytes);
// Records msg for mgpu_last_error() and returns code.
int api_fail(int code, const char *msg);

}  // namespace mgpu
