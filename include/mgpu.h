/*
 * mgpu.h -- C ABI of the GB300 time-marching library for Multall-open 18.3.
 *
 * The library replaces the numeric body of SUBROUTINE LOOP
 * (multall-open-18.3.f:3664-5463): per step it recovers the primitive
 * variables, forms the mass / energy / momentum face fluxes, calls the
 * SCREE/SSS update TSTEP five times (multigrid, negative feedback, corner
 * scatter, SMOOTH_VAR, periodic / tip-gap / mixing-plane averaging), applies
 * the inlet and exit boundary conditions, the density and Mach limiters and
 * NEW_MIXPLAN, runs LOSS every NLOS steps and, every 5 steps, the convergence
 * monitors and STEPUP.  All flow-field arrays stay resident on one GPU.
 *
 * Reference call site replaced: `CALL LOOP` at multall-open-18.3.f:137.  The
 * reference has no FFI of its own: LOOP takes no arguments and exchanges all
 * data through COMMON blocks (commall-open-18.3:13-203).  This ABI therefore
 * binds arrays and scalars BY THEIR COMMON NAMES: a Fortran ISO_C_BINDING
 * shim passes `C_LOC(AQX)` under the name "AQX" and so on, once, after
 * SETUP.  Arrays are passed packed, Fortran order, I fastest:
 *   3-D node/cell arrays  A(I,J,K)  -> IM*JM*KM values
 *   2-D meridional        A(J,K)    -> JM*KM
 *   2-D pitch/span        A(I,K)    -> IM*KM      (FBL, FBR, FTL, FTR)
 *   2-D endwall           A(I,J)    -> IM*JM      (YPLUS_K1, YPLUS_KM)
 *   per-J / per-I / per-K / per-row 1-D arrays of length JM / IM / KM / NROWS
 *   STEP1(NIB1,NJB1+1,NKB1), STEP2(NIB2,NJB2+1,NKB2), STEPSBK(NSBLK)
 * A shim on a compiled-in ID/JD/KD layout passes the sections
 * RO(1:IM,1:JM,1:KM) etc., which gfortran packs on the call.
 *
 * Conventions (all entry points):
 *   - return 0 on success, a negative MGPU_E_* code on failure; the text of
 *     the last failure on this thread is available from mgpu_last_error();
 *   - no C++ exception crosses the ABI; nothing here calls exit();
 *   - one handle = one flow problem = one CUDA stream owned by the handle;
 *     calls on one handle are not re-entrant, distinct handles are
 *     independent;
 *   - host buffers passed in are only read (set_*) or only written (get_*)
 *     during the call; the library keeps no host pointer.
 */
#ifndef MGPU_H_
#define MGPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGPU_ABI_VERSION 1

/* status codes */
#define MGPU_OK              0
#define MGPU_E_ARG          -1  /* bad argument, unknown name, size mismatch   */
#define MGPU_E_STATE        -2  /* call out of order (e.g. step before commit) */
#define MGPU_E_CUDA         -3  /* CUDA runtime error                          */
#define MGPU_E_UNSUPPORTED  -4  /* an input option the library does not cover */
#define MGPU_E_NONFINITE    -5  /* health check: NaN/Inf or RO <= 0 found      */
#define MGPU_E_NOMEM        -6  /* device allocation failed                    */

typedef struct mgpu_handle mgpu_handle;

/* Per-step monitors, the quantities LOOP prints every 5 steps
 * (multall-open-18.3.f:5264-5317, 3840-3864, 9000 FORMAT).  Filled by
 * mgpu_step()/mgpu_run() on steps where the 5-step tail ran (tail_ran=1). */
typedef struct mgpu_monitors {
    int32_t nstep;        /* NSTEP of the step these values belong to       */
    int32_t tail_ran;     /* 1 if the every-5-step tail ran on this step    */
    int32_t ifend;        /* convergence / NSTEPS_MAX test after this step  */
    int32_t health;       /* 0 ok, else count of non-finite or RO<=0 nodes  */
    float   emax;         /* signed max % change of Vm  (EMAX)              */
    int32_t imax, jmax, kmax;
    float   eavg;         /* mean |% change of Vm|      (EAVG)              */
    float   econt;        /* max |1 - CHECK_FLOW(J)/CHECK_FLOW(1)| (ECONT)  */
    int32_t jcont;
    float   vref;         /* SQRT(VRMS*RIJKM)           (VREF)              */
    float   vmax;         /* max relative speed         (VMAX)              */
    int32_t ivmax, jvmax, kvmax;
    double  flow_in;      /* BLADE_FLOW(1)  [kg/s]                          */
    double  flow_out;     /* BLADE_FLOW(JM) [kg/s]                          */
} mgpu_monitors;

/* Whole-machine performance, EFICOOL with IFCOOL=0
 * (multall-open-18.3.f:10662-10849, 11253-11394; SUMFLX 7873-7912). */
typedef struct mgpu_integrals {
    double mass_flow_in;   /* BLADE_FLOW(J1)                                */
    double mass_flow_out;  /* BLADE_FLOW(J2M1)                              */
    double eta_tt;         /* total-to-total isentropic efficiency ETAIS    */
    double eta_ts;         /* total-to-static efficiency ETATS              */
    double po_ratio;       /* PORAT = PO2/POIN                              */
    double to_ratio;       /* TORAT = TO_OUT/TO_IN                          */
    int32_t j1, j2m1;      /* stations used                                 */
} mgpu_integrals;

/* One row of EFICOOL's stage table (multall-open-18.3.f:11253-11420,
 * IFCOOL = 0): the mass-averaged performance between the stations j1 and
 * j2m1 and, for a stage, the reactions at hub, mid-span and tip from the
 * pitchwise static pressures at j1, jmix and j2m1. */
typedef struct mgpu_stage {
    int32_t j1, j2m1, jmix;   /* stations (J1, J2M1, JMIX_STAGE)             */
    int32_t has_reaction;     /* 0 for the whole machine                      */
    double mass_flow_in;      /* BLADE_FLOW(J1)                               */
    double mass_flow_out;     /* BLADE_FLOW(J2M1)                             */
    double po_ratio, to_ratio, delta_to;   /* PORAT, TORAT, DELTO             */
    double eta_tt, eta_ts, eta_poly;       /* ETAIS, ETATS, EPOLY             */
    double reac_hub, reac_mid, reac_tip;   /* REAC_HUB, REAC_MID, REAC_TIP    */
} mgpu_stage;

/* ---- library information --------------------------------------------- */
int32_t mgpu_abi_version(void);
/* Copies the text of the last error raised on the calling thread. */
int32_t mgpu_last_error(char *buf, int32_t len);
/* Number of CUDA devices visible; negative code if the runtime fails. */
int32_t mgpu_device_count(void);

/* ---- handle lifetime -------------------------------------------------- */
/* Creates a problem of IM x JM x KM nodes and NROWS blade rows on the
 * current CUDA device (replaces the COMMON PARAMETER sizing, commall:4-9).
 * Allocates the device working set. */
int32_t mgpu_create(int32_t im, int32_t jm, int32_t km, int32_t nrows,
                    mgpu_handle **out);
void    mgpu_destroy(mgpu_handle *h);

/* ---- binding COMMON data (before mgpu_commit) -------------------------- */
/* Integer / real COMMON scalars by name, e.g. "ITIMST", "CFL". */
int32_t mgpu_set_int(mgpu_handle *h, const char *name, int32_t value);
int32_t mgpu_set_real(mgpu_handle *h, const char *name, float value);
/* Copies a packed COMMON array (float32 for REAL, int32 for INTEGER) to
 * the device.  nbytes must equal the array's packed size.  State arrays
 * (RO, ROVX, ... ) may also be set after commit, e.g. on restart. */
int32_t mgpu_set_array(mgpu_handle *h, const char *name,
                       const void *host, int64_t nbytes);
/* Copies a packed COMMON array back from the device into host memory. */
int32_t mgpu_get_array(mgpu_handle *h, const char *name,
                       void *host, int64_t nbytes);
/* Reads back a real / integer scalar the loop updates (e.g. "VISLAM"). */
int32_t mgpu_get_real(mgpu_handle *h, const char *name, float *value);
int32_t mgpu_get_int(mgpu_handle *h, const char *name, int32_t *value);

/* Validates that every input LOOP reads has been bound, rejects options
 * outside the covered set with MGPU_E_UNSUPPORTED, derives the tables
 * LOSS builds on its first call, and performs the LOOP prologue
 * (multall-open-18.3.f:3677-3709: RO_REF, ROLIM, PLIM, PREFF, SFXIN/SFTIN
 * scaled by CFL).  NSTEP starts at 0. */
int32_t mgpu_commit(mgpu_handle *h);

/* ---- the calls SETUP makes into the hot path --------------------------- */
/* STEPUP(RELAX), multall-open-18.3.f:7916-8002 (SETUP calls it with 1.0 at
 * 7057, LOOP with 0.25 at 5349).  Valid after commit. */
int32_t mgpu_stepup(mgpu_handle *h, float relax);
/* LOSS called from SETUP with RF_VIS=1, FMIXUP=1, NSTEP=1
 * (multall-open-18.3.f:7350-7357) to initialise the body forces. */
int32_t mgpu_loss_init(mgpu_handle *h);

/* ---- time marching ----------------------------------------------------- */
/* One LOOP iteration, multall-open-18.3.f:5000-5240 plus the every-5-step
 * tail 8000-5438 (monitors, STEPUP; printing is left to the caller).
 * force_end=1 marks the final step (IFEND): the tail runs whatever NSTEP.
 * mon may be NULL.  Returns MGPU_E_NONFINITE if the tail's health check
 * finds a NaN/Inf or a non-positive density. */
int32_t mgpu_step(mgpu_handle *h, int32_t force_end, mgpu_monitors *mon);
/* Up to nsteps LOOP iterations (CUDA graph replay); mon receives the last
 * tail's values.  The steps between two tails are launched back to back and
 * the control block is read once per tail.  Returns 1 right after the final
 * step (IFEND: the convergence test of multall-open-18.3.f:3762-3764 met at
 * a tail, or NSTEP reaching NSTEPS_MAX), where LOOP stops (5444-5451), and
 * at once, without stepping, on a handle whose final step has run; 0 when
 * all nsteps ran without reaching it. */
int32_t mgpu_run(mgpu_handle *h, int32_t nsteps, mgpu_monitors *mon);
/* Bytes one mgpu_step() call moves between host and device: the
 * end-of-run flag it sends and the control block (monitors) it reads back. */
int32_t mgpu_step_io_bytes(int32_t *h2d, int32_t *d2h);
/* Blocks until all work on the handle's stream has finished. */
int32_t mgpu_sync(mgpu_handle *h);
/* EFICOOL's mass averages and efficiencies on the current state, computed
 * on the device with FP64 accumulation. */
int32_t mgpu_integrals_compute(mgpu_handle *h, mgpu_integrals *out);

/* EFICOOL's table for stage nstg = 1..NSTAGES, or with nstg = NSTAGES+1 for
 * the whole machine (multi-stage machines only, as EFICOOL prints it).  The
 * stage of each row comes from the integer row array NSTAGE (bound like the
 * COMMON arrays); the stations follow the reader's JSTG_START/JSTG_END
 * (1522-1536).  The mass averages are the FP64 sums of
 * mgpu_integrals_compute; the pitchwise pressures of the reactions are
 * summed in REAL*4 in the reference's order. */
int32_t mgpu_stage_performance(mgpu_handle *h, int32_t nstg, mgpu_stage *out);

/* ---- restart / plotting file ------------------------------------------- */
/* Writes the combined restart/plotting file "flow_out" from the device
 * state, as OUTPUT writes it (multall-open-18.3.f:5942-5978): the records
 * NSTEP, RO, ROVX, ROVR, ROVT, ROE, ROSUB, DPDS_CELL*1.0E-6 and PEFF+PREFF
 * (PREFF = (P(IMID,1,KMID) + P(IMID,JM,KMID))/2 of the current pressures)
 * in gfortran's sequential unformatted layout (each record between two
 * 4-byte byte counts).  rosub: the caller's packed ROSUB, which LOOP does
 * not change for ITIMST = 3, or NULL to write RO in its place.  Valid after
 * mgpu_commit. */
int32_t mgpu_write_flow_out(mgpu_handle *h, const char *path, const float *rosub);
/* Reads a flow_out file as SETUP's IF_RESTART branch does
 * (multall-open-18.3.f:6920-6992): sets RO, ROVX, ROVR, ROVT and ROE from it
 * and forms RORVT, VX, VR, VT, T_STATIC, HO, P, PEFF = P and, for IPOUT 0 or
 * -1, the exit pressures PD.  Valid after the COMMON arrays are bound and
 * before mgpu_commit, whose LOOP prologue (PREFF, ROLIM, PLIM) then starts
 * from the restarted flow.  *nstep (may be NULL) receives the file's NSTEP;
 * like LOOP, the step counter itself starts again from the bound NSTEP. */
int32_t mgpu_read_flow_out(mgpu_handle *h, const char *path, int32_t *nstep);
/* Writes the plotting file "grid_out" as SETUP writes it (6585-6597): the
 * records NSTEPS_MAX; IM, JM, KM; CP, GA; INDLETE(J) (1 on the leading- and
 * trailing-edge planes, 6307-6309); WRAD(J); NBLADE(J); then for each J and
 * K (K fastest) X, R and RTHETA(1..IM), from the bound COMMON data. */
int32_t mgpu_write_grid_out(mgpu_handle *h, const char *path);

/* ---- SETUP's metrics on the device ------------------------------------ */
/* Forms THETA = RTHETA/R, the theta extrapolated onto the upstream side of
 * each mixing plane, and SETUP's face areas and volumes (multall-open-
 * 18.3.f:6490-6502, 6570-6578, 6605-6711): AQX, AQR, ABT, WRABT, ABX, ABR,
 * VOL, ASX, ASR and VOLOR, from the bound X, R, RTHETA, INDMIX and WRAD, in
 * REAL*4 in SETUP's order of operations, and binds them.  Replaces SETUP's
 * metric loops for a caller that binds the grid instead of the areas.
 * Valid before mgpu_commit (the geometry is fixed after it). */
int32_t mgpu_setup_metrics(mgpu_handle *h);
/* SETUP's grid from a deck's blade sections, then its metrics: NEW_INTPOL
 * (multall-open-18.3.f:7493-7613) onto the KM stream surfaces with the
 * tip-gap grid, the alignment of the rows at mid-span (6442-6448), the
 * pinched-tip thickness (6452-6459) and RTHETA (6490-6501), in REAL*4 in
 * SETUP's order of operations; binds X, R, RT_THICK and RTHETA and then
 * does what mgpu_setup_metrics does.  sections: XSURF, RSURF, RT_UPP and
 * RT_THICK of the nsecs input sections as the reader leaves them, each
 * (nsecs, JM) with J fastest; fthick: FTHICK (NROWS, KM) with K fastest;
 * fractip: FRACTIP1, FRACTIP2 per row.  Needs FR and FP (normalised), NROW,
 * NBLADE, INDMIX, JSTART, JLE, JTE, JMIX, KTIPS, KTIPE, KS1, KS2 and WRAD
 * bound.  Valid before mgpu_commit. */
int32_t mgpu_setup_geometry(mgpu_handle *h, int32_t nsecs, const float *sections, const float *fthick,
                            const float *fractip);
/* The same metrics in double precision from double X, R (JM*KM each) and
 * RTHETA (IM*JM*KM), with the handle's INDMIX and WRAD; the handle is not
 * changed.  out receives AQX, AQR, ABX, ABR, VOL, ASX, ASR, VOLOR (IM*JM*KM
 * each) then ABT, WRABT (JM*KM each); n_out is its length in doubles.  For
 * geometry sensitivities, where REAL*4 metrics would bury a small change of
 * the grid in rounding.  Valid once INDMIX and WRAD are bound. */
int32_t mgpu_setup_metrics64(mgpu_handle *h, const double *x, const double *r, const double *rtheta, double *out,
                             int64_t n_out);

/* The same integrals as mgpu_integrals_compute, through a path that
 * allocates nothing.  This entry point has no counterpart in the reference
 * (whose efficiency summary is plain Fortran over COMMON arrays).
 *
 * Who needs it: a caller that must not allocate once the solver is
 * marching -- a Fortran driver that sized the problem to fill the device
 * from fixed COMMON extents, a monitoring thread that reports the
 * efficiency during a long run, a host whose own allocator holds the rest
 * of device memory.  mgpu_integrals_compute allocates host memory on every
 * call and overwrites the handle's node-sized work arrays; this variant
 * allocates no device or host memory (no cudaMalloc/cudaFree, no library
 * routine that allocates; only recording an error message for
 * mgpu_last_error may take host memory) and writes nothing of the handle's
 * arrays.  Its scratch is
 * one fixed array of (4 * MGPU_NOALLOC_MAX_JM + 8) doubles (131,136 bytes)
 * in the library's static device memory, one copy per device and process.
 *
 * Limits and rules:
 *  - JM (the handle's J extent) must be <= MGPU_NOALLOC_MAX_JM; larger
 *    problems are rejected with MGPU_E_ARG before any device work.
 *  - Nothing in the scratch has to start at zero: every slot a call reads
 *    it has written earlier in the same call.
 *  - The first call on each device looks up the scratch's device address
 *    (with the handle's device current, which it must be: otherwise
 *    MGPU_E_STATE) and loads this path's two kernels, so that under CUDA's
 *    lazy module loading no later call loads a module (which could take
 *    device memory).  A call with out == NULL performs only this set-up
 *    and returns 0; make it once per device before marching begins.
 *  - Every call with out != NULL synchronises the handle's stream and
 *    copies its results to the host, so it must not be made while that
 *    stream is capturing.
 *  - Calls whose executions overlap in time on the same device (two host
 *    threads, or two handles on one device) share the one scratch array and
 *    race: serialise them.  The call returns only after its results are on
 *    the host. */
#define MGPU_NOALLOC_MAX_JM 4096
int32_t mgpu_integrals_noalloc(mgpu_handle *h, mgpu_integrals *out);

/* ---- batches of independent problems ----------------------------------- */
/* No counterpart in the reference, which marches one problem per process.
 * A batch steps several committed handles (operating points, grids of any
 * size) with one CUDA graph launch per LOOP iteration: the graph holds one
 * branch per handle, so the kernels of all instances share the GPU at the
 * same time.  The handles must live on the current device and outlive the
 * batch; each keeps its own NSTEP, monitors and end test, and every value it
 * computes is bitwise the same as when the handle is stepped alone.  Do not
 * step a member on its own while a batch call is running. */
typedef struct mgpu_batch mgpu_batch;
int32_t mgpu_batch_create(mgpu_handle *const *handles, int32_t n, mgpu_batch **out);
void    mgpu_batch_destroy(mgpu_batch *b);
/* nsteps iterations of every member, launched back to back.  mons (n
 * entries, or NULL) receives each member's control block after the last
 * step.  Returns the number of members whose end test (convergence,
 * NSTEPS_MAX) has been met; they keep marching with the others, so a caller
 * that wants them stopped builds a new batch without them.  Returns
 * MGPU_E_NONFINITE if a member's health check fails. */
int32_t mgpu_batch_run(mgpu_batch *b, int32_t nsteps, mgpu_monitors *mons);
/* As mgpu_bench_steps, for the whole batch. */
int32_t mgpu_batch_bench_steps(mgpu_batch *b, int32_t nsteps, int32_t flush_l2, double *total_ms);

/* ---- discrete adjoint -------------------------------------------------- */
/* No counterpart in the reference.  Gradients of the efficiency and mass
 * flow of a converged flow with respect to the geometry arrays, by the
 * discrete adjoint of one LOOP iteration (multall-open-18.3.f:3759-5240)
 * with the LOSS body forces and the STEPUP time steps held at their current
 * values (frozen mixing length; set FROZEN = 1 for a primal that holds them
 * too).  The converged state U* is a fixed point U* = G(U*, A); the adjoint
 * lambda = (dG/dU)^T lambda + (dJ/dU)^T is iterated like the flow itself,
 * and dJ/dA = dJ/dA|_U + lambda^T dG/dA.  Covered: SCREE without residual
 * smoothing, IPOUT = 0, IN_PRESS = 0, IN_VTAN = 0, IN_VR <= 0, mixing planes
 * with subsonic relative flow at JMIX+2; other options return
 * MGPU_E_UNSUPPORTED.  Where the density or Mach limiter acts in the
 * recorded step it is differentiated with the rows' limits (VLIMIT,
 * ROLIMIT) held. */

/* Records one step from the current state (the linearisation point),
 * restores the state, and resets the adjoint to zero. */
int32_t mgpu_adjoint_prepare(mgpu_handle *h);
/* Selects the objective: 0 eta_tt, 1 mass flow at the inlet station, 2 at
 * the exit station (the EFICOOL stations of mgpu_integrals_compute), -1
 * none (the plain transposed step).  *value = the objective at the
 * recorded step. */
int32_t mgpu_adjoint_objective(mgpu_handle *h, int32_t which, double *value);
/* n adjoint iterations lambda <- (dG/dU)^T lambda + (dJ/dU)^T, one CUDA
 * graph launch each; *rel_change (or NULL) = |lambda_n - lambda_(n-1)| /
 * |lambda_n| over the five conserved variables. */
int32_t mgpu_adjoint_iterate(mgpu_handle *h, int32_t n, double *rel_change);
/* Iterates until the relative change falls below tol or max_iters
 * iterations are done; returns 0 if converged, 1 if not. */
int32_t mgpu_adjoint_solve(mgpu_handle *h, int32_t max_iters, double tol, int32_t *iters, double *rel_change);
/* The same fixed point by restarted GMRES on the inner-step map,
 * (I - ((dG/dU)^T)^inner) lambda = sum_{i<inner} ((dG/dU)^T)^i (dJ/dU)^T: the
 * marching iteration acts as the preconditioner and GMRES removes the few
 * slow or growing modes that stall it (a frozen step can have a slowly
 * growing mode; the plain iteration then diverges).  Starts from the current
 * lambda; restart = basis size (2-200); *steps = transposed steps used in
 * all; *rel_residual = the preconditioned system's |b - A lambda| / |b|.
 * stall > 0 also ends the solve when a restart cycle lowers the residual by
 * less than that fraction of it (stagnation); 0 runs to tol or max_steps.
 * Returns 0 if converged, 1 if not.  Holds (restart + 4) packed adjoint
 * vectors (14 node arrays each) on the device. */
int32_t mgpu_adjoint_solve_krylov(mgpu_handle *h, int32_t inner, int32_t restart, int32_t max_steps, double tol,
                                  double stall, int32_t *steps, double *rel_residual);
/* One more reverse step that also accumulates dJ/dA for the geometry
 * arrays AQX, AQR, ABX, ABR, ABT, ASX, ASR and VOLOR. */
int32_t mgpu_adjoint_gradient(mgpu_handle *h);
/* dJ/dTHETA (IM*JM*KM values, per radian) from the geometry gradient of the
 * last mgpu_adjoint_gradient.  SETUP's face areas and volumes (3030-4045)
 * are linear in the node angles THETA for fixed X and R, so this is the
 * transposed metric map applied to dJ/d(AQX, AQR, ABX, ABR, ASX, ASR,
 * VOLOR), through the extrapolation of THETA onto the mixing planes
 * (3025).  Computed on the device. */
int32_t mgpu_adjoint_gradient_theta(mgpu_handle *h, float *djdtheta, int64_t nbytes);
/* The adjoint of a state array by its COMMON name (RO, ROVX, ROVR, RORVT,
 * ROE, DRO, DROE, DROVX, DROVR, DRORVT, P, HO, ROVT, PEFF, PD), or, with a
 * "d" prefix (dAQX ...), the geometry gradient of mgpu_adjoint_gradient.
 * Packed like the COMMON array, FP32. */
int32_t mgpu_adjoint_get(mgpu_handle *h, const char *name, float *out, int64_t nbytes);
/* Sets the adjoint of a state array (a user-defined objective's seed, or
 * a test of the transposed step). */
int32_t mgpu_adjoint_set(mgpu_handle *h, const char *name, const float *in, int64_t nbytes);

/* ---- instrumentation --------------------------------------------------- */
/* The reference prints "CPU TIME PER STEP" every 50 steps
 * (multall-open-18.3.f:5404-5414); these are the device-side equivalents. */

/* Number of kernel launches one LOOP iteration issues from the step graph:
 * which = 0 a plain step, 1 a LOSS step, 2 a tail step (every 5th), 3 a step
 * that is both. */
int32_t mgpu_kernels_per_step(mgpu_handle *h, int32_t which);
/* The autotuner: times each of the two TSTEP launches of a step (RO and
 * ROE; the three momenta) with 128, 192, 256 and 512 threads per J-plane CTA
 * on the handle's current arrays, restores them, and keeps the fastest size
 * of each launch for the handle's step graph.  chosen (2 entries, or NULL)
 * = the threads per CTA of the RO/ROE launch and of the momentum launch;
 * ms (8 entries, or NULL) = the time of one launch per candidate, the RO/ROE
 * launch's four first.  The default without tuning is 256 for both.  The
 * candidates differ in the association of per-plane sums (FP32 within a
 * thread, FP64 across threads), so a tuned handle is deterministic for its
 * choice; two choices can differ in the last bits of a value.  A member of
 * a batch keeps its own choice. */
int32_t mgpu_autotune(mgpu_handle *h, int32_t *chosen, double *ms);
/* Runs nsteps iterations, each bracketed by CUDA events on the handle's
 * stream; with flush_l2=1 a buffer larger than L2 is rewritten between the
 * iterations (outside the events).  *total_ms = sum of the iteration
 * times. */
int32_t mgpu_bench_steps(mgpu_handle *h, int32_t nsteps, int32_t flush_l2, double *total_ms);

typedef struct mgpu_kernel_time {
    char    name[48];
    int32_t launches;
    double  total_ms;
} mgpu_kernel_time;
/* Runs nsteps iterations launching kernel by kernel (no graph) with a CUDA
 * event after each launch, and reports per kernel its launch count and
 * summed duration.  *n_out = entries written (<= max_entries). */
int32_t mgpu_profile_steps(mgpu_handle *h, int32_t nsteps, mgpu_kernel_time *out, int32_t max_entries,
                           int32_t *n_out);

#ifdef __cplusplus
}
#endif
#endif /* MGPU_H_ */
