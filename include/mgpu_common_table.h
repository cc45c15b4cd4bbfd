/*
 * mgpu_common_table.h -- the COMMON-block contract of the mgpu C ABI.
 *
 * Every scalar and array that the time-marching loop of Multall-open 18.3
 * reads or updates, listed under its COMMON name (commall-open-18.3:13-203)
 * together with its type and packed shape.  The shim binds by these names;
 * the device library and the CPU oracle use this one table, so both agree on
 * what a name means.  X-macro form:
 *
 *   MGPU_INT_SCALARS:  M_(NAME, default)             INTEGER scalar
 *   MGPU_REAL_SCALARS: M_(NAME, default)             REAL scalar
 *   MGPU_ARRAYS:       M_(NAME, type, shape, role)   array; type INT32/FLOAT32,
 *       shape  IJK  IM*JM*KM     JK  JM*KM     IK  IM*KM     IJ  IM*JM
 *              J   JM           I   IM        K   KM        ROW NROWS
 *              MG1 NIB1*(NJB1+1)*NKB1         MG2 NIB2*(NJB2+1)*NKB2
 *              SB  NSBLK
 *       role   GEOM  constant input, must be bound before commit
 *              OPT   constant input of an option (IF_CUSP=2), must be bound
 *                    before commit when a row uses that option
 *              STATE evolves in the loop, must be bound, can be read back
 *              OUT   produced by the loop, readable only
 *
 * A scalar default of NAN-like sentinel (-1e30f / INT32_MIN) marks a value
 * that must be set explicitly.
 */
#ifndef MGPU_COMMON_TABLE_H_
#define MGPU_COMMON_TABLE_H_

#define MGPU_REQUIRED_REAL (-1.0e30f)
#define MGPU_REQUIRED_INT  (-2147483647 - 1)

/* ----- INTEGER scalars: /BKINTG/, /BKLOSS/, /BKMGRD/, /BKSTAG/ ... ------ */
#define MGPU_INT_SCALARS(M_)                                              \
    M_(ITIMST,   3)                                                       \
    M_(ILOS,     10)                                                      \
    M_(NLOS,     5)                                                       \
    M_(IBOUND,   0)                                                       \
    M_(IFMIX,    1)                                                       \
    M_(IPOUT,    0)                                                       \
    M_(IN_PRESS, 0)                                                       \
    M_(IN_VTAN,  0)                                                       \
    M_(IN_VR,    0)                                                       \
    M_(IN_FLOW,  0)                                                       \
    M_(IF_REPEAT,0)                                                       \
    M_(NRSMTH,   0)                                                       \
    M_(NSFEXIT,  0)                                                       \
    M_(NSTEPS_MAX, MGPU_REQUIRED_INT)                                     \
    M_(NCHANGE,  MGPU_REQUIRED_INT)                                       \
    M_(NMIXUP,   1000)                                                    \
    M_(IF_RESTART, 0)                                                     \
    M_(IR,       3)                                                       \
    M_(JR,       3)                                                       \
    M_(KR,       3)                                                       \
    M_(NIB1,     MGPU_REQUIRED_INT)                                       \
    M_(NJB1,     MGPU_REQUIRED_INT)                                       \
    M_(NKB1,     MGPU_REQUIRED_INT)                                       \
    M_(NIB2,     MGPU_REQUIRED_INT)                                       \
    M_(NJB2,     MGPU_REQUIRED_INT)                                       \
    M_(NKB2,     MGPU_REQUIRED_INT)                                       \
    M_(NSBLK,    MGPU_REQUIRED_INT)                                       \
    M_(NSTAGES,  1)                                                       \
    M_(IFGAS,    0)                                                       \
    M_(IFCOOL,   0)                                                       \
    M_(IFBLEED,  0)                                                       \
    M_(IFSHROUD, 0)                                                       \
    M_(NSTEP,    0)                                                       \
    /* not a COMMON variable: order of the long reductions on the GPU,   */ \
    /* 0 = FP64 tree sums (default), 1 = the reference's sequential REAL*4 */ \
    /* order for the superblock and row-average sums (parity checks),    */ \
    /* 2 = the trees of 0 with FP32 adds (the plain FP32 path)           */ \
    M_(REDUCE_ORDER, 0)                                                   \
    /* not a COMMON variable: 1 holds the LOSS body forces and the STEPUP */ \
    /* time steps at their current values (frozen-turbulence stepping,    */ \
    /* the primal of the discrete adjoint)                                */ \
    M_(FROZEN,   0)                                                       \
    /* not a COMMON variable: threads per J-plane CTA of TSTEP, 128, 256  */ \
    /* or 512 (0: 256 until mgpu_autotune chooses)                        */ \
    M_(TS_THREADS, 0)                                                     \
    /* not a COMMON variable: 1 (default) runs TSTEP's damping and corner */ \
    /* gather over pairs of J-planes (one CTA of twice the threads per    */ \
    /* pair), 0 one CTA per J-plane; the results are bitwise the same     */ \
    M_(TS_PAIR, 1)

/* ----- REAL scalars: /BKGAS/, /BKCNTL/, /BKSMTH/, /BKLOSS/, /BKINPT/ ---- */
#define MGPU_REAL_SCALARS(M_)                                             \
    M_(CP,        MGPU_REQUIRED_REAL)                                     \
    M_(GA,        MGPU_REQUIRED_REAL)                                     \
    M_(CFL,       0.4f)                                                   \
    M_(DAMPIN,    10.0f)                                                  \
    M_(MACHLIM,   2.0f)                                                   \
    M_(F_PDOWN,   0.0f)                                                   \
    M_(SFXIN,     0.005f)                                                 \
    M_(SFTIN,     0.005f)                                                 \
    M_(FAC_4TH,   0.8f)                                                   \
    M_(RFIN,      0.25f)                                                  \
    M_(FEXTRAP,   0.8f)                                                   \
    M_(RFMIX,     0.025f)                                                 \
    M_(FSMTHB,    1.0f)                                                   \
    M_(FANGLE,    0.8f)                                                   \
    M_(SFEXIT,    0.0f)                                                   \
    M_(RSMTH,     0.4f)                                                   \
    M_(F1,        2.0f)                                                   \
    M_(F2,        -1.0f)                                                  \
    M_(F3,        0.0f)                                                   \
    M_(REYNO,     MGPU_REQUIRED_REAL)                                     \
    M_(RF_VIS,    0.5f)                                                   \
    M_(FTRANS,    0.0001f)                                                \
    M_(PRANDTL,   1.0f)                                                   \
    M_(YPLUSWALL, 0.0f)                                                   \
    M_(YPLAM,     5.0f)                                                   \
    M_(YPTURB,    25.0f)                                                  \
    M_(CFWALL,    0.0f)                                                   \
    M_(FACMIXUP,  2.0f)                                                   \
    M_(VORT_MAX,  0.0f)                                                   \
    M_(TURBVIS_LIM, 3000.0f)                                              \
    M_(PDOWN_HUB, MGPU_REQUIRED_REAL)                                     \
    M_(PDOWN_TIP, MGPU_REQUIRED_REAL)                                     \
    M_(PLATE_LOSS, 0.0f)                                                  \
    M_(THROTTLE_EXIT, 0.0f)                                               \
    M_(THROTTLE_PRES, 0.0f)                                               \
    M_(THROTTLE_MAS, 0.0f)                                                \
    M_(RFTHROTL,  0.0f)                                                   \
    M_(FLOWIN,    0.0f)                                                   \
    M_(RFLOW,     0.0f)                                                   \
    M_(VSOUND,    MGPU_REQUIRED_REAL)                                     \
    M_(CONLIM,    0.001f)                                                 \
    M_(VISLAM,    0.0f)                                                   \
    M_(FTCOND,    0.0f)                                                   \
    /* Spalart-Allmaras (ILOS >= 200) source-term factors, reader 631-652 */ \
    M_(FAC_STMIX, 0.0f)                                                   \
    M_(FAC_ST0,   1.0f)                                                   \
    M_(FAC_ST1,   1.0f)                                                   \
    M_(FAC_ST2,   1.0f)                                                   \
    M_(FAC_ST3,   1.0f)                                                   \
    M_(FAC_SFVIS, 2.0f)                                                   \
    M_(FAC_VORT,  0.0f)                                                   \
    M_(FAC_PGRAD, 0.0f)

/* ----- arrays ------------------------------------------------------------ */
#define MGPU_ARRAYS(M_)                                                   \
    /* per blade row */                                                  \
    M_(JSTART,   INT32,   ROW, GEOM)                                      \
    M_(JMIX,     INT32,   ROW, GEOM)                                      \
    M_(JLE,      INT32,   ROW, GEOM)                                      \
    M_(JTE,      INT32,   ROW, GEOM)                                      \
    M_(JLED,     INT32,   ROW, GEOM)                                      \
    M_(KTIPS,    INT32,   ROW, GEOM)                                      \
    M_(KTIPE,    INT32,   ROW, GEOM)                                      \
    M_(KS1,      INT32,   ROW, GEOM)                                      \
    M_(KS2,      INT32,   ROW, GEOM)                                      \
    M_(JTRAN_I1, INT32,   ROW, GEOM)                                      \
    M_(JTRAN_IM, INT32,   ROW, GEOM)                                      \
    M_(JTRAN_K1, INT32,   ROW, GEOM)                                      \
    M_(JTRAN_KM, INT32,   ROW, GEOM)                                      \
    M_(IF_CUSP,  INT32,   ROW, GEOM)                                      \
    M_(XLLIM_I1, FLOAT32, ROW, GEOM)                                      \
    M_(XLLIM_IM, FLOAT32, ROW, GEOM)                                      \
    M_(XLLIM_K1, FLOAT32, ROW, GEOM)                                      \
    M_(XLLIM_KM, FLOAT32, ROW, GEOM)                                      \
    M_(XLLIM_DWN,FLOAT32, ROW, GEOM)                                      \
    M_(XLLIM_UP, FLOAT32, ROW, GEOM)                                      \
    M_(ROUGH_H,  FLOAT32, ROW, GEOM)                                      \
    M_(ROUGH_T,  FLOAT32, ROW, GEOM)                                      \
    M_(ROUGH_L,  FLOAT32, ROW, GEOM)                                      \
    M_(ROUGH_U,  FLOAT32, ROW, GEOM)                                      \
    M_(CHORD,    FLOAT32, ROW, GEOM)                                      \
    M_(NUP_I1,   INT32,   ROW, OPT)                                       \
    M_(NUP_IM,   INT32,   ROW, OPT)                                       \
    M_(N_WAKE,   INT32,   ROW, OPT)                                       \
    M_(SEP_THIK, FLOAT32, ROW, OPT)                                       \
    M_(SEP_DRAG, FLOAT32, ROW, OPT)                                       \
    M_(NSTAGE,   INT32,   ROW, OPT)     /* stage of each row (EFICOOL) */ \
    /* Spalart-Allmaras: free-stream turbulence and mixing-plane decay   */ \
    /* of the transported viscosity (reader 2070-2073)                   */ \
    M_(FSTURB,   FLOAT32, ROW, OPT)                                       \
    M_(TURBVIS_DAMP, FLOAT32, ROW, OPT)                                   \
    /* per streamwise station J */                                       \
    M_(NBLADE,   INT32,   J,   GEOM)                                      \
    M_(IND,      INT32,   J,   GEOM)                                      \
    M_(INDLE,    INT32,   J,   GEOM)                                      \
    M_(INDMIX,   INT32,   J,   GEOM)                                      \
    M_(NROW,     INT32,   J,   GEOM)                                      \
    M_(JB1,      INT32,   J,   GEOM)                                      \
    M_(JB2,      INT32,   J,   GEOM)                                      \
    M_(JSBLK,    INT32,   J,   GEOM)                                      \
    M_(WRAD,     FLOAT32, J,   GEOM)                                      \
    M_(WHUB,     FLOAT32, J,   GEOM)                                      \
    M_(WTIP,     FLOAT32, J,   GEOM)                                      \
    M_(FACUP,    FLOAT32, J,   GEOM)                                      \
    M_(FACDWN,   FLOAT32, J,   GEOM)                                      \
    /* per pitchwise index I */                                          \
    M_(FP,       FLOAT32, I,   GEOM)                                      \
    M_(FU,       FLOAT32, I,   GEOM)                                      \
    M_(FD,       FLOAT32, I,   GEOM)                                      \
    M_(IB1,      INT32,   I,   GEOM)                                      \
    M_(IB2,      INT32,   I,   GEOM)                                      \
    /* per spanwise index K */                                           \
    M_(FR,       FLOAT32, K,   GEOM)                                      \
    M_(FKU,      FLOAT32, K,   GEOM)                                      \
    M_(FKD,      FLOAT32, K,   GEOM)                                      \
    M_(KB1,      INT32,   K,   GEOM)                                      \
    M_(KB2,      INT32,   K,   GEOM)                                      \
    M_(PO1,      FLOAT32, K,   GEOM)                                      \
    M_(TO1,      FLOAT32, K,   GEOM)                                      \
    M_(RPO1,     FLOAT32, K,   GEOM)                                      \
    M_(BSSIN,    FLOAT32, K,   GEOM)                                      \
    M_(BSCOS,    FLOAT32, K,   GEOM)                                      \
    M_(BRSIN,    FLOAT32, K,   GEOM)                                      \
    M_(BRCOS,    FLOAT32, K,   GEOM)                                      \
    M_(VTIN,     FLOAT32, K,   GEOM)                                      \
    M_(VM1,      FLOAT32, K,   GEOM)                                      \
    M_(PD,       FLOAT32, K,   STATE)                                     \
    /* corner-distribution weights, /BKDIST/ */                          \
    M_(FBL,      FLOAT32, IK,  GEOM)                                      \
    M_(FBR,      FLOAT32, IK,  GEOM)                                      \
    M_(FTL,      FLOAT32, IK,  GEOM)                                      \
    M_(FTR,      FLOAT32, IK,  GEOM)                                      \
    /* meridional geometry, /BKGEOM/ /BKAREA/ /BKSTAG/ */                 \
    M_(X,        FLOAT32, JK,  GEOM)                                      \
    M_(RT_THICK, FLOAT32, JK,  OPT)                                       \
    M_(R,        FLOAT32, JK,  GEOM)                                      \
    M_(ABT,      FLOAT32, JK,  GEOM)                                      \
    M_(WRABT,    FLOAT32, JK,  GEOM)                                      \
    M_(UBLADE,   FLOAT32, JK,  GEOM)                                      \
    M_(RAVG_CELL,FLOAT32, JK,  GEOM)                                      \
    M_(DX,       FLOAT32, JK,  GEOM)                                      \
    M_(DR,       FLOAT32, JK,  GEOM)                                      \
    M_(DS,       FLOAT32, JK,  GEOM)                                      \
    M_(SMERID,   FLOAT32, JK,  GEOM)                                      \
    M_(YPLUS_I1, FLOAT32, JK,  STATE)                                     \
    M_(YPLUS_IM, FLOAT32, JK,  STATE)                                     \
    M_(YPLUS_K1, FLOAT32, IJ,  STATE)                                     \
    M_(YPLUS_KM, FLOAT32, IJ,  STATE)                                     \
    /* face areas, volumes, time steps, wall distance */                 \
    M_(AQX,      FLOAT32, IJK, GEOM)                                      \
    M_(AQR,      FLOAT32, IJK, GEOM)                                      \
    M_(ABX,      FLOAT32, IJK, GEOM)                                      \
    M_(ABR,      FLOAT32, IJK, GEOM)                                      \
    M_(ASX,      FLOAT32, IJK, GEOM)                                      \
    M_(ASR,      FLOAT32, IJK, GEOM)                                      \
    M_(VOL,      FLOAT32, IJK, GEOM)                                      \
    M_(VOLOR,    FLOAT32, IJK, GEOM)                                      \
    M_(BSTEP,    FLOAT32, IJK, GEOM)                                      \
    M_(DWALLSQ,  FLOAT32, IJK, GEOM)                                      \
    /* NEW_LOSS (ILOS 100-199) mixing lengths, SET_XLENGTH 12476-12492 */ \
    M_(XLENGTH,  FLOAT32, IJK, OPT)                                       \
    M_(FST_RAT,  FLOAT32, IJK, OPT)                                       \
    M_(ROAVG_CELL, FLOAT32, IJK, OPT)                                     \
    M_(RTHETA,   FLOAT32, IJK, OPT)                                       \
    /* multigrid block time steps, /BKMGRD/ */                           \
    M_(STEP1,    FLOAT32, MG1, GEOM)                                      \
    M_(STEP2,    FLOAT32, MG2, GEOM)                                      \
    M_(STEPSBK,  FLOAT32, SB,  GEOM)                                      \
    /* flow state, /BKPRIM/ /BKSEC/ /BKDIFF/ /BKLOSS/ /BKFLUX/ */          \
    M_(RO,       FLOAT32, IJK, STATE)                                     \
    M_(ROVX,     FLOAT32, IJK, STATE)                                     \
    M_(ROVR,     FLOAT32, IJK, STATE)                                     \
    M_(RORVT,    FLOAT32, IJK, STATE)                                     \
    M_(ROE,      FLOAT32, IJK, STATE)                                     \
    M_(ROVT,     FLOAT32, IJK, STATE)                                     \
    M_(ROWT,     FLOAT32, IJK, STATE)                                     \
    M_(VX,       FLOAT32, IJK, STATE)                                     \
    M_(VR,       FLOAT32, IJK, STATE)                                     \
    M_(VT,       FLOAT32, IJK, STATE)                                     \
    M_(WT,       FLOAT32, IJK, STATE)                                     \
    M_(P,        FLOAT32, IJK, STATE)                                     \
    M_(HO,       FLOAT32, IJK, STATE)                                     \
    M_(T_STATIC, FLOAT32, IJK, STATE)                                     \
    M_(PEFF,     FLOAT32, IJK, STATE)                                     \
    M_(DRO,      FLOAT32, IJK, STATE)                                     \
    M_(DROE,     FLOAT32, IJK, STATE)                                     \
    M_(DROVX,    FLOAT32, IJK, STATE)                                     \
    M_(DROVR,    FLOAT32, IJK, STATE)                                     \
    M_(DRORVT,   FLOAT32, IJK, STATE)                                     \
    M_(XFORCE,   FLOAT32, IJK, STATE)                                     \
    M_(RFORCE,   FLOAT32, IJK, STATE)                                     \
    M_(TFORCE,   FLOAT32, IJK, STATE)                                     \
    M_(QSOURCE,  FLOAT32, IJK, STATE)                                     \
    M_(STEP,     FLOAT32, IJK, STATE)                                     \
    M_(RSTEP,    FLOAT32, IJK, STATE)                                     \
    M_(Y_PLUS,   FLOAT32, IJK, STATE)                                     \
    M_(DPDS_CELL,FLOAT32, IJK, STATE)                                     \
    M_(VISC_RAT, FLOAT32, IJK, OUT)                                       \
    M_(VISC_LAM, FLOAT32, IJK, OUT)                                       \
    /* Spalart-Allmaras (ILOS >= 200): the transported (cell-centred)    */ \
    /* turbulent viscosity, its SCREE history, its kinematic value and    */ \
    /* its relaxed source term, /BKNEWLOS/                                */ \
    M_(TRANS_DYN_VIS, FLOAT32, IJK, OPT)                                  \
    M_(DEL_DYNVIS, FLOAT32, IJK, OPT)                                     \
    M_(TRANS_KVIS, FLOAT32, IJK, OPT)                                     \
    M_(T_SOURCE, FLOAT32, IJK, OPT)                                       \
    M_(VISC_TURB, FLOAT32, IJK, OUT)

#endif /* MGPU_COMMON_TABLE_H_ */
