/*
 * multall_oracle.cpp -- CPU ORACLE of the Multall-open 18.3 time-marching loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the GPU
 * library: the tests, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py may load it; the product path never does.
 *
 * It restates, in serial C++ and in the reference's own loop order, the
 * FORTRAN77 routines of multall-open-18.3.f that make up the hot path:
 *   LOOP            3664-5463   (step body 3759-5240, 5-step tail 8000-5349)
 *   TSTEP           5470-5932
 *   SMOOTH_VAR      15352-15594
 *   SMOOTH_RESID    14833-14917
 *   LOSS            8058-9066   (ILOS=10)
 *   NEW_LOSS        12522-13508 (ILOS 100-199) and the cell-average density 4255-4267
 *   SPAL_LOSS       13586-14832 (ILOS 200-299), GRADCELL 13516-13585, the
 *                   transported viscosity's fluxes 4279-4347, TSTEP's
 *                   NCALL = 2 branch 5736-5777 and its inlet value 4679-4689
 *   WALLFUN         15980-16047
 *   NEW_MIXPLAN     14922-15251
 *   STEPUP          7916-8002
 *   EFICOOL/SUMFLX  10662-10849, 11253-11394 / 7873-7912  (IFCOOL=0)
 * Templated on the REAL type: float reproduces the reference's REAL*4
 * arithmetic (build with -ffp-contract=off: the reference's x86-64 gfortran
 * build emits no FMA); double stands for the reference built with
 * -fdefault-real-8 (every REAL and literal promoted).
 *
 * Parity status: the reference ships no outputs, golden vectors or tests,
 * and no Fortran compiler exists where this is built, so this restatement
 * is NOT pinned against the reference's own results ("parity unpinned").
 *
 * Options covered (the rest are rejected at commit): ITIMST=3 (SCREE, or
 * SSS through F1,F2,F3,NRSMTH), ILOS=10, IFGAS=0, no cooling, bleed or
 * shroud, IN_FLOW=0, IF_REPEAT=0, IF_CUSP<2, IM>2, KM>2, no throttle or
 * plate loss.  Wall treatments: YPLUSWALL > 5 (fixed Y+), in [-0.001, 5) (log-law
 * skin friction), in (-10, -0.001) (Shih wall functions) and <= -10 (Shih
 * with the SET_PWALLGRAD pressure-gradient term).
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <string>
#include <vector>
#include <algorithm>
#include <type_traits>
#include <utility>

#include "../include/mgpu.h"
#include "../include/mgpu_common_table.h"
#include "ad_tape.h"

/* math on the REAL type: the std overloads for float and double, the tape's
   overloads (found by argument-dependent lookup) for adt::AD */
namespace om {
#define OM_FN1(f) template <class T> inline T f(const T &x) { using std::f; return f(x); }
OM_FN1(sqrt) OM_FN1(fabs) OM_FN1(log) OM_FN1(log10) OM_FN1(sin) OM_FN1(cos) OM_FN1(asin) OM_FN1(tanh)
#undef OM_FN1
template <class T> inline T pow(const T &x, const T &y) { using std::pow; return pow(x, y); }
template <class T> inline T atan2(const T &y, const T &x) { using std::atan2; return atan2(y, x); }
template <class T> inline bool isfinite(const T &x) { using std::isfinite; return isfinite(x); }
}  // namespace om

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

enum Shape { SH_IJK, SH_JK, SH_IK, SH_IJ, SH_J, SH_I, SH_K, SH_ROW, SH_MG1, SH_MG2, SH_SB };

struct OracleBase {
    virtual ~OracleBase() {}
    virtual int set_int(const char *n, int v) = 0;
    virtual int set_real(const char *n, double v) = 0;
    virtual int get_real(const char *n, double *v) = 0;
    virtual int get_int(const char *n, int *v) = 0;
    virtual int set_array(const char *n, const void *p, int64_t nb) = 0;
    virtual int get_array(const char *n, void *p, int64_t nb, int as_double) = 0;
    virtual int commit() = 0;
    virtual int stepup(double relax) = 0;
    virtual int loss_init() = 0;
    virtual int step(int force_end, mgpu_monitors *mon) = 0;
    virtual int integrals(mgpu_integrals *out) = 0;
    virtual int stage_performance(int nstg, mgpu_stage *out) = 0;
    /* reverse mode (the adt::AD instantiation only): ad_begin makes every
       REAL array of the COMMON table an independent variable and starts the
       tape; after a step, ad_seed adds output adjoints to the arrays' current
       values, ad_reverse sweeps the tape and ad_grad reads the adjoints of
       the arrays as they were at ad_begin */
    virtual int set_array_f64(const char *n, const double *p, int64_t cnt) = 0;
    virtual int ad_begin() { return fail(MGPU_E_STATE, "not a differentiating oracle"); }
    virtual int ad_zero() { return fail(MGPU_E_STATE, "not a differentiating oracle"); }
    virtual int ad_seed(const char *, const double *, int64_t) { return fail(MGPU_E_STATE, "not a differentiating oracle"); }
    virtual int ad_reverse() { return fail(MGPU_E_STATE, "not a differentiating oracle"); }
    virtual int ad_grad(const char *, double *, int64_t) { return fail(MGPU_E_STATE, "not a differentiating oracle"); }
    virtual int64_t ad_tape_size() { return 0; }
    /* the restart/plotting file flow_out (OUTPUT 5942-5978; SETUP's
       IF_RESTART branch 6920-6992) */
    virtual int write_flow_out(const char *, const float *) { return fail(MGPU_E_STATE, "flow_out needs a REAL oracle"); }
    virtual int read_flow_out(const char *, int *) { return fail(MGPU_E_STATE, "flow_out needs a REAL oracle"); }
    virtual int write_grid_out(const char *) { return fail(MGPU_E_STATE, "grid_out needs a REAL oracle"); }
};

/* gfortran's sequential unformatted records: the payload between two copies
   of its byte count (4-byte integers) */
bool fo_put(FILE *f, const void *p, uint32_t n) {
    return fwrite(&n, 4, 1, f) == 1 && (n == 0 || fwrite(p, 1, n, f) == n) && fwrite(&n, 4, 1, f) == 1;
}
bool fo_get(FILE *f, void *p, uint32_t n) {
    uint32_t a = 0, b = 0;
    if (fread(&a, 4, 1, f) != 1 || a != n) return false;
    if (p ? fread(p, 1, n, f) != n : fseek(f, (long)n, SEEK_CUR) != 0) return false;
    return fread(&b, 4, 1, f) == 1 && b == n;
}

template <typename R>
struct Oracle : OracleBase {
    typedef R Real;
    int IM, JM, KM, NROWS;
    int IMM1, JMM1, KMM1, IMM2, JMM2, KMM2, IMID, KMID, NRWSM1;
    bool committed = false;

#define O_DECL_I(n, d) int n = d;
    MGPU_INT_SCALARS(O_DECL_I)
#define O_DECL_R(n, d) R n = R(d);
    MGPU_REAL_SCALARS(O_DECL_R)
#define O_T_INT32 int
#define O_T_FLOAT32 R
#define O_DECL_A(n, t, s, r) std::vector<O_T_##t> n##_v; bool n##_set = false;
    MGPU_ARRAYS(O_DECL_A)

    /* COMMON variables the loop derives (SETUP 6459-6468, LOOP 3677-3709) */
    R GA1, FGA, RFGA, RCP, CV, RCV, RGAS;
    R RFTHROTL1 = R(1);
    R RO_REF, ROMIN, ROLIM, RIJKM, PREFF, RFIN1, RFIN2, TCOOL_MIN;
    R SFT = 0, SFX = 0, DAMP = 0, SFT1, SFTH, SFX1, SFXH, SFX15, SFX14, SFXB, SFXB1, SFXBH, SFXHM1;
    R FMIXUP = 1, ECONT, EAVG, EMAX, VRMS = 0, VMAX = 0, TCOND;
    int IFEND = 0, IFPRINT = 0;
    int IVMAX = 0, JVMAX = 0, KVMAX = 0, IMAXE = 0, JMAXE = 0, KMAXE = 0, JCONT = 0;
    std::vector<R> PLIM, VLIMIT, ROLIMIT, AVG_CHG, AVG_BLK, BLADE_FLOW, CHECK_FLOW;
    std::vector<R> FILAM, FITURB, FIWAKE, FIUP, FKLAM, FKTURB;   /* (NRS, IM|KM) */
    /* work arrays (COMMON /BKFLUX/ /BKFLOW/ /BKUTIL/ scratch) */
    std::vector<R> XFLUX, TFLUX, RFLUX, SOURCE, FLOWX, FLOWT, FLOWR, STORE, TEMP1;
    std::vector<R> B1CHG, B2CHG, SBCHG;

    Oracle(int im, int jm, int km, int nrows) : IM(im), JM(jm), KM(km), NROWS(nrows) {
        IMM1 = IM - 1; JMM1 = JM - 1; KMM1 = KM - 1;
        IMM2 = IM - 2; JMM2 = JM - 2; KMM2 = KM - 2;
        IMID = (int)(0.5f * IM);   /* IFIX(0.5*IM), SETUP 6299 */
        KMID = (int)(0.5f * KM);
        NRWSM1 = NROWS - 1;
    }

    /* ---- indexing: Fortran 1-based, packed, I fastest ------------------ */
    inline size_t ijk(int i, int j, int k) const {
        return (size_t)(i - 1) + (size_t)IM * ((size_t)(j - 1) + (size_t)JM * (size_t)(k - 1));
    }
    inline size_t jk(int j, int k) const { return (size_t)(j - 1) + (size_t)JM * (size_t)(k - 1); }
    inline size_t ik(int i, int k) const { return (size_t)(i - 1) + (size_t)IM * (size_t)(k - 1); }
    inline size_t ij(int i, int j) const { return (size_t)(i - 1) + (size_t)IM * (size_t)(j - 1); }
#define A3(a, i, j, k) a[ijk(i, j, k)]
#define F3(n, i, j, k) n##_v[ijk(i, j, k)]
#define F2(n, j, k) n##_v[jk(j, k)]
#define FIK(n, i, k) n##_v[ik(i, k)]
#define FIJ(n, i, j) n##_v[ij(i, j)]
#define F1(n, x) n##_v[(x) - 1]
#define ROWT2(a, nr, x, len) a[(size_t)((nr) - 1) * (len) + (x) - 1]

    size_t shape_count(Shape s) const {
        switch (s) {
        case SH_IJK: return (size_t)IM * JM * KM;
        case SH_JK: return (size_t)JM * KM;
        case SH_IK: return (size_t)IM * KM;
        case SH_IJ: return (size_t)IM * JM;
        case SH_J: return JM;
        case SH_I: return IM;
        case SH_K: return KM;
        case SH_ROW: return NROWS;
        case SH_MG1: return (size_t)NIB1 * (NJB1 + 1) * NKB1;
        case SH_MG2: return (size_t)NIB2 * (NJB2 + 1) * NKB2;
        case SH_SB: return NSBLK;
        }
        return 0;
    }

    int set_int(const char *n, int v) override {
#define O_SI(nm, d) if (!strcmp(n, #nm)) { nm = v; return 0; }
        MGPU_INT_SCALARS(O_SI)
        return fail(MGPU_E_ARG, std::string("unknown integer scalar ") + n);
    }
    int set_real(const char *n, double v) override {
#define O_SR(nm, d) if (!strcmp(n, #nm)) { nm = (R)(float)v; return 0; }
        MGPU_REAL_SCALARS(O_SR)
        return fail(MGPU_E_ARG, std::string("unknown real scalar ") + n);
    }
    int get_real(const char *n, double *v) override {
#define O_GR(nm, d) if (!strcmp(n, #nm)) { *v = (double)nm; return 0; }
        MGPU_REAL_SCALARS(O_GR)
        if (!strcmp(n, "PREFF")) { *v = (double)PREFF; return 0; }
        if (!strcmp(n, "SFT")) { *v = (double)SFT; return 0; }
        if (!strcmp(n, "SFX")) { *v = (double)SFX; return 0; }
        if (!strcmp(n, "DAMP")) { *v = (double)DAMP; return 0; }
        if (!strcmp(n, "FMIXUP")) { *v = (double)FMIXUP; return 0; }
        return fail(MGPU_E_ARG, std::string("unknown real scalar ") + n);
    }
    /* branch counters of the last step, for tests that must show a branch
       ran before they compare it: density-limiter changes (7200), Mach-
       limiter changes (7100: RO raised to RO_LIMIT or FACSAFE < 1), and
       NEW_MIXPLAN Prandtl-Meyer sweep updates (15151-15173) */
    int cnt_dens = 0, cnt_mach = 0, cnt_pm = 0;

    int get_int(const char *n, int *v) override {
        if (!strcmp(n, "ORACLE_NDENS")) { *v = cnt_dens; return 0; }
        if (!strcmp(n, "ORACLE_NMACH")) { *v = cnt_mach; return 0; }
        if (!strcmp(n, "ORACLE_NPM")) { *v = cnt_pm; return 0; }
#define O_GI(nm, d) if (!strcmp(n, #nm)) { *v = nm; return 0; }
        MGPU_INT_SCALARS(O_GI)
        return fail(MGPU_E_ARG, std::string("unknown integer scalar ") + n);
    }

    template <typename T>
    int put(std::vector<T> &dst, bool &flag, Shape s, bool is_int, const void *p, int64_t nb, const char *n) {
        size_t cnt = shape_count(s);
        if ((int64_t)(cnt * 4) != nb)
            return fail(MGPU_E_ARG, std::string("size mismatch for ") + n + ": expected " +
                                        std::to_string(cnt * 4) + " bytes, got " + std::to_string(nb));
        dst.resize(cnt);
        if (is_int) {
            const int32_t *q = (const int32_t *)p;
            for (size_t i = 0; i < cnt; ++i) dst[i] = (T)q[i];
        } else {
            const float *q = (const float *)p;
            for (size_t i = 0; i < cnt; ++i) dst[i] = (T)q[i];
        }
        flag = true;
        return 0;
    }
    template <typename T>
    int take(const std::vector<T> &src, Shape s, void *p, int64_t nb, int as_double, const char *n, bool is_int) {
        size_t cnt = shape_count(s);
        if (src.size() != cnt) return fail(MGPU_E_STATE, std::string("array not available: ") + n);
        if (as_double) {
            if ((int64_t)(cnt * 8) != nb) return fail(MGPU_E_ARG, std::string("size mismatch for ") + n);
            double *q = (double *)p;
            for (size_t i = 0; i < cnt; ++i) q[i] = (double)src[i];
        } else if (is_int) {
            if ((int64_t)(cnt * 4) != nb) return fail(MGPU_E_ARG, std::string("size mismatch for ") + n);
            int32_t *q = (int32_t *)p;
            for (size_t i = 0; i < cnt; ++i) q[i] = (int32_t)src[i];
        } else {
            if ((int64_t)(cnt * 4) != nb) return fail(MGPU_E_ARG, std::string("size mismatch for ") + n);
            float *q = (float *)p;
            for (size_t i = 0; i < cnt; ++i) q[i] = (float)src[i];
        }
        return 0;
    }
#define O_ISINT_INT32 true
#define O_ISINT_FLOAT32 false
    int set_array(const char *n, const void *p, int64_t nb) override {
#define O_SA(nm, t, s, r) if (!strcmp(n, #nm)) return put(nm##_v, nm##_set, SH_##s, O_ISINT_##t, p, nb, n);
        MGPU_ARRAYS(O_SA)
        return fail(MGPU_E_ARG, std::string("unknown array ") + n);
    }
    int get_array(const char *n, void *p, int64_t nb, int as_double) override {
#define O_GA(nm, t, s, r) if (!strcmp(n, #nm)) return take(nm##_v, SH_##s, p, nb, as_double, n, O_ISINT_##t);
        MGPU_ARRAYS(O_GA)
        if (!strcmp(n, "STORE")) return take(STORE, SH_IJK, p, nb, as_double, n, false);
        if (!strcmp(n, "FLOWX")) return take(FLOWX, SH_IJK, p, nb, as_double, n, false);
        return fail(MGPU_E_ARG, std::string("unknown array ") + n);
    }

    /* ---- flow_out: REAL*4 records for float, REAL*8 for double (the
       -fdefault-real-8 build) ------------------------------------------ */
    static constexpr bool kPlainReal = std::is_same<R, float>::value || std::is_same<R, double>::value;
    int write_flow_out(const char *path, const float *rosub) override {
        if constexpr (!kPlainReal) {
            return fail(MGPU_E_STATE, "flow_out needs a REAL oracle");
        } else {
            if (!committed) return fail(MGPU_E_STATE, "write_flow_out before commit");
            const size_t N = (size_t)IM * JM * KM;
            /* OUTPUT's own PREFF (5950) */
            const R PRF = R(0.5) * (F3(P, IMID, 1, KMID) + F3(P, IMID, JM, KMID));
            const R E6 = std::is_same<R, float>::value ? R(1.0e-6f) : R(1.0e-6);
            std::vector<R> dp(N), pe(N), rs(N);
            /* the seventh array: the transported viscosity with the S-A model,
               else DPDS_CELL * 1e-6 for plotting (5966-5972) */
            for (size_t n = 0; n < N; ++n) {
                dp[n] = ILOS >= 200 ? TRANS_DYN_VIS_v[n] : DPDS_CELL_v[n] * E6;
                pe[n] = PEFF_v[n] + PRF;
                rs[n] = rosub ? R(rosub[n]) : RO_v[n];
            }
            FILE *f = fopen(path, "wb");
            if (!f) return fail(MGPU_E_ARG, std::string("cannot open for writing: ") + path);
            const uint32_t rb = (uint32_t)(N * sizeof(R));
            int32_t ns = NSTEP;
            bool ok = fo_put(f, &ns, 4);
            const std::vector<R> *recs[] = {&RO_v, &ROVX_v, &ROVR_v, &ROVT_v, &ROE_v, &rs, &dp, &pe};
            for (auto *r : recs) ok = ok && fo_put(f, r->data(), rb);
            ok = fclose(f) == 0 && ok;
            return ok ? 0 : fail(MGPU_E_ARG, std::string("write failed: ") + path);
        }
    }
    /* SETUP's plotting file grid_out (6585-6597) */
    int write_grid_out(const char *path) override {
        if constexpr (!kPlainReal) {
            return fail(MGPU_E_STATE, "grid_out needs a REAL oracle");
        } else {
            std::vector<int32_t> INDLETE(JM, 0);     /* 6307-6309 */
            for (int j = 1; j <= JM; ++j)
                if (INDLE_v[j - 1] == 1) INDLETE[j - 1] = 1;
            for (int nr = 0; nr < NROWS; ++nr)
                if (JTE_v[nr] >= 1 && JTE_v[nr] <= JM) INDLETE[JTE_v[nr] - 1] = 1;
            FILE *f = fopen(path, "wb");
            if (!f) return fail(MGPU_E_ARG, std::string("cannot open for writing: ") + path);
            const int32_t ns = NSTEPS_MAX, dims[3] = {IM, JM, KM};
            const R gas[2] = {CP, GA};
            const std::vector<int32_t> nb(NBLADE_v.begin(), NBLADE_v.end());
            bool ok = fo_put(f, &ns, 4) && fo_put(f, dims, 12) && fo_put(f, gas, 2 * sizeof(R)) &&
                      fo_put(f, INDLETE.data(), (uint32_t)JM * 4) && fo_put(f, WRAD_v.data(), (uint32_t)(JM * sizeof(R))) &&
                      fo_put(f, nb.data(), (uint32_t)JM * 4);
            std::vector<R> rec((size_t)IM + 2);
            for (int j = 1; j <= JM && ok; ++j)
                for (int k = 1; k <= KM && ok; ++k) {
                    rec[0] = F2(X, j, k);
                    rec[1] = F2(R, j, k);
                    for (int i = 1; i <= IM; ++i) rec[(size_t)i + 1] = F3(RTHETA, i, j, k);
                    ok = fo_put(f, rec.data(), (uint32_t)(rec.size() * sizeof(R)));
                }
            ok = fclose(f) == 0 && ok;
            return ok ? 0 : fail(MGPU_E_ARG, std::string("write failed: ") + path);
        }
    }

    int read_flow_out(const char *path, int *nstep) override {
        if constexpr (!kPlainReal) {
            return fail(MGPU_E_STATE, "flow_out needs a REAL oracle");
        } else {
            if (committed) return fail(MGPU_E_STATE, "read_flow_out after commit (SETUP reads the restart file)");
            const size_t N = (size_t)IM * JM * KM;
            const uint32_t rb = (uint32_t)(N * sizeof(R));
            std::vector<R> ro(N), rovx(N), rovr(N), rovt(N), roe(N), tdv(N);
            int32_t ns = 0;
            FILE *f = fopen(path, "rb");
            if (!f) return fail(MGPU_E_ARG, std::string("cannot open: ") + path);
            /* the seventh array is read into TRANS_DYN_VIS whatever the model
               (6934) */
            const bool ok = fo_get(f, &ns, 4) && fo_get(f, ro.data(), rb) && fo_get(f, rovx.data(), rb) &&
                            fo_get(f, rovr.data(), rb) && fo_get(f, rovt.data(), rb) && fo_get(f, roe.data(), rb) &&
                            fo_get(f, nullptr, rb) && fo_get(f, tdv.data(), rb);
            fclose(f);
            if (!ok) return fail(MGPU_E_ARG, std::string("not a flow_out file of this grid: ") + path);
            if (!R_v.size() || !FP_v.size() || !PD_v.size()) return fail(MGPU_E_ARG, "bind R, FP and PD before the restart");
            const R CVr = CP / GA, RGASr = CP - CVr;   /* SETUP 6459-6468 */
            RO_v = ro; ROVX_v = rovx; ROVR_v = rovr; ROVT_v = rovt; ROE_v = roe;
            TRANS_DYN_VIS_v = tdv;
            TRANS_DYN_VIS_set = true;
            for (std::vector<R> *v : {&VX_v, &VR_v, &VT_v, &RORVT_v, &T_STATIC_v, &HO_v, &P_v, &PEFF_v}) v->assign(N, R(0));
            /* 3900, IFGAS = 0, ITIMST < 5 */
            for (int k = 1; k <= KM; ++k)
                for (int j = 1; j <= JM; ++j)
                    for (int i = 1; i <= IM; ++i) {
                        F3(VX, i, j, k) = F3(ROVX, i, j, k) / F3(RO, i, j, k);
                        F3(VR, i, j, k) = F3(ROVR, i, j, k) / F3(RO, i, j, k);
                        F3(VT, i, j, k) = F3(ROVT, i, j, k) / F3(RO, i, j, k);
                        F3(RORVT, i, j, k) = F3(ROVT, i, j, k) * F2(R, j, k);
                        const R EKE = R(0.5) * (F3(VX, i, j, k) * F3(VX, i, j, k) + F3(VR, i, j, k) * F3(VR, i, j, k) +
                                                F3(VT, i, j, k) * F3(VT, i, j, k));
                        const R TSTATIC = (F3(ROE, i, j, k) / F3(RO, i, j, k) - EKE) / CVr;
                        F3(T_STATIC, i, j, k) = TSTATIC;
                        F3(HO, i, j, k) = CP * TSTATIC + EKE;
                        F3(P, i, j, k) = F3(RO, i, j, k) * RGASr * TSTATIC;
                        F3(PEFF, i, j, k) = F3(P, i, j, k);
                    }
            /* 3902-3903 */
            if (IPOUT <= 0) {
                std::vector<R> PDOWN(KM + 1, R(0));
                for (int k = 1; k <= KM; ++k)
                    for (int i = 1; i <= IMM1; ++i)
                        PDOWN[k] = PDOWN[k] + FP_v[i - 1] * R(0.5) * (F3(P, i, JM, k) + F3(P, i + 1, JM, k));
                const R PDIFF = IPOUT == 0 ? PD_v[0] - PDOWN[1] : PD_v[KM - 1] - PDOWN[KM];
                for (int k = 1; k <= KM; ++k) PD_v[k - 1] = PDOWN[k] + PDIFF;
            }
            RO_set = ROVX_set = ROVR_set = ROVT_set = ROE_set = true;
            VX_set = VR_set = VT_set = RORVT_set = T_STATIC_set = HO_set = P_set = PEFF_set = true;
            if (nstep) *nstep = ns;
            return 0;
        }
    }

    /* ------------------------------------------------------------------ */
    int commit() override {
        if (IM <= 2 || KM <= 2) return fail(MGPU_E_UNSUPPORTED, "IM=2 (throughflow) or KM=2 (Q3D) not covered");
#define O_CHK_A(nm, t, s, r) \
    if (!nm##_set && std::string(#r) != "OUT" && std::string(#r) != "OPT") return fail(MGPU_E_ARG, "array not bound: " #nm);
        MGPU_ARRAYS(O_CHK_A)
#define O_CHK_I(nm, d) if (nm == MGPU_REQUIRED_INT) return fail(MGPU_E_ARG, "integer not set: " #nm);
        MGPU_INT_SCALARS(O_CHK_I)
#define O_CHK_R(nm, d) if ((float)nm == MGPU_REQUIRED_REAL) return fail(MGPU_E_ARG, "real not set: " #nm);
        MGPU_REAL_SCALARS(O_CHK_R)
        if (ITIMST != 3) return fail(MGPU_E_UNSUPPORTED, "ITIMST other than 3 (incompressible 5/6) not covered");
        if (ILOS != 0 && ILOS != 10 && !(ILOS >= 100 && ILOS < 300))
            return fail(MGPU_E_UNSUPPORTED,
                        "only ILOS=0 (inviscid), 10 (LOSS), 100-199 (NEW_LOSS) and 200-299 (SPAL_LOSS) are covered");
        if (ILOS >= 100 && !(VORT_MAX > R(0))) return fail(MGPU_E_ARG, "ILOS >= 100 needs VORT_MAX > 0 (SETUP 7322-7328)");
        if (ILOS >= 100 && !(XLENGTH_set && FST_RAT_set && ROAVG_CELL_set))
            return fail(MGPU_E_ARG, "ILOS >= 100 needs XLENGTH, FST_RAT and ROAVG_CELL");
        if (IFGAS != 0) return fail(MGPU_E_UNSUPPORTED, "real-gas IFGAS=1 not covered");
        if (IFCOOL || IFBLEED || IFSHROUD) return fail(MGPU_E_UNSUPPORTED, "cooling/bleed/shroud not covered");
        if (IF_REPEAT != 0) return fail(MGPU_E_UNSUPPORTED, "IF_REPEAT not covered");
        if (IPOUT == 3 || IPOUT < -1) return fail(MGPU_E_UNSUPPORTED, "IPOUT not covered");
        if (THROTTLE_EXIT > R(0.001) && THROTTLE_MAS == R(0)) return fail(MGPU_E_ARG, "THROTTLE_MAS must be set with THROTTLE_EXIT");
        bool cusp2 = false;
        for (int nr = 1; nr <= NROWS; ++nr) {
            if (F1(IF_CUSP, nr) > 2) return fail(MGPU_E_UNSUPPORTED, "IF_CUSP above 2 not covered");
            if (F1(IF_CUSP, nr) == 2) cusp2 = true;
        }
        if (cusp2 && !(NUP_I1_set && NUP_IM_set && N_WAKE_set && SEP_THIK_set && SEP_DRAG_set && RT_THICK_set && RTHETA_set))
            return fail(MGPU_E_ARG, "IF_CUSP=2 needs NUP_I1, NUP_IM, N_WAKE, SEP_THIK, SEP_DRAG, RT_THICK and RTHETA");
        RFTHROTL1 = R(1.0) - RFTHROTL;
        if (NCHANGE <= 0 || NMIXUP <= 0) return fail(MGPU_E_ARG, "NCHANGE and NMIXUP must be positive");

        size_t n3 = (size_t)IM * JM * KM;
        XFLUX.assign(n3, R(0)); TFLUX.assign(n3, R(0)); RFLUX.assign(n3, R(0));
        SOURCE.assign(n3, R(0)); FLOWX.assign(n3, R(0)); FLOWT.assign(n3, R(0));
        FLOWR.assign(n3, R(0)); STORE.assign(n3, R(0)); TEMP1.assign(n3, R(0));
        VISC_RAT_v.assign(n3, R(0));
        VISC_LAM_v.assign(n3, R(0));
        VISC_TURB_v.assign(n3, R(0));
        /* Spalart-Allmaras state: zero unless bound (SETUP 6905-6908), the
           reader's defaults FSTURB = 1, TURBVIS_DAMP = 0.5 (2052-2053) */
        if (!TRANS_DYN_VIS_set) TRANS_DYN_VIS_v.assign(n3, R(0));
        if (!DEL_DYNVIS_set) DEL_DYNVIS_v.assign(n3, R(0));
        if (!TRANS_KVIS_set) TRANS_KVIS_v.assign(n3, R(0));
        if (!T_SOURCE_set) T_SOURCE_v.assign(n3, R(0));
        if (!FSTURB_set) FSTURB_v.assign(NROWS, R(1.0));
        if (!TURBVIS_DAMP_set) TURBVIS_DAMP_v.assign(NROWS, R(0.5));
        PLIM.assign(KM, R(0)); VLIMIT.assign(NROWS, R(0)); ROLIMIT.assign(NROWS, R(0));
        AVG_CHG.assign(NROWS, R(0)); AVG_BLK.assign(NROWS, R(0));
        BLADE_FLOW.assign(JM, R(0)); CHECK_FLOW.assign(JM, R(0));
        FILAM.assign((size_t)NROWS * IM, R(0)); FITURB.assign((size_t)NROWS * IM, R(0));
        FIWAKE.assign((size_t)NROWS * IM, R(0)); FIUP.assign((size_t)NROWS * IM, R(0));
        FKLAM.assign((size_t)NROWS * KM, R(0)); FKTURB.assign((size_t)NROWS * KM, R(0));
        B1CHG.assign(shape_count(SH_MG1), R(0));
        B2CHG.assign(shape_count(SH_MG2), R(0));
        SBCHG.assign((size_t)NSBLK, R(0));

        /* gas constants, SETUP 6459-6468 */
        GA1 = GA - R(1.0);
        FGA = GA1 / GA;
        RFGA = R(1.0) / FGA;
        RCP = R(1.0) / CP;
        CV = CP / GA;
        RCV = R(1.0) / CV;
        RGAS = CP - CV;

        /* LOOP prologue 3677-3709 */
        RO_REF = F1(PO1, KMID) / (RGAS * F1(TO1, KMID));
        ROMIN = std::min(F3(RO, IMID, 1, KMID), F3(RO, IMID, JM, KMID));
        ROLIM = R(0.25) * ROMIN;
        RIJKM = R(2.) / R(IM * JM * KM);
        for (int k = 1; k <= KM; ++k) PLIM[k - 1] = R(0.9) * F1(PO1, k) + R(0.1) * F3(P, 1, 1, k);
        PREFF = R(0.5) * (F3(P, IMID, 1, KMID) + F3(P, IMID, JM, KMID));
        SFXIN = SFXIN * CFL / R(0.5);
        SFTIN = SFTIN * CFL / R(0.5);
        RFIN1 = R(1.0) - RFIN;
        RFIN2 = R(2.) * RFIN;
        ECONT = R(1.);
        EAVG = R(1.0E06);
        EMAX = R(1.0E06);
        TCOOL_MIN = R(1.0E6);
        IFEND = 0;
        committed = true;
        return 0;
    }

    /* ================================================================== */
    /*  STEPUP(RELAX)   multall-open-18.3.f:7916-8002                      */
    /* ================================================================== */
    int stepup(double relax_in) override {
        if (!committed) return fail(MGPU_E_STATE, "stepup before commit");
        R RELAX = (R)(float)relax_in;
        R TLIM = R(0.1) * F1(TO1, KMID);
        R VLIM = R(0.01) * F1(VM1, KMID) * F1(VM1, KMID);
        R RELAX1 = R(1.0) - RELAX;
        for (int k = 1; k <= KM; ++k)
            for (int j = 1; j <= JM; ++j)
                for (int i = 1; i <= IM; ++i) {
                    R vx = F3(VX, i, j, k), vt = F3(VT, i, j, k), vr = F3(VR, i, j, k);
                    R VSQ = vx * vx + vt * vt + vr * vr;
                    R HSTAT = F3(HO, i, j, k) - R(0.5) * VSQ;
                    R TSTATIC = HSTAT * RCP;
                    R GAMNOW = GA;
                    if (TSTATIC < TLIM) TSTATIC = TLIM;
                    R WTREL = F3(WT, i, j, k);
                    R WSQ = VSQ - (vt * vt - WTREL * WTREL);
                    if (WSQ < VLIM) WSQ = VLIM;
                    R V_SONIC = om::sqrt(GAMNOW * RGAS * TSTATIC);
                    R VPLUSC = om::sqrt(WSQ) + V_SONIC;
                    A3(TEMP1, i, j, k) = VSOUND / VPLUSC;
                }
        for (int i = 1; i <= IMM1; ++i) {
            int ip1 = i + 1;
            for (int k = 1; k <= KMM1; ++k) {
                int kp1 = k + 1;
                R AMACHP = A3(TEMP1, i, 1, k) + A3(TEMP1, ip1, 1, k) + A3(TEMP1, i, 1, kp1) + A3(TEMP1, ip1, 1, kp1);
                for (int j = 2; j <= JM; ++j) {
                    R AMACHL = A3(TEMP1, i, j, k) + A3(TEMP1, i, j, kp1) + A3(TEMP1, ip1, j, k) + A3(TEMP1, ip1, j, kp1);
                    R AVMACH = R(0.125) * (AMACHL + AMACHP);
                    AMACHP = AMACHL;
                    R STEPNEW = F3(BSTEP, i, j, k) * AVMACH;
                    F3(STEP, i, j, k) = RELAX * STEPNEW + RELAX1 * F3(STEP, i, j, k);
                    F3(RSTEP, i, j, k) = F3(STEP, i, j, k) / F3(BSTEP, i, j, k);
                }
            }
        }
        for (int nr = 1; nr <= NRWSM1; ++nr) {
            int j = F1(JMIX, nr);
            for (int k = 1; k <= KMM1; ++k)
                for (int i = 1; i <= IMM1; ++i) {
                    F3(STEP, i, j + 1, k) = F3(STEP, i, j + 2, k);
                    F3(RSTEP, i, j + 1, k) = R(0.0);
                }
        }
        return 0;
    }

    /* ================================================================== */
    /*  SMOOTH_RESID   multall-open-18.3.f:14833-14917                     */
    /* ================================================================== */
    void smooth_resid(std::vector<R> &VAR, R SMFAC, int NSMTH) {
        R SFAC1 = R(1.0) - SMFAC;
        R SFACH = R(0.5) * SMFAC;
        std::vector<R> tmp(std::max(std::max(IM, JM), KM) + 2);
        for (int nsm = 1; nsm <= NSMTH; ++nsm) {
            for (int nr = 1; nr <= NROWS; ++nr) {
                int J1 = F1(JSTART, nr), J1P1 = J1 + 1, J1P2 = J1 + 2, J2 = F1(JMIX, nr), J2M1 = J2 - 1;
                for (int k = 1; k <= KMM1; ++k)
                    for (int i = 1; i <= IMM1; ++i) {
                        for (int j = J1P2; j <= J2M1; ++j)
                            tmp[j] = SFAC1 * A3(VAR, i, j, k) + SFACH * (A3(VAR, i, j + 1, k) + A3(VAR, i, j - 1, k));
                        tmp[J1P1] = A3(VAR, i, J1P1, k) + SFACH * (A3(VAR, i, J1P2, k) - A3(VAR, i, J1P1, k));
                        tmp[J2] = A3(VAR, i, J2, k) + SFACH * (A3(VAR, i, J2M1, k) - A3(VAR, i, J2, k));
                        for (int j = J1P1; j <= J2; ++j) A3(VAR, i, j, k) = tmp[j];
                    }
                for (int k = 1; k <= KMM1; ++k)
                    for (int j = J1P1; j <= J2; ++j) {
                        for (int i = 2; i <= IMM2; ++i)
                            tmp[i] = SFAC1 * A3(VAR, i, j, k) + SFACH * (A3(VAR, i + 1, j, k) + A3(VAR, i - 1, j, k));
                        tmp[1] = A3(VAR, 1, j, k) + SFACH * (A3(VAR, 2, j, k) - A3(VAR, 1, j, k));
                        tmp[IMM1] = A3(VAR, IMM1, j, k) + SFACH * (A3(VAR, IMM2, j, k) - A3(VAR, IMM1, j, k));
                        for (int i = 1; i <= IMM1; ++i) A3(VAR, i, j, k) = tmp[i];
                    }
                for (int i = 1; i <= IMM1; ++i)
                    for (int j = J1P1; j <= J2; ++j) {
                        for (int k = 2; k <= KMM2; ++k)
                            tmp[k] = SFAC1 * A3(VAR, i, j, k) + SFACH * (A3(VAR, i, j, k + 1) + A3(VAR, i, j, k - 1));
                        tmp[1] = A3(VAR, i, j, 1) + SFACH * (A3(VAR, i, j, 2) - A3(VAR, i, j, 1));
                        tmp[KMM1] = A3(VAR, i, j, KMM1) + SFACH * (A3(VAR, i, j, KMM2) - A3(VAR, i, j, KMM1));
                        for (int k = 1; k <= KMM1; ++k) A3(VAR, i, j, k) = tmp[k];
                    }
            }
        }
    }

    /* ================================================================== */
    /*  SMOOTH_VAR(D)   multall-open-18.3.f:15352-15594                    */
    /* ================================================================== */
    void smooth_var(std::vector<R> &D) {
        const int NUM3 = 3;
        if (!(SFX < R(0.0001))) {
            for (int nr = 1; nr <= NROWS; ++nr) {
                int J1 = F1(JSTART, nr), J2 = F1(JMIX, nr);
                for (int j = J1 + 3; j <= J2 - 3; ++j)
                    for (int k = 1; k <= KM; ++k)
                        for (int i = 1; i <= IM; ++i) {
                            R AVERG = R(0.5) * (A3(D, i, j + 1, k) + A3(D, i, j - 1, k));
                            R CURV = AVERG - R(0.5) * A3(D, i, j, k) - R(0.25) * (A3(D, i, j - 2, k) + A3(D, i, j + 2, k));
                            A3(STORE, i, j, k) = SFX1 * A3(D, i, j, k) + SFX * (AVERG + FAC_4TH * CURV);
                        }
                for (int k = 1; k <= KM; ++k)
                    for (int i = 1; i <= IM; ++i) {
                        A3(STORE, i, J2, k) = A3(D, i, J2, k);
                        A3(STORE, i, J1, k) = A3(D, i, J1, k);
                    }
                for (int k = 1; k <= KM; ++k)
                    for (int i = 1; i <= IM; ++i) {
                        A3(STORE, i, J1 + 2, k) = SFXB1 * A3(D, i, J1 + 2, k) + SFXBH * (A3(D, i, J1 + 3, k) + A3(D, i, J1 + 1, k));
                        A3(STORE, i, J1 + 1, k) = SFXB1 * A3(D, i, J1 + 1, k) +
                            SFXB * (R(1.25) * A3(D, i, J1 + 2, k) + R(0.5) * A3(D, i, J1 + 3, k) - R(0.75) * A3(D, i, J1 + 4, k));
                        A3(STORE, i, J2 - 2, k) = SFXB1 * A3(D, i, J2 - 2, k) + SFXBH * (A3(D, i, J2 - 1, k) + A3(D, i, J2 - 3, k));
                        A3(STORE, i, J2 - 1, k) = SFXB1 * A3(D, i, J2 - 1, k) +
                            SFXB * (R(1.25) * A3(D, i, J2 - 2, k) + R(0.5) * A3(D, i, J2 - 3, k) - R(0.75) * A3(D, i, J2 - 4, k));
                    }
            }
            for (int nr = 1; nr <= NROWS; ++nr) {
                int JS = F1(JLED, nr) - 2, JE = JS + 1;
                for (int j = JS; j <= JE; ++j)
                    for (int k = 1; k <= KM; ++k) {
                        A3(STORE, 1, j, k) = SFXHM1 * A3(D, 1, j, k) + SFX14 * (A3(D, 2, j, k) + A3(D, IMM1, j, k));
                        A3(STORE, IM, j, k) = SFXHM1 * A3(D, IM, j, k) + SFX14 * (A3(D, 2, j, k) + A3(D, IMM1, j, k));
                    }
                int j = F1(JLED, nr);
                for (int k = 1; k <= KM; ++k) {
                    A3(STORE, 1, j, k) = SFXHM1 * A3(D, 1, j, k) + SFX14 * (A3(D, 1, j + 1, k) + A3(D, IM, j, k));
                    A3(STORE, IM, j, k) = SFXHM1 * A3(D, IM, j, k) + SFX14 * (A3(D, IM, j + 1, k) + A3(D, 1, j, k));
                }
            }
            for (int nr = 1; nr <= NROWS; ++nr) {
                int J1 = F1(JSTART, nr), J2 = F1(JMIX, nr);
                for (int j = J1; j <= J2; ++j)
                    for (int k = 1; k <= KM; ++k)
                        for (int i = 1; i <= IM; ++i) A3(D, i, j, k) = A3(STORE, i, j, k);
            }
        }
        if (!(SFT < R(0.0001))) {
            int LEN = std::max(IM, KM) + 1;
            std::vector<R> AVG(LEN), CURVE(LEN), SCURVE(LEN);
            for (int j = 2; j <= JM; ++j) {
                for (int k = 1; k <= KM; ++k) {
                    for (int i = 2; i <= IMM1; ++i) {
                        AVG[i] = F1(FD, i) * A3(D, i + 1, j, k) + F1(FU, i) * A3(D, i - 1, j, k);
                        CURVE[i] = A3(D, i, j, k) - AVG[i];
                    }
                    if (F1(IND, j) == 1 || F1(INDLE, j) == 1) {
                        AVG[1] = A3(D, 2, j, k) + F1(FU, 1) * (A3(D, 2, j, k) - A3(D, NUM3, j, k));
                        AVG[IM] = A3(D, IMM1, j, k) + F1(FU, IM) * (A3(D, IMM1, j, k) - A3(D, IMM2, j, k));
                        CURVE[1] = R(0.0); CURVE[IM] = R(0.0); SCURVE[1] = R(0.0); SCURVE[IM] = R(0.0);
                    } else {
                        AVG[1] = R(0.5) * (A3(D, 2, j, k) + A3(D, IMM1, j, k));
                        AVG[IM] = AVG[1];
                        CURVE[1] = A3(D, 1, j, k) - AVG[1];
                        CURVE[IM] = CURVE[1];
                        SCURVE[1] = R(0.5) * (CURVE[2] + CURVE[IMM1]);
                        SCURVE[IM] = SCURVE[1];
                    }
                    for (int i = 2; i <= IMM1; ++i) SCURVE[i] = F1(FU, i) * CURVE[i - 1] + F1(FD, i) * CURVE[i + 1];
                    for (int i = 1; i <= IM; ++i)
                        A3(D, i, j, k) = SFT1 * A3(D, i, j, k) + SFT * (AVG[i] + FAC_4TH * SCURVE[i]);
                }
                for (int i = 1; i <= IM; ++i) {
                    for (int k = 2; k <= KMM1; ++k) {
                        AVG[k] = F1(FKD, k) * A3(D, i, j, k + 1) + F1(FKU, k) * A3(D, i, j, k - 1);
                        CURVE[k] = A3(D, i, j, k) - AVG[k];
                    }
                    AVG[1] = A3(D, i, j, 2) + R(0.5) * F1(FKU, 1) * (A3(D, i, j, 2) - A3(D, i, j, 3));
                    AVG[KM] = A3(D, i, j, KMM1) + R(0.5) * F1(FKU, KM) * (A3(D, i, j, KMM1) - A3(D, i, j, KMM2));
                    CURVE[1] = R(0.0); CURVE[KM] = R(0.0); SCURVE[1] = R(0.0); SCURVE[KM] = R(0.0);
                    for (int k = 2; k <= KMM1; ++k) SCURVE[k] = F1(FKU, k) * CURVE[k - 1] + F1(FKD, k) * CURVE[k + 1];
                    for (int k = 1; k <= KM; ++k)
                        A3(D, i, j, k) = SFT1 * A3(D, i, j, k) + SFT * (AVG[k] + FAC_4TH * SCURVE[k]);
                }
                A3(D, 1, j, 1) = SFT1 * A3(D, 1, j, 1) + SFTH * (A3(D, 2, j, 1) + A3(D, 1, j, 2));
                A3(D, IM, j, 1) = SFT1 * A3(D, IM, j, 1) + SFTH * (A3(D, IMM1, j, 1) + A3(D, IM, j, 2));
                A3(D, 1, j, KM) = SFT1 * A3(D, 1, j, KM) + SFTH * (A3(D, 1, j, KMM1) + A3(D, 2, j, KM));
                A3(D, IM, j, KM) = SFT1 * A3(D, IM, j, KM) + SFTH * (A3(D, IMM1, j, KM) + A3(D, IM, j, KMM1));
            }
        }
        if (!(SFEXIT < R(0.0001))) {
            R SFEX1 = R(1.) - SFEXIT, SFEXH = R(0.5) * SFEXIT;
            int JSSTART = JM + 1 - NSFEXIT;
            for (int j = JSSTART; j <= JM; ++j) {
                for (int k = 1; k <= KM; ++k) {
                    for (int i = 2; i <= IMM1; ++i)
                        A3(D, i, j, k) = SFEX1 * A3(D, i, j, k) + SFEXH * (A3(D, i + 1, j, k) + A3(D, i - 1, j, k));
                    A3(D, 1, j, k) = A3(D, 1, j, k) + SFEXIT * (R(2.) * A3(D, 2, j, k) - A3(D, NUM3, j, k) - A3(D, 1, j, k));
                    A3(D, IM, j, k) = A3(D, IM, j, k) + SFEXIT * (R(2.) * A3(D, IMM1, j, k) - A3(D, IMM2, j, k) - A3(D, IM, j, k));
                }
                for (int i = 1; i <= IM; ++i) {
                    for (int k = 2; k <= KMM1; ++k)
                        A3(D, i, j, k) = SFEX1 * A3(D, i, j, k) + SFEXH * (A3(D, i, j, k - 1) + A3(D, i, j, k + 1));
                    A3(D, i, j, 1) = A3(D, i, j, 1) + SFEXIT * (R(2.) * A3(D, i, j, 2) - A3(D, i, j, 3) - A3(D, i, j, 1));
                    A3(D, i, j, KM) = A3(D, i, j, KM) + SFEXIT * (R(2.) * A3(D, i, j, KMM1) - A3(D, i, j, KMM2) - A3(D, i, j, KM));
                }
            }
        }
    }

    /* ================================================================== */
    /*  TSTEP(D, DIFF, NCALL)   multall-open-18.3.f:5470-5932               */
    /* ================================================================== */
    void tstep(std::vector<R> &D, std::vector<R> &DIFF, int NCALL = 1) {
        std::fill(B1CHG.begin(), B1CHG.end(), R(0.0));
        std::fill(B2CHG.begin(), B2CHG.end(), R(0.0));
        std::fill(SBCHG.begin(), SBCHG.end(), R(0.0));
        auto b1 = [&](int i1, int j1, int k1) -> R & {
            return B1CHG[(size_t)(i1 - 1) + (size_t)NIB1 * ((size_t)(j1 - 1) + (size_t)(NJB1 + 1) * (k1 - 1))];
        };
        auto b2 = [&](int i2, int j2, int k2) -> R & {
            return B2CHG[(size_t)(i2 - 1) + (size_t)NIB2 * ((size_t)(j2 - 1) + (size_t)(NJB2 + 1) * (k2 - 1))];
        };
        auto s1 = [&](int i1, int j1, int k1) -> R {
            return STEP1_v[(size_t)(i1 - 1) + (size_t)NIB1 * ((size_t)(j1 - 1) + (size_t)(NJB1 + 1) * (k1 - 1))];
        };
        auto s2 = [&](int i2, int j2, int k2) -> R {
            return STEP2_v[(size_t)(i2 - 1) + (size_t)NIB2 * ((size_t)(j2 - 1) + (size_t)(NJB2 + 1) * (k2 - 1))];
        };
        /* tip-gap flux balance 5503-5510 */
        for (int j = 2; j <= JM; ++j) {
            int nr = F1(NROW, j);
            if (F1(KTIPS, nr) <= 0) continue;
            for (int k = F1(KTIPS, nr); k <= F1(KTIPE, nr) - 1; ++k) {
                A3(TFLUX, 1, j, k) = R(0.5) * (A3(TFLUX, 1, j, k) + A3(TFLUX, IM, j, k));
                A3(TFLUX, IM, j, k) = A3(TFLUX, 1, j, k);
            }
        }
        /* mixing-plane upstream flux extrapolation 5516-5555 */
        if (!(FEXTRAP < R(0.001))) {
            for (int nr = 1; nr <= NRWSM1; ++nr) {
                int j = F1(JMIX, nr), jp1 = j + 1, jm1 = j - 1, jp2 = j + 2;
                for (int k = 1; k <= KMM1; ++k) {
                    R FLOWDIRN = -A3(FLOWX, IMID, j, k);
                    R AVFLXJM1 = R(0.0), AVFLXJP2 = R(0.0);
                    for (int i = 1; i <= IMM1; ++i) {
                        AVFLXJM1 = AVFLXJM1 + A3(XFLUX, i, jm1, k);
                        AVFLXJP2 = AVFLXJP2 + A3(XFLUX, i, jp2, k);
                    }
                    for (int i = 1; i <= IMM1; ++i) {
                        if (FLOWDIRN > R(0.0)) {
                            R DFLUX = (A3(XFLUX, i, jm1, k) - AVFLXJM1 * F1(FP, i)) * FEXTRAP;
                            A3(SOURCE, i, j, k) = A3(SOURCE, i, j, k) - DFLUX;
                        } else {
                            R DFLUX = (A3(XFLUX, i, jp2, k) - AVFLXJP2 * F1(FP, i)) * FEXTRAP;
                            A3(SOURCE, i, jp2, k) = A3(SOURCE, i, jp2, k) + DFLUX;
                        }
                        A3(SOURCE, i, jp1, k) = R(0.0);
                    }
                }
            }
        }
        /* flux sum and SCREE/SSS update 1000 */
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j) {
                R RATPITCH = R(F1(NBLADE, j - 1)) / R(F1(NBLADE, j));
                for (int i = 1; i <= IMM1; ++i) {
                    R DELTA = A3(XFLUX, i, j, k) - A3(XFLUX, i, j - 1, k) * RATPITCH + A3(RFLUX, i, j, k) -
                              A3(RFLUX, i, j, k + 1) + A3(TFLUX, i, j, k) - A3(TFLUX, i + 1, j, k) -
                              A3(SOURCE, i, j, k);
                    A3(STORE, i, j, k) = F1 * DELTA + F2 * A3(DIFF, i, j, k);
                    A3(DIFF, i, j, k) = DELTA + F3 * A3(DIFF, i, j, k);
                }
            }
        /* mixing-plane pitchwise redistribution 1750 */
        for (int nr = 1; nr <= NRWSM1; ++nr) {
            int j = F1(JMIX, nr);
            for (int k = 1; k <= KMM1; ++k) {
                R FLOWDIRN = -A3(FLOWX, IMID, j, k);
                if (FLOWDIRN > R(0.0) || FEXTRAP < R(0.001)) {
                    int jmx = j + 2;
                    R SUM_STORE = R(0.0);
                    for (int i = 1; i <= IMM1; ++i) SUM_STORE = SUM_STORE + A3(STORE, i, jmx, k);
                    for (int i = 1; i <= IMM1; ++i) A3(STORE, i, jmx, k) = SUM_STORE * F1(FP, i);
                }
                if (FLOWDIRN < R(0.0) || FEXTRAP < R(0.001)) {
                    R SUM_STORE = R(0.0);
                    for (int i = 1; i <= IMM1; ++i) SUM_STORE = SUM_STORE + A3(STORE, i, j, k);
                    for (int i = 1; i <= IMM1; ++i) A3(STORE, i, j, k) = SUM_STORE * F1(FP, i);
                }
            }
        }
        /* multigrid restriction 700 */
        bool mg = !(IR <= 1 && JR <= 1 && KR <= 1);
        if (mg) {
            for (int k = 1; k <= KMM1; ++k) {
                int k1 = F1(KB1, k), k2 = F1(KB2, k);
                for (int j = 2; j <= JM; ++j) {
                    int jsb = F1(JSBLK, j), j1 = F1(JB1, j), j2 = F1(JB2, j);
                    for (int i = 1; i <= IMM1; ++i) {
                        int i1 = F1(IB1, i), i2 = F1(IB2, i);
                        R DELTA = A3(STORE, i, j, k);
                        b1(i1, j1, k1) = b1(i1, j1, k1) + DELTA;
                        b2(i2, j2, k2) = b2(i2, j2, k2) + DELTA;
                        SBCHG[jsb - 1] = SBCHG[jsb - 1] + DELTA;
                    }
                }
            }
        }
        /* prolongation and time step 1500 */
        for (int k = 1; k <= KMM1; ++k) {
            int k1 = F1(KB1, k), k2 = F1(KB2, k);
            for (int j = 2; j <= JM; ++j) {
                int jsb = F1(JSBLK, j), j1 = F1(JB1, j), j2 = F1(JB2, j);
                for (int i = 1; i <= IMM1; ++i) {
                    int i1 = F1(IB1, i), i2 = F1(IB2, i);
                    R DELTA = A3(STORE, i, j, k) * F3(STEP, i, j, k) +
                              (b1(i1, j1, k1) * s1(i1, j1, k1) + b2(i2, j2, k2) * s2(i2, j2, k2) +
                               SBCHG[jsb - 1] * STEPSBK_v[jsb - 1]) * F3(RSTEP, i, j, k);
                    A3(STORE, i, j, k) = DELTA;
                }
            }
        }
        if (NRSMTH > 0) smooth_resid(STORE, RSMTH, NRSMTH);
        /* negative feedback 1501-1525 */
        if (!(DAMP < R(2.0) || DAMP > R(100))) {
            for (int nr = 1; nr <= NROWS; ++nr) {
                R SUMCHG = R(0.0);
                int JST = F1(JSTART, nr) + 1, JEN = F1(JMIX, nr) - 1;
                int JCHANGE = JEN - JST + 1;
                int NSUM = IMM1 * KMM1 * JCHANGE;
                for (int k = 1; k <= KMM1; ++k)
                    for (int j = JST; j <= JEN; ++j)
                        for (int i = 1; i <= IMM1; ++i) SUMCHG = SUMCHG + om::fabs(A3(STORE, i, j, k));
                AVG_CHG[nr - 1] = SUMCHG / R(NSUM);
            }
            if (NROWS == 1) AVG_BLK[0] = AVG_CHG[0];
            if (NROWS == 2) {
                AVG_BLK[1] = R(0.5) * (AVG_CHG[0] + AVG_CHG[1]);
                AVG_BLK[0] = AVG_BLK[1];
            }
            if (NROWS > 2) {
                for (int nr = 2; nr <= NROWS - 1; ++nr)
                    AVG_BLK[nr - 1] = R(0.25) * (AVG_CHG[nr - 2] + AVG_CHG[nr]) + R(0.5) * AVG_CHG[nr - 1];
                AVG_BLK[NROWS - 1] = R(0.5) * (AVG_CHG[NROWS - 2] + AVG_CHG[NROWS - 1]);
                AVG_BLK[0] = R(0.5) * (AVG_CHG[0] + AVG_CHG[1]);
            }
            for (int k = 1; k <= KMM1; ++k)
                for (int j = 2; j <= JM; ++j) {
                    int nr = F1(NROW, j);
                    for (int i = 1; i <= IMM1; ++i) {
                        R DELTA = A3(STORE, i, j, k);
                        R ABSCHG = om::fabs(DELTA);
                        R FDAMP = ABSCHG / AVG_BLK[nr - 1];
                        A3(STORE, i, j, k) = DELTA / (R(1.) + FDAMP / DAMP);
                    }
                }
        }
        if (NCALL == 2) {
            /* the cell-centred transported viscosity (5736-5777): the change
               is added to the cell, the row's last plane is carried across
               the mixing plane with the decay TURBVIS_DAMP, then one
               residual-smoothing pass */
            for (int k = 1; k <= KMM1; ++k)
                for (int j = 2; j <= JM; ++j)
                    for (int i = 1; i <= IMM1; ++i) A3(D, i, j, k) = A3(D, i, j, k) + A3(STORE, i, j, k);
            for (int nr = 1; nr <= NROWS - 1; ++nr) {
                int j = F1(JMIX, nr);
                R FMULT = F1(TURBVIS_DAMP, nr);
                for (int k = 1; k <= KMM1; ++k) {
                    R AVG = R(0.0);
                    for (int i = 1; i <= IMM1; ++i) AVG = AVG + F1(FP, i) * A3(D, i, j, k);
                    for (int jav = j + 1; jav <= j + 2; ++jav)
                        for (int i = 1; i <= IMM1; ++i) A3(D, i, jav, k) = FMULT * AVG;
                }
            }
            smooth_resid(D, FAC_SFVIS * SFT, 1);
        } else {
        /* second mixing-plane pitchwise average 1850 */
        for (int nr = 1; nr <= NRWSM1; ++nr) {
            int j = F1(JMIX, nr);
            for (int k = 1; k <= KMM1; ++k) {
                R FLOWDIRN = -A3(FLOWX, IMID, j, k);
                if (FLOWDIRN > R(0.0) || FEXTRAP < R(0.001)) {
                    int jmx = j + 2;
                    R SUM_STORE = R(0.0);
                    for (int i = 1; i <= IMM1; ++i) SUM_STORE = SUM_STORE + A3(STORE, i, jmx, k);
                    SUM_STORE = SUM_STORE / R(IMM1);
                    for (int i = 1; i <= IMM1; ++i) A3(STORE, i, jmx, k) = SUM_STORE;
                }
                if (FLOWDIRN < R(0.0) || FEXTRAP < R(0.001)) {
                    R SUM_STORE = R(0.0);
                    for (int i = 1; i <= IMM1; ++i) SUM_STORE = SUM_STORE + A3(STORE, i, j, k);
                    SUM_STORE = SUM_STORE / R(IMM1);
                    for (int i = 1; i <= IMM1; ++i) A3(STORE, i, j, k) = SUM_STORE;
                }
            }
        }
        /* scatter the cell change to its 8 corners 1100 */
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    R ADD = A3(STORE, i, j, k);
                    R fdn = F1(FACDWN, j), fup = F1(FACUP, j);
                    A3(D, i, j, k) = A3(D, i, j, k) + ADD * FIK(FBL, i, k) * fdn;
                    A3(D, i + 1, j, k) = A3(D, i + 1, j, k) + ADD * FIK(FBR, i, k) * fdn;
                    A3(D, i, j, k + 1) = A3(D, i, j, k + 1) + ADD * FIK(FTL, i, k) * fdn;
                    A3(D, i + 1, j, k + 1) = A3(D, i + 1, j, k + 1) + ADD * FIK(FTR, i, k) * fdn;
                    A3(D, i, j - 1, k) = A3(D, i, j - 1, k) + ADD * FIK(FBL, i, k) * fup;
                    A3(D, i + 1, j - 1, k) = A3(D, i + 1, j - 1, k) + ADD * FIK(FBR, i, k) * fup;
                    A3(D, i, j - 1, k + 1) = A3(D, i, j - 1, k + 1) + ADD * FIK(FTL, i, k) * fup;
                    A3(D, i + 1, j - 1, k + 1) = A3(D, i + 1, j - 1, k + 1) + ADD * FIK(FTR, i, k) * fup;
                }
        smooth_var(D);
        }
        /* periodic boundaries 8000 */
        int ILAST = NCALL == 2 ? IMM1 : IM;
        for (int j = 1; j <= JM; ++j) {
            if (F1(IND, j) == 1 || F1(INDLE, j) == 1) continue;
            for (int k = 1; k <= KM; ++k) {
                A3(D, 1, j, k) = R(0.5) * (A3(D, 1, j, k) + A3(D, ILAST, j, k));
                A3(D, ILAST, j, k) = A3(D, 1, j, k);
            }
        }
        /* tip-gap periodicity 510 */
        for (int j = 1; j <= JM; ++j) {
            int nr = F1(NROW, j);
            if (F1(KTIPS, nr) <= 0) continue;
            int K1 = F1(KTIPS, nr), K2 = F1(KTIPE, nr);
            if (K1 == 1) K2 = K2 - 1;
            if (K2 == KM) K1 = K1 + 1;
            for (int k = K1; k <= K2; ++k) {
                A3(D, 1, j, k) = R(0.5) * (A3(D, 1, j, k) + A3(D, ILAST, j, k));
                A3(D, ILAST, j, k) = A3(D, 1, j, k);
            }
        }
        /* mixing-plane pitchwise average of the variable 100 */
        if (IFMIX != 0) {
            for (int nr = 1; nr <= NRWSM1; ++nr) {
                int j = F1(JMIX, nr), jp1 = j + 1;
                for (int k = 1; k <= KM; ++k) {
                    R AVGVARJ = R(0.0), AVGVARJP1 = R(0.0);
                    for (int i = 1; i <= IMM1; ++i) {
                        AVGVARJ = AVGVARJ + F1(FP, i) * (A3(D, i, j, k) + A3(D, i + 1, j, k));
                        AVGVARJP1 = AVGVARJP1 + F1(FP, i) * (A3(D, i, jp1, k) + A3(D, i + 1, jp1, k));
                    }
                    AVGVARJ = R(0.5) * AVGVARJ;
                    AVGVARJP1 = R(0.5) * AVGVARJP1;
                    for (int i = 1; i <= IM; ++i) {
                        A3(D, i, j, k) = AVGVARJ;
                        A3(D, i, jp1, k) = AVGVARJP1;
                    }
                }
            }
        }
    }

    /* ================================================================== */
    /*  GRADVEL   multall-open-18.3.f:13468-13508: cell gradient of a node  */
    /*  quantity by Gauss' theorem (corner storage)                        */
    /* ================================================================== */
    void gradvel(int i, int j, int k, const std::vector<R> &V, R &DVDX, R &DVDR, R &DVDT) {
        int ip1 = i + 1, jm1 = j - 1, kp1 = k + 1;
        auto v = [&](int a, int b, int c) { return V[ijk(a, b, c)]; };
        R RVOL = R(0.25) / F3(VOL, i, j, k);
        R VAVGJ1 = v(i, jm1, k) + v(ip1, jm1, k) + v(ip1, jm1, kp1) + v(i, jm1, kp1);
        R VAVGJ2 = v(i, j, k) + v(ip1, j, k) + v(ip1, j, kp1) + v(i, j, kp1);
        R VAVGI1 = v(i, j, k) + v(i, jm1, k) + v(i, jm1, kp1) + v(i, j, kp1);
        R VAVGI2 = v(ip1, j, k) + v(ip1, jm1, k) + v(ip1, jm1, kp1) + v(ip1, j, kp1);
        R VAVGK1 = v(i, j, k) + v(ip1, j, k) + v(ip1, jm1, k) + v(i, jm1, k);
        R VAVGK2 = v(i, j, kp1) + v(ip1, j, kp1) + v(ip1, jm1, kp1) + v(i, jm1, kp1);
        R VAVGCELL = R(0.125) * (VAVGJ1 + VAVGJ2);
        DVDX = -((VAVGJ2 * F3(AQX, i, j, k) - VAVGJ1 * F3(AQX, i, jm1, k) + VAVGI1 * F3(ABX, i, j, k) -
                  VAVGI2 * F3(ABX, ip1, j, k) + VAVGK1 * F3(ASX, i, j, k) - VAVGK2 * F3(ASX, i, j, kp1)) *
                 RVOL);
        DVDR = -((VAVGJ2 * F3(AQR, i, j, k) - VAVGJ1 * F3(AQR, i, jm1, k) + VAVGI1 * F3(ABR, i, j, k) -
                  VAVGI2 * F3(ABR, ip1, j, k) + VAVGK1 * F3(ASR, i, j, k) - VAVGK2 * F3(ASR, i, j, kp1)) *
                 RVOL) -
               VAVGCELL / F2(RAVG_CELL, j, k);
        DVDT = -((VAVGI1 - VAVGI2) * F2(ABT, j, k) * RVOL);
    }

    /* ================================================================== */
    /*  SET_PWALLGRAD   multall-open-18.3.f:16052-16114: streamwise        */
    /*  pressure gradient per cell for the Shih wall functions, limited    */
    /*  and smoothed along J within each row.  The last row's smoothing    */
    /*  touches J = JM+1 .. JM+4, outside the grid: storage the reference  */
    /*  never writes otherwise (zero), so those reads give 0 here and the  */
    /*  writes are dropped.                                                 */
    /* ================================================================== */
    void set_pwallgrad() {
        R t = R(0.5) * (PDOWN_HUB + PDOWN_TIP);
        t = t / R(NROWS);
        t = t / (F1(CHORD, 1) + F1(CHORD, NROWS));
        R DPDS_LIM = om::fabs(R(20.0) * (F1(PO1, KMID) - t));
        for (int j = 2; j <= JM; ++j)
            for (int k = 1; k <= KMM1; ++k)
                for (int i = 1; i <= IMM1; ++i) {
                    R DPDX, DPDR, DPDT;
                    gradvel(i, j, k, PEFF_v, DPDX, DPDR, DPDT);
                    auto c8 = [&](const std::vector<R> &A) {
                        return A[ijk(i, j, k)] + A[ijk(i, j - 1, k)] + A[ijk(i + 1, j, k)] + A[ijk(i + 1, j - 1, k)] +
                               A[ijk(i, j, k + 1)] + A[ijk(i, j - 1, k + 1)] + A[ijk(i + 1, j, k + 1)] +
                               A[ijk(i + 1, j - 1, k + 1)];
                    };
                    R VXCELL = c8(VX_v), VRCELL = c8(VR_v), WTCELL = c8(WT_v);
                    R WREL_CELL = om::sqrt(VXCELL * VXCELL + VRCELL * VRCELL + WTCELL * WTCELL);
                    R DPDS = (DPDX * VXCELL + DPDR * VRCELL + DPDT * WTCELL) / WREL_CELL;
                    if (om::fabs(DPDS) > DPDS_LIM) DPDS = DPDS_LIM * DPDS / om::fabs(DPDS);
                    F3(DPDS_CELL, i, j, k) = DPDS;
                }
        std::vector<R> TEMPP((size_t)JM + 8);
        for (int nr = 1; nr <= NROWS; ++nr) {
            int J1 = F1(JSTART, nr), J2 = F1(JMIX, nr);
            for (int k = 1; k <= KMM1; ++k)
                for (int i = 1; i <= IMM1; ++i) {
                    auto D = [&](int jj) -> R { return jj <= JM ? F3(DPDS_CELL, i, jj, k) : R(0); };
                    auto setD = [&](int jj, R v) {
                        if (jj <= JM) F3(DPDS_CELL, i, jj, k) = v;
                    };
                    auto ends = [&]() {
                        setD(J2 + 1, R(0.0));
                        setD(J2 + 2, R(2) * D(J2 + 3) - D(J2 + 4));
                        setD(J2, R(2) * D(J2 - 1) - D(J2 - 2));
                    };
                    ends();
                    for (int jj = J1 + 2; jj <= J2 - 1; ++jj) TEMPP[jj] = R(0.5) * D(jj) + R(0.25) * (D(jj - 1) + D(jj + 1));
                    TEMPP[J2 + 1] = R(0.0);
                    for (int jj = J1 + 3; jj <= J2 - 2; ++jj)
                        setD(jj, R(0.5) * TEMPP[jj] + R(0.25) * (TEMPP[jj - 1] + TEMPP[jj + 1]));
                    ends();
                }
        }
    }

    /* ================================================================== */
    /*  WALLFUN   multall-open-18.3.f:15980-16047.  DPDS is the caller's    */
    /*  DPDS_CELL element: the pressure-gradient branch (YPLUSWALL <= -10)  */
    /*  raises |DPDS| < 1 to 1.0 in place, as the Fortran argument does.    */
    /* ================================================================== */
    void wallfun(R PERP, R &DPDS, R DENSITY, R &TWALL, R YPLUS_OLD, R WREL_WALL, R &YPLUS_NEW) {
        R SGN_DPDS = R(0), VPRES = R(0), VSTAR_P = R(0), FYPLUSP = R(0);
        const bool pres = !(YPLUSWALL > R(-10.0));
        if (pres) {
            if (om::fabs(DPDS) < R(1.0)) DPDS = R(1.0);
            SGN_DPDS = om::fabs(DPDS) / DPDS;
            VPRES = om::pow(VISLAM / DENSITY / DENSITY * om::fabs(DPDS), R(0.33333));
            VSTAR_P = YPLUS_OLD * VISLAM / (DENSITY * PERP);
            if (SGN_DPDS < R(0.0) && VPRES > R(0.33) * VSTAR_P) VPRES = R(0.33) * VSTAR_P;
            if (SGN_DPDS > R(0.0) && VPRES > R(2.0) * VSTAR_P) VPRES = R(2.0) * VSTAR_P;
            R YPLUS_PRES = VPRES * PERP * DENSITY / VISLAM;
            R P1 = YPLUS_PRES, P2 = P1 * P1, P3 = P2 * P1, P4 = P2 * P2;
            if (P1 <= R(4.0)) FYPLUSP = R(0.5) * P2 - R(7.31E-3) * P3;
            if (P1 > R(4.0) && P1 <= R(15.0))
                FYPLUSP = R(-15.138) + R(8.4688) * P1 - R(0.81976) * P2 + R(3.7292E-2) * P3 - R(6.3866E-4) * P4;
            if (P1 > R(15.0) && P1 <= R(30.0))
                FYPLUSP = R(11.925) + R(0.934) * P1 - R(2.7805E-2) * P2 + R(4.6262E-4) * P3 - R(3.1442E-6) * P4;
            if (P1 > R(30.0)) FYPLUSP = R(5) * om::log(P1) + R(8.0);
        }
        R YP1 = YPLUS_OLD, YP2 = YP1 * YP1, YP3 = YP2 * YP1, YP4 = YP2 * YP2;
        R FYPLUS = R(0);
        if (YP1 <= R(5.0)) FYPLUS = YP1 + R(1.0E-2) * YP2 - R(2.9E-03) * YP3;
        if (YP1 > R(5.0) && YP1 <= R(30.0))
            FYPLUS = R(-0.872) + R(1.465) * YP1 - R(7.02E-2) * YP2 + R(1.66E-03) * YP3 - R(1.495E-5) * YP4;
        if (YP1 > R(30) && YP1 <= R(140.0))
            FYPLUS = R(8.6) + R(0.1864) * YP1 - R(2.006E-3) * YP2 + R(1.144E-5) * YP3 - R(2.551E-8) * YP4;
        if (YP1 > R(140.0)) FYPLUS = R(2.439) * om::log(YP1) + R(5.0);
        R FRACP = pres ? SGN_DPDS * (VPRES / VSTAR_P) * FYPLUSP / FYPLUS : R(0.0);
        R VPLUS = FYPLUS * (R(1.0) + FRACP);
        R VSTAR = WREL_WALL / VPLUS;
        TWALL = DENSITY * VSTAR * VSTAR;
        YPLUS_NEW = DENSITY * VSTAR * PERP / VISLAM;
    }

    /* log-law skin friction with optional roughness, LOSS 8285-8331 etc.
     * re/relog/rough as in the reference; returns TWALL for the given
     * density and wall-relative speed used in the final expression. */
    R skin_friction(R RE, R PERP, R ROUGH_IN, R dens, R wb) {
        R RELOG = R(1.0) / om::log(RE);
        R ROUGH = ROUGH_IN;
        R CF;
        if (ROUGH > R(1.0E-7)) {
            if (ROUGH > PERP) ROUGH = PERP;
            R REK = RE * ROUGH / PERP;
            REK = REK - R(80.0);
            if (REK < R(0.0)) REK = R(0.0);
            R REKSQ = REK * REK;
            R A1 = R(-.00178493) + R(.0000814923) * REK + R(.000000150445) * REKSQ;
            R A2 = R(.029072) - R(.001584) * REK - R(.00000225194) * REKSQ;
            R A3c = R(.270313) + R(.0091409) * REK + R(.00000451537) * REKSQ + R(.00000000464767) * REKSQ * REK;
            CF = A1 + A2 * RELOG + A3c * RELOG * RELOG;
        } else {
            CF = R(-0.00178493) + R(0.029072) * RELOG + R(0.270313) * RELOG * RELOG;
        }
        R CFLAM = R(2.0) / RE;
        CF = std::max(CF, CFLAM);
        if (RE < R(125.)) CF = CFLAM;
        if (ROUGH > R(1.0E-7)) {
            R TW = R(0.5) * CF * dens * wb * wb;
            R VSTAR = om::sqrt(TW / dens);
            R PLUSK = ROUGH * VSTAR * dens / VISLAM;
            R RELOG10 = om::log10(PERP / ROUGH);
            R FUNCN = R(5.75) * RELOG10 + R(8.5);
            R CF_FULL_ROUGH = R(2.0) / (FUNCN * FUNCN);
            if (PLUSK > R(45) && CF > CF_FULL_ROUGH) CF = CF_FULL_ROUGH;
        }
        return R(0.5) * CF * dens * wb * wb;
    }

    static inline R fyplus_of(R yp, R yplam, R ypturb, R prev) {
        R f = prev;
        if (yp <= yplam) f = R(0.0);
        if (yp > yplam) {
            R XFAC = (yp - yplam) / (ypturb - yplam);
            if (XFAC > R(1.0)) XFAC = R(1.0);
            f = XFAC * XFAC * (R(3.0) - R(2.0) * XFAC);
        }
        return f;
    }

    /* ================================================================== */
    /*  LOSS  (ILOS=10)   multall-open-18.3.f:8058-9066                    */
    /* ================================================================== */
    void loss() {
        if (NSTEP == 1 || NSTEP < NSTEPS_MAX / 4) {
            if (REYNO > R(100.)) {
                int J1 = F1(JLE, 1), J2 = F1(JTE, 1);
                if (F1(JLE, 1) > JM) J1 = 1;
                if (F1(JTE, 1) > JM) J2 = JM;
                R XCHORD = F2(SMERID, J2, KMID) - F2(SMERID, J1, KMID);
                R a = F3(ROVX, IMID, J2, KMID), b = F3(ROVR, IMID, J2, KMID), c = F3(ROWT, IMID, J2, KMID);
                R ROW2 = om::sqrt(a * a + b * b + c * c);
                VISLAM = XCHORD * ROW2 / REYNO;
            }
            if (REYNO > R(0.0) && REYNO < R(99.99)) VISLAM = REYNO / R(100000.);
            if (REYNO < R(0.0)) VISLAM = -REYNO * R(1.0E-5);
            TCOND = CP * VISLAM / PRANDTL;
            FTCOND = TCOND / VISLAM;
        }
        if (NSTEP <= NLOS) loss_tables();
        if (YPLUSWALL < R(-10.0)) set_pwallgrad();

        int LEN = std::max(IM, KM) + 2;
        std::vector<R> VXAVG(LEN), VRAVG(LEN), WTAVG(LEN), WABS(LEN), ROAVG(LEN), XSTRES(LEN), RAVG(LEN),
            RSTRES(LEN), TSTRES(LEN), AREA(LEN), WBOUND(LEN), WTB(LEN), VTAVG(LEN), TAVG(LEN), WVISC(LEN),
            QFLOW(LEN), VLAM(LEN), VTURB(LEN);
        R FYPLUS = R(0);
        R RF_VIS1 = R(1.) - RF_VIS;
        /* ---- stresses on the streamwise (K = const) faces, DO 50 ---- */
        for (int j = 2; j <= JM; ++j) {
            int NRW = F1(NROW, j);
            int J1 = F1(JSTART, NRW);
            int JROW = j - J1 + 1;
            int JTRHUB = F1(JTRAN_K1, NRW), JTRTIP = F1(JTRAN_KM, NRW);
            R WREL = F1(WRAD, j);
            for (int i = 1; i <= IMM1; ++i) {
                for (int k = 1; k <= KM; ++k) {
                    R asx = F3(ASX, i, j, k), asr = F3(ASR, i, j, k);
                    AREA[k] = om::sqrt(asx * asx + asr * asr);
                    VXAVG[k] = R(0.25) * (F3(VX, i, j, k) + F3(VX, i, j - 1, k) + F3(VX, i + 1, j, k) + F3(VX, i + 1, j - 1, k));
                    VRAVG[k] = R(0.25) * (F3(VR, i, j, k) + F3(VR, i, j - 1, k) + F3(VR, i + 1, j, k) + F3(VR, i + 1, j - 1, k));
                    VTAVG[k] = R(0.25) * (F3(VT, i, j, k) + F3(VT, i, j - 1, k) + F3(VT, i + 1, j, k) + F3(VT, i + 1, j - 1, k));
                    ROAVG[k] = R(0.25) * (F3(RO, i, j, k) + F3(RO, i, j - 1, k) + F3(RO, i + 1, j, k) + F3(RO, i + 1, j - 1, k));
                    TAVG[k] = R(0.25) * (F3(T_STATIC, i, j, k) + F3(T_STATIC, i, j - 1, k) + F3(T_STATIC, i + 1, j, k) +
                                         F3(T_STATIC, i + 1, j - 1, k));
                    RAVG[k] = R(0.5) * (F2(R, j, k) + F2(R, j - 1, k));
                    WTAVG[k] = VTAVG[k] - WREL * RAVG[k];
                    R WABSQ = VXAVG[k] * VXAVG[k] + VRAVG[k] * VRAVG[k] + WTAVG[k] * WTAVG[k];
                    WABS[k] = om::sqrt(WABSQ);
                    WTB[k] = VTAVG[k] - F1(WHUB, j) * RAVG[k];
                    if (k > KMID) WTB[k] = VTAVG[k] - F1(WTIP, j) * RAVG[k];
                    WBOUND[k] = om::sqrt(VXAVG[k] * VXAVG[k] + VRAVG[k] * VRAVG[k] + WTB[k] * WTB[k]);
                }
                if (REYNO < R(0.0001)) {
                    VISLAM = (om::fabs(REYNO) / R(100000.0)) * om::pow(TAVG[KMID] / R(288.0), R(0.62));
                    TCOND = CP * VISLAM / PRANDTL;
                    FTCOND = TCOND / VISLAM;
                }
                R TWALLK1, TWALLKM;
                if (YPLUSWALL < R(-0.001)) {
                    R PERPK1 = F3(VOL, i, j, 1) / AREA[1];
                    R YPLUS_NEW;
                    wallfun(PERPK1, F3(DPDS_CELL, i, j, 1), ROAVG[1], TWALLK1, FIJ(YPLUS_K1, i, j), WBOUND[1], YPLUS_NEW);
                    FIJ(YPLUS_K1, i, j) = std::min(R(1000.0), YPLUS_NEW);
                } else if (YPLUSWALL < R(5.)) {
                    R PERP = F3(VOL, i, j, 1) / AREA[1];
                    R RE = PERP * ROAVG[2] * WBOUND[2] / VISLAM;
                    TWALLK1 = skin_friction(RE, PERP, F1(ROUGH_H, NRW), ROAVG[2], WBOUND[2]);
                } else {
                    TWALLK1 = CFWALL * ROAVG[1] * WBOUND[1] * WBOUND[1];
                }
                if (YPLUSWALL < R(-0.001)) {
                    R PERPKM = F3(VOL, i, j, KMM1) / AREA[KM];
                    R YPLUS_NEW;
                    wallfun(PERPKM, F3(DPDS_CELL, i, j, KMM1), ROAVG[KMM1], TWALLKM, FIJ(YPLUS_KM, i, j), WBOUND[KMM1], YPLUS_NEW);
                    FIJ(YPLUS_KM, i, j) = std::min(R(1000.0), YPLUS_NEW);
                } else if (YPLUSWALL < R(5.)) {
                    R PERP = F3(VOL, i, j, KMM1) / AREA[KM];
                    R RE = PERP * ROAVG[KMM1] * WBOUND[KMM1] / VISLAM;
                    TWALLKM = skin_friction(RE, PERP, F1(ROUGH_T, NRW), ROAVG[KMM1], WBOUND[KMM1]);
                } else {
                    TWALLKM = CFWALL * ROAVG[KM] * WBOUND[KM] * WBOUND[KM];
                }
                R VSTAR = om::sqrt(TWALLK1 / ROAVG[1]);
                for (int k = 1; k <= KMID; ++k) {
                    R PERP = om::sqrt(F3(DWALLSQ, i, j, k));
                    R YPLSK1 = VSTAR * PERP * ROAVG[1] / VISLAM;
                    F3(Y_PLUS, i, j, k) = std::min(YPLSK1, R(1000.0));
                }
                VSTAR = om::sqrt(TWALLKM / ROAVG[KM]);
                for (int k = KMID + 1; k <= KMM1; ++k) {
                    R PERP = om::sqrt(F3(DWALLSQ, i, j, k));
                    R YPLS = VSTAR * PERP * ROAVG[KM] / VISLAM;
                    F3(Y_PLUS, i, j, k) = std::min(YPLS, R(1000.0));
                }
                R FMULT = TWALLK1 * AREA[1] / WBOUND[1];
                if (IBOUND == 1 || IBOUND > 2) FMULT = R(0.0);
                XSTRES[1] = FMULT * VXAVG[1];
                RSTRES[1] = FMULT * VRAVG[1];
                TSTRES[1] = FMULT * WTB[1];
                FMULT = -TWALLKM * AREA[KM] / WBOUND[KM];
                if (IBOUND >= 2) FMULT = R(0.0);
                XSTRES[KM] = FMULT * VXAVG[KM];
                RSTRES[KM] = FMULT * VRAVG[KM];
                TSTRES[KM] = FMULT * WTB[KM];
                WVISC[1] = TSTRES[1] * F1(WHUB, j) * RAVG[1];
                QFLOW[1] = R(0.0);
                WVISC[KM] = TSTRES[KM] * F1(WTIP, j) * RAVG[KM];
                QFLOW[KM] = R(0.0);
                for (int k = 2; k <= KMM1; ++k) {
                    FYPLUS = fyplus_of(F3(Y_PLUS, i, j, k), YPLAM, YPTURB, FYPLUS);
                    R DPERP = F3(VOL, i, j, k) / AREA[k];
                    VLAM[k] = ROWT2(FKLAM, NRW, k, KM) * VISLAM / DPERP;
                    VTURB[k] = ROWT2(FKTURB, NRW, k, KM) * ROAVG[k] * om::fabs(WABS[k + 1] - WABS[k - 1]) * FMIXUP;
                    VTURB[k] = VTURB[k] * FYPLUS;
                }
                bool turb = false;
                if (!(JROW < JTRHUB)) {
                    R RMAX = R(0.0);
                    for (int k = 2; k <= KMID; ++k) {
                        R RATVIS = VTURB[k] / VLAM[k];
                        if (RATVIS < RMAX) continue;
                        RMAX = RATVIS;
                    }
                    turb = RMAX > FTRANS;
                }
                if (!turb)
                    for (int k = 2; k <= KMID; ++k) VTURB[k] = R(0.0);
                turb = false;
                if (!(JROW < JTRTIP)) {
                    R RMAX = R(0.0);
                    for (int k = KMID; k <= KMM1; ++k) {
                        R RATVIS = VTURB[k] / VLAM[k];
                        if (RATVIS < RMAX) continue;
                        RMAX = RATVIS;
                    }
                    turb = RMAX > FTRANS;
                }
                if (!turb)
                    for (int k = KMID; k <= KMM1; ++k) VTURB[k] = R(0.0);
                for (int k = 2; k <= KMM1; ++k) {
                    R FM = AREA[k] * (VLAM[k] + VTURB[k]);
                    XSTRES[k] = FM * (VXAVG[k + 1] - VXAVG[k - 1]);
                    RSTRES[k] = FM * (VRAVG[k + 1] - VRAVG[k - 1]);
                    R VISTOT = VISLAM * (R(1.0) + VTURB[k] / VLAM[k]);
                    TSTRES[k] = FM * (VTAVG[k + 1] - VTAVG[k - 1]) - VISTOT * AREA[k] * VTAVG[k] / RAVG[k];
                    QFLOW[k] = FM * FTCOND * (TAVG[k + 1] - TAVG[k - 1]);
                    WVISC[k] = XSTRES[k] * VXAVG[k] + TSTRES[k] * VTAVG[k] + RSTRES[k] * VRAVG[k];
                }
                for (int k = 1; k <= KMM1; ++k) {
                    F3(XFORCE, i, j, k) = RF_VIS1 * F3(XFORCE, i, j, k) + RF_VIS * (XSTRES[k] - XSTRES[k + 1]);
                    F3(RFORCE, i, j, k) = RF_VIS1 * F3(RFORCE, i, j, k) + RF_VIS * (RSTRES[k] - RSTRES[k + 1]);
                    F3(TFORCE, i, j, k) = RF_VIS1 * F3(TFORCE, i, j, k) +
                                          RF_VIS * (TSTRES[k] * RAVG[k] - TSTRES[k + 1] * RAVG[k + 1]);
                    F3(QSOURCE, i, j, k) = RF_VIS1 * F3(QSOURCE, i, j, k) +
                                           RF_VIS * (QFLOW[k] - QFLOW[k + 1] + WVISC[k] - WVISC[k + 1]);
                }
            }
        }
        /* ---- stresses on the bladewise (I = const) faces, DO 100 ---- */
        for (int j = 2; j <= JM; ++j) {
            int NRW = F1(NROW, j);
            int J1 = F1(JSTART, NRW);
            int JROW = j - J1 + 1;
            int JTRLOW = F1(JTRAN_I1, NRW), JTRUP = F1(JTRAN_IM, NRW);
            int JLEDGE = F1(JLE, NRW), JTEDGE = F1(JTE, NRW);
            R WREL = F1(WRAD, j);
            for (int k = 1; k <= KMM1; ++k) {
                RAVG[k] = F2(RAVG_CELL, j, k);
                for (int i = 1; i <= IM; ++i) {
                    R abx = F3(ABX, i, j, k), abr = F3(ABR, i, j, k), abt = F2(ABT, j, k);
                    AREA[i] = om::sqrt(abx * abx + abr * abr + abt * abt);
                    VXAVG[i] = R(0.25) * (F3(VX, i, j, k) + F3(VX, i, j - 1, k) + F3(VX, i, j - 1, k + 1) + F3(VX, i, j, k + 1));
                    VRAVG[i] = R(0.25) * (F3(VR, i, j, k) + F3(VR, i, j - 1, k) + F3(VR, i, j - 1, k + 1) + F3(VR, i, j, k + 1));
                    VTAVG[i] = R(0.25) * (F3(VT, i, j, k) + F3(VT, i, j - 1, k) + F3(VT, i, j - 1, k + 1) + F3(VT, i, j, k + 1));
                    WTAVG[i] = R(0.25) * (F3(WT, i, j, k) + F3(WT, i, j - 1, k) + F3(WT, i, j - 1, k + 1) + F3(WT, i, j, k + 1));
                    ROAVG[i] = R(0.25) * (F3(RO, i, j, k) + F3(RO, i, j - 1, k) + F3(RO, i, j - 1, k + 1) + F3(RO, i, j, k + 1));
                    TAVG[i] = R(0.25) * (F3(T_STATIC, i, j, k) + F3(T_STATIC, i, j - 1, k) + F3(T_STATIC, i, j - 1, k + 1) +
                                         F3(T_STATIC, i, j, k + 1));
                    R WABSQ = VXAVG[i] * VXAVG[i] + VRAVG[i] * VRAVG[i] + WTAVG[i] * WTAVG[i];
                    WABS[i] = om::sqrt(WABSQ);
                    WBOUND[i] = WABS[i];
                }
                if (REYNO < R(0.0001)) {
                    VISLAM = (om::fabs(REYNO) / R(100000.0)) * om::pow(TAVG[IMID] / R(288.0), R(0.62));
                    TCOND = CP * VISLAM / PRANDTL;
                    FTCOND = TCOND / VISLAM;
                }
                bool in_blade = !(j <= JLEDGE || j > JTEDGE);
                bool in_gap = (F1(KTIPS, NRW) > 0) && (k >= F1(KTIPS, NRW)) && (k < F1(KTIPE, NRW));
                if (in_blade) {
                    if (!in_gap) {
                        R TWALLI1, TWALLIM;
                        if (YPLUSWALL < R(-0.001)) {
                            R PERPI1 = F3(VOL, 1, j, k) / AREA[1];
                            R YPLUS_NEW;
                            wallfun(PERPI1, F3(DPDS_CELL, 1, j, k), ROAVG[1], TWALLI1, F2(YPLUS_I1, j, k), WBOUND[2], YPLUS_NEW);
                            F2(YPLUS_I1, j, k) = std::min(R(1000.0), YPLUS_NEW);
                        } else if (YPLUSWALL < R(5.)) {
                            R PERP = F3(VOL, 1, j, k) / AREA[1];
                            R RE = ROAVG[2] * WABS[2] * PERP / VISLAM;
                            TWALLI1 = skin_friction(RE, PERP, F1(ROUGH_L, NRW), ROAVG[2], WBOUND[2]);
                        } else {
                            TWALLI1 = CFWALL * ROAVG[1] * WABS[1] * WABS[1];
                        }
                        if (YPLUSWALL < R(-0.001)) {
                            R PERPIM = F3(VOL, IMM1, j, k) / AREA[IM];
                            R YPLUS_NEW;
                            wallfun(PERPIM, F3(DPDS_CELL, IMM1, j, k), ROAVG[IMM1], TWALLIM, F2(YPLUS_IM, j, k), WBOUND[IMM1], YPLUS_NEW);
                            F2(YPLUS_IM, j, k) = std::min(R(1000.0), YPLUS_NEW);
                        } else if (YPLUSWALL < R(5.)) {
                            R PERP = F3(VOL, IMM1, j, k) / AREA[IM];
                            R RE = ROAVG[IMM1] * WABS[IMM1] * PERP / VISLAM;
                            TWALLIM = skin_friction(RE, PERP, F1(ROUGH_U, NRW), ROAVG[IMM1], WBOUND[IMM1]);
                        } else {
                            TWALLIM = CFWALL * ROAVG[IM] * WABS[IM] * WABS[IM];
                        }
                        R VSTAR = om::sqrt(TWALLI1 / ROAVG[1]);
                        for (int i = 1; i <= IMID; ++i) {
                            R YPLS = VSTAR * om::sqrt(F3(DWALLSQ, i, j, k)) * ROAVG[1] / VISLAM;
                            R YPLSP = F3(Y_PLUS, i, j, k);
                            F3(Y_PLUS, i, j, k) = std::min(YPLS, YPLSP);
                        }
                        VSTAR = om::sqrt(TWALLIM / ROAVG[IM]);
                        for (int i = IMID + 1; i <= IMM1; ++i) {
                            R YPLS = VSTAR * om::sqrt(F3(DWALLSQ, i, j, k)) * ROAVG[IM] / VISLAM;
                            R YPLSP = F3(Y_PLUS, i, j, k);
                            F3(Y_PLUS, i, j, k) = std::min(YPLS, YPLSP);
                        }
                        R FMULT = TWALLI1 * AREA[1] / WABS[1];
                        XSTRES[1] = FMULT * VXAVG[1];
                        RSTRES[1] = FMULT * VRAVG[1];
                        TSTRES[1] = FMULT * WTAVG[1];
                        FMULT = -TWALLIM * AREA[IM] / WABS[IM];
                        XSTRES[IM] = FMULT * VXAVG[IM];
                        RSTRES[IM] = FMULT * VRAVG[IM];
                        TSTRES[IM] = FMULT * WTAVG[IM];
                        QFLOW[1] = R(0.0);
                        WVISC[1] = TSTRES[1] * WREL * RAVG[k];
                        QFLOW[IM] = R(0.0);
                        WVISC[IM] = TSTRES[IM] * WREL * RAVG[k];
                    }
                    for (int i = 2; i <= IMM1; ++i) {
                        FYPLUS = fyplus_of(F3(Y_PLUS, i, j, k), YPLAM, YPTURB, FYPLUS);
                        R DPERP = F3(VOL, i, j, k) / AREA[i];
                        VLAM[i] = ROWT2(FILAM, NRW, i, IM) * VISLAM / DPERP;
                        VTURB[i] = ROWT2(FITURB, NRW, i, IM) * ROAVG[i] * om::fabs(WABS[i + 1] - WABS[i - 1]) * FMIXUP;
                        VTURB[i] = VTURB[i] * FYPLUS;
                    }
                    bool turb = false;
                    if (!(JROW < JTRLOW)) {
                        R RMAX = R(0.0);
                        for (int i = 2; i <= IMID; ++i) {
                            R RATVIS = VTURB[i] / VLAM[i];
                            if (RATVIS < RMAX) continue;
                            RMAX = RATVIS;
                        }
                        turb = RMAX > FTRANS;
                    }
                    if (!turb)
                        for (int i = 2; i <= IMID; ++i) VTURB[i] = R(0.0);
                    turb = false;
                    if (!(JROW < JTRUP)) {
                        R RMAX = R(0.0);
                        for (int i = IMID; i <= IMM1; ++i) {
                            R RATVIS = VTURB[i] / VLAM[i];
                            if (RATVIS < RMAX) continue;
                            RMAX = RATVIS;
                        }
                        turb = RMAX > FTRANS;
                    }
                    if (!turb)
                        for (int i = IMID; i <= IMM1; ++i) VTURB[i] = R(0.0);
                    for (int i = 2; i <= IMM1; ++i) {
                        R FM = (VLAM[i] + VTURB[i]) * AREA[i];
                        XSTRES[i] = FM * (VXAVG[i + 1] - VXAVG[i - 1]);
                        RSTRES[i] = FM * (VRAVG[i + 1] - VRAVG[i - 1]);
                        TSTRES[i] = FM * (WTAVG[i + 1] - WTAVG[i - 1]);
                        F3(VISC_RAT, i, j, k) = VTURB[i] / VLAM[i];
                        QFLOW[i] = FM * FTCOND * (TAVG[i + 1] - TAVG[i - 1]);
                        WVISC[i] = XSTRES[i] * VXAVG[i] + RSTRES[i] * VRAVG[i] + TSTRES[i] * VTAVG[i];
                    }
                    if (in_gap) {
                        XSTRES[1] = R(0.5) * (XSTRES[2] + XSTRES[IMM1]);
                        RSTRES[1] = R(0.5) * (RSTRES[2] + RSTRES[IMM1]);
                        TSTRES[1] = R(0.5) * (TSTRES[2] + TSTRES[IMM1]);
                        XSTRES[IM] = XSTRES[1];
                        TSTRES[IM] = TSTRES[1];
                        RSTRES[IM] = RSTRES[1];
                        QFLOW[1] = R(0.5) * (QFLOW[2] + QFLOW[IMM1]);
                        WVISC[1] = R(0.5) * (WVISC[2] + WVISC[IMM1]);
                        QFLOW[IM] = QFLOW[1];
                        WVISC[IM] = WVISC[1];
                    }
                } else {
                    if (j > JTEDGE) {
                        R FACJ = R(0.1) * R(j - JTEDGE);
                        if (FACJ > R(1.)) FACJ = R(1.);
                        for (int i = 1; i <= IM; ++i) {
                            int ISUB = (i == IM) ? IMM1 : i;
                            int IM1 = (i == 1) ? IMM1 : i - 1;
                            int IP1 = (i == IM) ? 2 : i + 1;
                            R FBLEND = (FACJ * ROWT2(FIWAKE, NRW, i, IM) + (R(1.) - FACJ) * ROWT2(FITURB, NRW, i, IM)) * FMIXUP;
                            R DPERP = F3(VOL, ISUB, j, k) / AREA[i];
                            VLAM[i] = ROWT2(FILAM, NRW, i, IM) * VISLAM / DPERP;
                            VTURB[i] = FBLEND * ROAVG[i] * om::fabs(WABS[IP1] - WABS[IM1]);
                            F3(VISC_RAT, i, j, k) = VTURB[i] / VLAM[i];
                            R FM = AREA[i] * (VLAM[i] + VTURB[i]);
                            XSTRES[i] = FM * (VXAVG[IP1] - VXAVG[IM1]);
                            RSTRES[i] = FM * (VRAVG[IP1] - VRAVG[IM1]);
                            TSTRES[i] = FM * (WTAVG[IP1] - WTAVG[IM1]);
                            QFLOW[i] = FM * FTCOND * (TAVG[IP1] - TAVG[IM1]);
                            WVISC[i] = XSTRES[i] * VXAVG[i] + TSTRES[i] * VTAVG[i] + RSTRES[i] * VRAVG[i];
                        }
                    }
                    if (j <= JLEDGE) {
                        for (int i = 1; i <= IM; ++i) {
                            int ISUB = (i == IM) ? IMM1 : i;
                            int IM1 = (i == 1) ? IMM1 : i - 1;
                            int IP1 = (i == IM) ? 2 : i + 1;
                            R DPERP = F3(VOL, ISUB, j, k) / AREA[i];
                            VLAM[i] = ROWT2(FILAM, NRW, i, IM) * VISLAM / DPERP;
                            VTURB[i] = FMIXUP * ROWT2(FIUP, NRW, i, IM) * ROAVG[i] * om::fabs(WABS[IP1] - WABS[IM1]);
                            F3(VISC_RAT, i, j, k) = VTURB[i] / VLAM[i];
                            R FM = AREA[i] * (VLAM[i] + VTURB[i]);
                            XSTRES[i] = FM * (VXAVG[IP1] - VXAVG[IM1]);
                            RSTRES[i] = FM * (VRAVG[IP1] - VRAVG[IM1]);
                            TSTRES[i] = FM * (WTAVG[IP1] - WTAVG[IM1]);
                            QFLOW[i] = FM * FTCOND * (TAVG[IP1] - TAVG[IM1]);
                            WVISC[i] = XSTRES[i] * VXAVG[i] + TSTRES[i] * VTAVG[i] + RSTRES[i] * VRAVG[i];
                        }
                    }
                    XSTRES[1] = R(0.5) * (XSTRES[IM] + XSTRES[1]);
                    RSTRES[1] = R(0.5) * (RSTRES[IM] + RSTRES[1]);
                    TSTRES[1] = R(0.5) * (TSTRES[IM] + TSTRES[1]);
                    XSTRES[IM] = XSTRES[1];
                    RSTRES[IM] = RSTRES[1];
                    TSTRES[IM] = TSTRES[1];
                    QFLOW[1] = R(0.5) * (QFLOW[IM] + QFLOW[1]);
                    WVISC[1] = R(0.5) * (WVISC[IM] + WVISC[1]);
                    QFLOW[IM] = QFLOW[1];
                    WVISC[IM] = WVISC[1];
                }
                for (int i = 1; i <= IMM1; ++i) {
                    F3(XFORCE, i, j, k) = F3(XFORCE, i, j, k) + RF_VIS * (XSTRES[i] - XSTRES[i + 1]);
                    F3(RFORCE, i, j, k) = F3(RFORCE, i, j, k) + RF_VIS * (RSTRES[i] - RSTRES[i + 1]);
                    F3(TFORCE, i, j, k) = F3(TFORCE, i, j, k) + RF_VIS * (TSTRES[i] - TSTRES[i + 1]) * RAVG[k];
                    F3(QSOURCE, i, j, k) = F3(QSOURCE, i, j, k) + RF_VIS * (QFLOW[i] - QFLOW[i + 1] + WVISC[i] - WVISC[i + 1]);
                }
            }
        }
    }

    /* the tables LOSS builds on its first call, 8123-8189 */
    void loss_tables() {
        for (int nrw = 1; nrw <= NROWS; ++nrw) {
            R SUMF = R(0.0);
            for (int i = 2; i <= IMM1; ++i) {
                SUMF = SUMF + F1(FP, i - 1);
                R XLIM = F1(XLLIM_I1, nrw) * (R(1.0) - SUMF) + F1(XLLIM_IM, nrw) * SUMF;
                R FPITCH = SUMF * (R(1.) - SUMF);
                if (FPITCH > XLIM) FPITCH = XLIM;
                R DF = F1(FP, i) + F1(FP, i - 1);
                ROWT2(FILAM, nrw, i, IM) = F1(FP, i) / DF;
                ROWT2(FITURB, nrw, i, IM) = R(0.16) * FPITCH * FPITCH / (DF * DF);
                ROWT2(FIWAKE, nrw, i, IM) = R(0.16) * F1(XLLIM_DWN, nrw) * F1(XLLIM_DWN, nrw) / (DF * DF);
                ROWT2(FIUP, nrw, i, IM) = R(0.16) * F1(XLLIM_UP, nrw) * F1(XLLIM_UP, nrw) / (DF * DF);
            }
            R DF = F1(FP, 1) + F1(FP, IMM1);
            ROWT2(FILAM, nrw, 1, IM) = F1(FP, 1) / DF;
            ROWT2(FIWAKE, nrw, 1, IM) = R(0.16) * F1(XLLIM_DWN, nrw) * F1(XLLIM_DWN, nrw) / (DF * DF);
            ROWT2(FIUP, nrw, 1, IM) = R(0.16) * F1(XLLIM_UP, nrw) * F1(XLLIM_UP, nrw) / (DF * DF);
            ROWT2(FITURB, nrw, 1, IM) = ROWT2(FITURB, nrw, 2, IM);
            ROWT2(FILAM, nrw, IM, IM) = F1(FP, IMM1) / DF;
            ROWT2(FIWAKE, nrw, IM, IM) = R(0.16) * F1(XLLIM_DWN, nrw) * F1(XLLIM_DWN, nrw) / (DF * DF);
            ROWT2(FIUP, nrw, IM, IM) = R(0.16) * F1(XLLIM_UP, nrw) * F1(XLLIM_UP, nrw) / (DF * DF);
            ROWT2(FITURB, nrw, IM, IM) = ROWT2(FITURB, nrw, IMM1, IM);

            R AVGSPAN = R(0.0);
            int JMID = (int)(R(0.5) * R(F1(JLE, nrw) + F1(JTE, nrw)));
            for (int k = 2; k <= KM; ++k) {
                R XDIF = F2(X, JMID, k) - F2(X, JMID, k - 1);
                R RDIF = F2(R, JMID, k) - F2(R, JMID, k - 1);
                AVGSPAN = AVGSPAN + om::sqrt(XDIF * XDIF + RDIF * RDIF);
            }
            R AVGPIT = R(2) * R(3.1415926) * F2(R, JMID, KMID) / R(F1(NBLADE, JMID));
            R XLIMH = F1(XLLIM_K1, nrw) * AVGPIT / AVGSPAN;
            R XLIMT = F1(XLLIM_KM, nrw) * AVGPIT / AVGSPAN;
            SUMF = R(0.0);
            for (int k = 2; k <= KMM1; ++k) {
                SUMF = SUMF + F1(FR, k - 1);
                R XLIM = XLIMH * (R(1.0) - SUMF) + XLIMT * SUMF;
                R FCSPAN = SUMF * (R(1.) - SUMF);
                if (FCSPAN > XLIM) FCSPAN = XLIM;
                R DFk = F1(FR, k) + F1(FR, k - 1);
                ROWT2(FKLAM, nrw, k, KM) = F1(FR, k) / DFk;
                ROWT2(FKTURB, nrw, k, KM) = R(0.16) * FCSPAN * FCSPAN / (DFk * DFk);
            }
        }
    }


    /* ================================================================== */
    /*  NEW_LOSS (ILOS 100-199)  multall-open-18.3.f:12522-13462, with      */
    /*  GRADVEL 13468-13508 and the cell-average density 4255-4267          */
    /* ================================================================== */
    void roavg_cell() {
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i)
                    F3(ROAVG_CELL, i, j, k) =
                        R(0.125) * (F3(RO, i, j, k) + F3(RO, i + 1, j, k) + F3(RO, i + 1, j, k + 1) + F3(RO, i, j, k + 1) +
                                    F3(RO, i, j - 1, k) + F3(RO, i + 1, j - 1, k) + F3(RO, i + 1, j - 1, k + 1) +
                                    F3(RO, i, j - 1, k + 1));
    }

    // NEW_LOSS's log-law skin friction on the sums of four corner values
    // (12879-12925 and its three copies)
    R nl_twall(R RE, R DPERP, R ROUGH, R RO4, R W4) {
        R RELOG = R(1.) / om::log(RE);
        R CF;
        if (ROUGH > R(1.0E-7)) {
            if (ROUGH > DPERP) ROUGH = DPERP;
            R REK = RE * ROUGH / DPERP;
            REK = REK - R(80.0);
            if (REK < R(0.0)) REK = R(0.0);
            R REKSQ = REK * REK;
            R A1 = R(-.00178493) + R(.0000814923) * REK + R(.000000150445) * REKSQ;
            R A2 = R(.029072) - R(.001584) * REK - R(.00000225194) * REKSQ;
            R A3c = R(.270313) + R(.0091409) * REK + R(.00000451537) * REKSQ + R(.00000000464767) * REKSQ * REK;
            CF = A1 + A2 * RELOG + A3c * RELOG * RELOG;
        } else {
            CF = R(-0.00178493) + R(0.029072) * RELOG + R(0.270313) * RELOG * RELOG;
        }
        R CFLAM = R(2.0) / RE;
        CF = std::max(CF, CFLAM);
        if (RE < R(125.)) CF = CFLAM;
        if (ROUGH > R(1.0E-7)) {
            R TW = CF * RO4 * W4 * W4 / R(128);
            R VSTAR = om::sqrt(TW / (RO4 / R(4)));
            R PLUSK = ROUGH * VSTAR * RO4 / VISLAM / R(4);
            R RELOG10 = om::log10(DPERP / ROUGH);
            R FUNCN = R(5.75) * RELOG10 + R(8.5);
            R CF_FULL_ROUGH = R(2.0) / (FUNCN * FUNCN);
            if (PLUSK > R(45) && CF > CF_FULL_ROUGH) CF = CF_FULL_ROUGH;
        }
        return CF * RO4 * W4 * W4 / R(128);
    }

    void new_loss() {
        if (NSTEP == 1 || NSTEP < NSTEPS_MAX / 4) {
            if (REYNO > R(100.)) {
                int J1 = F1(JLE, 1), J2 = F1(JTE, 1);
                if (F1(JLE, 1) > JM) J1 = 1;
                if (F1(JTE, 1) > JM) J2 = JM;
                R XCHORD = F2(SMERID, J2, KMID) - F2(SMERID, J1, KMID);
                R a = F3(ROVX, IMID, J2, KMID), b = F3(ROVR, IMID, J2, KMID), c = F3(ROWT, IMID, J2, KMID);
                VISLAM = XCHORD * om::sqrt(a * a + b * b + c * c) / REYNO;
            }
            if (REYNO > R(0.0) && REYNO < R(99.99)) VISLAM = REYNO / R(100000.);
            if (REYNO < R(0.0)) VISLAM = -REYNO * R(1.0E-5);
            TCOND = CP * VISLAM / PRANDTL;
            FTCOND = TCOND / VISLAM;
        }
        const size_t N = (size_t)IM * JM * KM;
        std::vector<R> TXR(N), TXX(N), TXT(N), TRR(N), TRT(N), TTT(N), QXX(N), QRR(N), QTT(N);
        R FYPLUS = R(0);
        /* ---- DO 150: strain rates and the eddy viscosity of every cell ---- */
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    auto avg8 = [&](const std::vector<R> &A) {
                        return R(0.125) * (A3(A, i, j, k) + A3(A, i + 1, j, k) + A3(A, i + 1, j, k + 1) + A3(A, i, j, k + 1) +
                                           A3(A, i, j - 1, k) + A3(A, i + 1, j - 1, k) + A3(A, i + 1, j - 1, k + 1) +
                                           A3(A, i, j - 1, k + 1));
                    };
                    R WTAVG = avg8(WT_v), ROAVG = F3(ROAVG_CELL, i, j, k), TSAVG = avg8(T_STATIC_v);
                    R RAVG = F2(RAVG_CELL, j, k);
                    R DVXDX, DVXDR, DVXDT, DVRDX, DVRDR, DVRDT, DWTDX, DWTDR, DWTDT, DTDX, DTDR, DTDT;
                    gradvel(i, j, k, VX_v, DVXDX, DVXDR, DVXDT);
                    gradvel(i, j, k, VR_v, DVRDX, DVRDR, DVRDT);
                    gradvel(i, j, k, WT_v, DWTDX, DWTDR, DWTDT);
                    gradvel(i, j, k, T_STATIC_v, DTDX, DTDR, DTDT);
                    size_t n = ijk(i, j, k);
                    TXR[n] = DVXDR + DVRDX;
                    TXX[n] = DVXDX;
                    TXT[n] = DWTDX + DVXDT;
                    TRR[n] = DVRDR;
                    TRT[n] = DWTDR + DVRDT - WTAVG / RAVG;
                    TTT[n] = DWTDT;
                    QXX[n] = DTDX;
                    QRR[n] = DTDR;
                    QTT[n] = DTDT;
                    R VORTX = DVRDT - DWTDR - WTAVG / RAVG, VORTR = DWTDX - DVXDT, VORTT = DVXDR - DVRDX;
                    R VORT = om::sqrt(VORTX * VORTX + VORTR * VORTR + VORTT * VORTT);
                    if (VORT > VORT_MAX) VORT = VORT_MAX;
                    R TURBVIS_WALL = ROAVG * F3(XLENGTH, i, j, k) * VORT * FMIXUP;
                    FYPLUS = fyplus_of(F3(Y_PLUS, i, j, k), YPLAM, YPTURB, FYPLUS);
                    TURBVIS_WALL = TURBVIS_WALL * FYPLUS;
                    if (REYNO < R(0.0001)) VISLAM = (om::fabs(REYNO) / R(100000.0)) * om::pow(TSAVG / R(288.0), R(0.62));
                    R VISTOT = VISLAM * (R(1) + F3(FST_RAT, i, j, k)) + TURBVIS_WALL;
                    R VISLIM = TURBVIS_LIM * VISLAM;
                    if (VISTOT > VISLIM) VISTOT = VISLIM;
                    F3(VISC_RAT, i, j, k) = VISTOT / VISLAM;
                    F3(VISC_LAM, i, j, k) = VISLAM;
                }
        /* ---- DO 160: transition ---- */
        for (int j = 2; j <= JM; ++j) {
            int NRW = F1(NROW, j);
            int JROW = j - F1(JSTART, NRW) + 1;
            auto line = [&](bool upstream, int i0, int i1, int k0, int k1) {
                bool lam = upstream;
                if (!lam) {
                    R RMAX = R(0.0);
                    for (int k = k0; k <= k1; ++k)
                        for (int i = i0; i <= i1; ++i)
                            if (!(F3(VISC_RAT, i, j, k) < RMAX)) RMAX = F3(VISC_RAT, i, j, k);
                    lam = !(RMAX > FTRANS);
                }
                if (lam)
                    for (int k = k0; k <= k1; ++k)
                        for (int i = i0; i <= i1; ++i) F3(VISC_RAT, i, j, k) = R(1.0);
            };
            for (int i = 1; i <= IMM1; ++i) {
                line(JROW < F1(JTRAN_K1, NRW), i, i, 1, KMID);
                line(JROW < F1(JTRAN_KM, NRW), i, i, KMID, KMM1);
            }
            for (int k = 1; k <= KMM1; ++k) {
                line(JROW < F1(JTRAN_I1, NRW), 1, IMID, k, k);
                line(JROW < F1(JTRAN_IM, NRW), IMID, IMM1, k, k);
            }
        }
        /* ---- DO 190: stresses and heat flows ---- */
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    size_t n = ijk(i, j, k);
                    VISLAM = F3(VISC_LAM, i, j, k);
                    R VISTOT = F3(VISC_RAT, i, j, k) * VISLAM;
                    R THCOND = CP * VISTOT / PRANDTL;
                    R VISTOT2 = R(2.0) * VISTOT;
                    TXR[n] = VISTOT * TXR[n];
                    TXX[n] = VISTOT2 * TXX[n];
                    TXT[n] = VISTOT * TXT[n];
                    TRR[n] = VISTOT2 * TRR[n];
                    TRT[n] = VISTOT * TRT[n];
                    TTT[n] = VISTOT2 * TTT[n];
                    QXX[n] = -THCOND * QXX[n];
                    QRR[n] = -THCOND * QRR[n];
                    QTT[n] = -THCOND * QTT[n];
                }
        viscous_walls_and_forces(TXR, TXX, TXT, TRR, TRT, TTT, QXX, QRR, QTT, false);
    }

    /* The wall shear stresses, the I- and K-face stresses and the body-force
       update that NEW_LOSS (12975-13462) and SPAL_LOSS (14160-14832) share;
       they differ only in SPAL_LOSS setting Y_PLUS up to I = IM on the
       I = IM side (14236) where NEW_LOSS stops at IMM1 (12742). */
    void viscous_walls_and_forces(std::vector<R> &TXR, std::vector<R> &TXX, std::vector<R> &TXT, std::vector<R> &TRR,
                                  std::vector<R> &TRT, std::vector<R> &TTT, std::vector<R> &QXX, std::vector<R> &QRR,
                                  std::vector<R> &QTT, bool sa) {
        const size_t N = (size_t)IM * JM * KM;
        std::vector<R> FX(N, R(0)), FRr(N, R(0)), FT(N, R(0)), ES(N, R(0));
        /* TRX = TXR, TTX = TXT, TTR = TRT */
        if (YPLUSWALL < R(-10.0)) set_pwallgrad();
        const R VISLAM16 = VISLAM * R(16.0);
        auto iface = [&](int I, int IM1, int j, int k, R &XFOR, R &RFOR, R &TFOR, R &QFLOW, R &WVISC) {
            size_t a = ijk(I, j, k), b = ijk(IM1, j, k);
            R abr = F3(ABR, I, j, k), abt = F2(ABT, j, k), abx = F3(ABX, I, j, k);
            XFOR = R(0.5) * ((TXR[a] + TXR[b]) * abr + (TXT[a] + TXT[b]) * abt + (TXX[a] + TXX[b]) * abx);
            RFOR = R(0.5) * ((TRR[a] + TRR[b]) * abr + (TRT[a] + TRT[b]) * abt + (TXR[a] + TXR[b]) * abx);
            TFOR = R(0.5) * ((TRT[a] + TRT[b]) * abr + (TTT[a] + TTT[b]) * abt + (TXT[a] + TXT[b]) * abx);
            QFLOW = R(0.5) * ((QXX[a] + QXX[b]) * abx + (QRR[a] + QRR[b]) * abr + (QTT[a] + QTT[b]) * abt);
            R VXAVG = F3(VX, I, j, k) + F3(VX, I, j - 1, k) + F3(VX, I, j - 1, k + 1) + F3(VX, I, j, k + 1);
            R VRAVG = F3(VR, I, j, k) + F3(VR, I, j - 1, k) + F3(VR, I, j - 1, k + 1) + F3(VR, I, j, k + 1);
            R VTAVG = F3(VT, I, j, k) + F3(VT, I, j - 1, k) + F3(VT, I, j - 1, k + 1) + F3(VT, I, j, k + 1);
            WVISC = R(-0.25) * (XFOR * VXAVG + RFOR * VRAVG + TFOR * VTAVG);
        };
        /* ---- DO 200: blade surfaces, the periodic face and the I faces ---- */
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j) {
                int NRW = F1(NROW, j);
                bool wall = F1(IND, j) != 0 &&
                            !(F1(KTIPS, NRW) > 0 && k >= F1(KTIPS, NRW) && k < F1(KTIPE, NRW));
                if (wall) {
                    for (int side = 0; side < 2; ++side) {
                        int iw = side == 0 ? 2 : IMM1, ic = side == 0 ? 1 : IMM1, ia = side == 0 ? 1 : IM;
                        auto s4 = [&](const std::vector<R> &A) {
                            return A3(A, iw, j, k) + A3(A, iw, j - 1, k) + A3(A, iw, j - 1, k + 1) + A3(A, iw, j, k + 1);
                        };
                        R VXA = s4(VX_v), VRA = s4(VR_v), WTA = s4(WT_v), ROA = s4(RO_v);
                        R WAVG = om::sqrt(WTA * WTA + VXA * VXA + VRA * VRA);
                        R bx = F3(ABX, ia, j, k), br = F3(ABR, ia, j, k), bt = F2(ABT, j, k);
                        R AREA = om::sqrt(bx * bx + br * br + bt * bt);
                        R DPERP = F3(VOL, ic, j, k) / AREA;
                        R TW;
                        if (YPLUSWALL < R(-0.001)) {
                            R &yp = side == 0 ? F2(YPLUS_I1, j, k) : F2(YPLUS_IM, j, k);
                            R YN;
                            wallfun(DPERP, F3(DPDS_CELL, ic, j, k), R(0.25) * ROA, TW, yp, R(0.25) * WAVG, YN);
                            yp = std::min(R(1000.0), YN);
                        } else {
                            R RE = DPERP * ROA * WAVG / VISLAM16;
                            TW = nl_twall(RE, DPERP, side == 0 ? F1(ROUGH_L, NRW) : F1(ROUGH_U, NRW), ROA, WAVG);
                        }
                        int i0 = side == 0 ? 1 : IMID + 1, i1 = side == 0 ? IMID : (sa ? IM : IMM1);
                        for (int i = i0; i <= i1; ++i) {
                            R VSTAR = om::sqrt(TW / (R(0.25) * ROA));
                            R YPLS = VSTAR * om::sqrt(F3(DWALLSQ, i, j, k)) * (R(0.25) * ROA) / VISLAM;
                            F3(Y_PLUS, i, j, k) = std::min(R(1000.0), YPLS);
                        }
                        R FMULT = -TW * AREA / WAVG;
                        R TFc = FMULT * WTA;
                        size_t c = ijk(ic, j, k);
                        FX[c] = FX[c] + FMULT * VXA;
                        FRr[c] = FRr[c] + FMULT * VRA;
                        FT[c] = FT[c] + TFc;
                        ES[c] = ES[c] + TFc * F1(WRAD, j) * F2(RAVG_CELL, j, k);
                    }
                }
                bool skip = (F1(IND, j) == 1 && k < F1(KTIPS, NRW)) || k > F1(KTIPE, NRW);
                R XFOR, RFOR, TFOR, QFLOW, WVISC;
                if (!skip) {
                    iface(1, IMM1, j, k, XFOR, RFOR, TFOR, QFLOW, WVISC);
                    size_t a = ijk(1, j, k), b = ijk(IMM1, j, k);
                    std::vector<R> *FF[3] = {&FX, &FRr, &FT};
                    R fl[3] = {XFOR, RFOR, TFOR};
                    for (int f = 0; f < 3; ++f) {
                        std::vector<R> &A = *FF[f];
                        A[b] = A[b] + fl[f];
                        A[a] = A[a] - fl[f];
                        R AVG = R(0.5) * (A[a] + A[b]);
                        A[a] = AVG;
                        A[b] = AVG;
                    }
                    ES[a] = ES[a] + QFLOW + WVISC;
                    ES[b] = ES[b] - QFLOW - WVISC;
                    R AVG = R(0.5) * (ES[a] + ES[b]);
                    ES[a] = AVG;
                    ES[b] = AVG;
                }
                for (int I = 2; I <= IMM1; ++I) {
                    iface(I, I - 1, j, k, XFOR, RFOR, TFOR, QFLOW, WVISC);
                    size_t a = ijk(I, j, k), b = ijk(I - 1, j, k);
                    FX[b] = FX[b] + XFOR;
                    FX[a] = FX[a] - XFOR;
                    FRr[b] = FRr[b] + RFOR;
                    FRr[a] = FRr[a] - RFOR;
                    FT[b] = FT[b] + TFOR;
                    FT[a] = FT[a] - TFOR;
                    ES[a] = ES[a] + QFLOW + WVISC;
                    ES[b] = ES[b] - QFLOW - WVISC;
                }
            }
        /* ---- DO 400: hub and casing, then the K faces ---- */
        for (int j = 2; j <= JM; ++j) {
            int NRW = F1(NROW, j);
            for (int i = 1; i <= IMM1; ++i) {
                for (int side = 0; side < 2; ++side) {
                    int kn = side == 0 ? 2 : KMM1, kc = side == 0 ? 1 : KMM1, ka = side == 0 ? 1 : KM;
                    auto s4 = [&](const std::vector<R> &A) {
                        return A3(A, i, j, kn) + A3(A, i + 1, j, kn) + A3(A, i + 1, j - 1, kn) + A3(A, i, j - 1, kn);
                    };
                    R VXA = s4(VX_v), VRA = s4(VR_v), VTA = s4(VT_v), ROA = s4(RO_v);
                    R RAVG = F2(R, j, kn) + F2(R, j, kn) + F2(R, j - 1, kn) + F2(R, j - 1, kn);
                    R WW = side == 0 ? F1(WHUB, j) : F1(WTIP, j);
                    R WTA = VTA - WW * RAVG;
                    R WAVG = om::sqrt(VXA * VXA + VRA * VRA + WTA * WTA);
                    R sx = F3(ASX, i, j, ka), sr = F3(ASR, i, j, ka);
                    R AREA = om::sqrt(sx * sx + sr * sr);
                    R DPERP = F3(VOL, i, j, kc) / AREA;
                    R TW;
                    if (YPLUSWALL < R(-0.001)) {
                        R &yp = side == 0 ? FIJ(YPLUS_K1, i, j) : FIJ(YPLUS_KM, i, j);
                        R YN;
                        wallfun(DPERP, F3(DPDS_CELL, i, j, kc), R(0.25) * ROA, TW, yp, R(0.25) * WAVG, YN);
                        yp = std::min(R(1000.0), YN);
                    } else {
                        R RE = DPERP * ROA * WAVG / VISLAM16;
                        TW = nl_twall(RE, DPERP, side == 0 ? F1(ROUGH_H, NRW) : F1(ROUGH_T, NRW), ROA, WAVG);
                    }
                    bool yset = side == 0 ? (IBOUND == 0 || IBOUND == 2) : (IBOUND <= 1);
                    if (yset) {
                        int k0 = side == 0 ? 1 : KMID + 1, k1 = side == 0 ? KMID : KMM1;
                        for (int k = k0; k <= k1; ++k) {
                            R VSTAR = om::sqrt(TW / (R(0.25) * ROA));
                            R YPLS = VSTAR * om::sqrt(F3(DWALLSQ, i, j, k)) * (R(0.25) * ROA) / VISLAM;
                            R YPLSP = F3(Y_PLUS, i, j, k);
                            F3(Y_PLUS, i, j, k) = std::min(YPLS, YPLSP);
                        }
                    }
                    R FMULT = -TW * AREA / WAVG;
                    if (side == 0 ? (IBOUND == 1 || IBOUND > 2) : (IBOUND >= 2)) FMULT = R(0.0);
                    R TFc = FMULT * WTA;
                    size_t c = ijk(i, j, kc);
                    FX[c] = FX[c] + FMULT * VXA;
                    FRr[c] = FRr[c] + FMULT * VRA;
                    FT[c] = FT[c] + TFc;
                    ES[c] = ES[c] + TFc * R(0.25) * WW * RAVG;
                }
                for (int K = 2; K <= KMM1; ++K) {
                    size_t a = ijk(i, j, K), b = ijk(i, j, K - 1);
                    R sr = F3(ASR, i, j, K), sx = F3(ASX, i, j, K);
                    R XFOR = R(0.5) * ((TXR[a] + TXR[b]) * sr + (TXX[a] + TXX[b]) * sx);
                    R RFOR = R(0.5) * ((TRR[a] + TRR[b]) * sr + (TXR[a] + TXR[b]) * sx);
                    R TFOR = R(0.5) * ((TRT[a] + TRT[b]) * sr + (TXT[a] + TXT[b]) * sx);
                    R QFLOW = R(0.5) * ((QXX[a] + QXX[b]) * sx + (QRR[a] + QRR[b]) * sr);
                    R VXAVG = F3(VX, i, j, K) + F3(VX, i + 1, j, K) + F3(VX, i + 1, j - 1, K) + F3(VX, i, j - 1, K);
                    R VRAVG = F3(VR, i, j, K) + F3(VR, i + 1, j, K) + F3(VR, i + 1, j - 1, K) + F3(VR, i, j - 1, K);
                    R VTAVG = F3(VT, i, j, K) + F3(VT, i + 1, j, K) + F3(VT, i + 1, j - 1, K) + F3(VT, i, j - 1, K);
                    R WVISC = R(-0.25) * (XFOR * VXAVG + RFOR * VRAVG + TFOR * VTAVG);
                    FX[b] = FX[b] + XFOR;
                    FX[a] = FX[a] - XFOR;
                    FRr[b] = FRr[b] + RFOR;
                    FRr[a] = FRr[a] - RFOR;
                    FT[b] = FT[b] + TFOR;
                    FT[a] = FT[a] - TFOR;
                    ES[a] = ES[a] + QFLOW + WVISC;
                    ES[b] = ES[b] - QFLOW - WVISC;
                }
            }
        }
        /* ---- DO 500 ---- */
        R RF_VIS1 = R(1.0) - RF_VIS;
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    size_t n = ijk(i, j, k);
                    F3(XFORCE, i, j, k) = RF_VIS1 * F3(XFORCE, i, j, k) - RF_VIS * FX[n];
                    F3(TFORCE, i, j, k) = RF_VIS1 * F3(TFORCE, i, j, k) - RF_VIS * FT[n] * F2(RAVG_CELL, j, k);
                    F3(RFORCE, i, j, k) = RF_VIS1 * F3(RFORCE, i, j, k) - RF_VIS * FRr[n];
                    F3(QSOURCE, i, j, k) = RF_VIS1 * F3(QSOURCE, i, j, k) - RF_VIS * ES[n];
                }
    }

    /* ================================================================== */
    /*  SPAL_LOSS (ILOS >= 200)  multall-open-18.3.f:13586-14832, with      */
    /*  GRADCELL 13516-13585; the wall shear and face stresses are         */
    /*  NEW_LOSS's (viscous_walls_and_forces)                              */
    /* ================================================================== */
    /* cell gradient of a cell-centred quantity by Gauss' theorem
       (13516-13585).  Cells past J = JM read the never-written COMMON slots
       of V, which hold zero. */
    void gradcell(int i, int j, int k, const std::vector<R> &V, R &DVDX, R &DVDR, R &DVDT) {
        int ip1 = i + 1, jp1 = j + 1, kp1 = k + 1, im1 = i - 1, jm1 = j - 1, km1 = k - 1;
        if (i == 1) im1 = IMM1;
        if (i == IMM1) ip1 = 1;
        if (k == 1) km1 = 1;
        if (k == KMM1) kp1 = KMM1;
        auto v = [&](int a, int b, int c) -> R { return b > JM ? R(0) : V[ijk(a, b, c)]; };
        R RVOL = R(0.5) / F3(VOL, i, j, k);
        R VAVGJ1 = v(i, j, k) + v(i, jm1, k);
        R VAVGJ2 = v(i, j, k) + v(i, jp1, k);
        R VAVGI1 = v(i, j, k) + v(im1, j, k);
        R VAVGI2 = v(i, j, k) + v(ip1, j, k);
        R VAVGK1 = v(i, j, k) + v(i, j, km1);
        R VAVGK2 = v(i, j, k) + v(i, j, kp1);
        if (F1(IND, j) == 1) {
            if (i == 1) VAVGI1 = R(0.0);
            if (i == IMM1) VAVGI2 = R(0.0);
        }
        if (k == 1 && (IBOUND == 0 || IBOUND == 2)) VAVGK1 = R(0.0);
        if (k == KMM1 && IBOUND <= 1) VAVGK2 = R(0.0);
        DVDX = -(VAVGJ2 * F3(AQX, i, j, k) - VAVGJ1 * F3(AQX, i, jm1, k) + VAVGI1 * F3(ABX, i, j, k) -
                 VAVGI2 * F3(ABX, ip1, j, k) + VAVGK1 * F3(ASX, i, j, k) - VAVGK2 * F3(ASX, i, j, kp1)) *
               RVOL;
        DVDR = -(VAVGJ2 * F3(AQR, i, j, k) - VAVGJ1 * F3(AQR, i, jm1, k) + VAVGI1 * F3(ABR, i, j, k) -
                 VAVGI2 * F3(ABR, ip1, j, k) + VAVGK1 * F3(ASR, i, j, k) - VAVGK2 * F3(ASR, i, j, kp1)) *
                   RVOL -
               v(i, j, k) / F2(RAVG_CELL, j, k);
        DVDT = -(VAVGI1 - VAVGI2) * F2(ABT, j, k) * RVOL;
    }

    /* the free-stream transported viscosity (13832-13838, 4681-4684) */
    R sa_transvis_in(R vislam) const {
        R fs = F1(FSTURB, 1);
        if (fs < R(1.0)) return R(4.35) * vislam * om::pow(fs, R(0.25));
        return vislam * (R(3.5) + fs * R(0.85));
    }

    std::vector<R> ABS_VORT_w, TRANS_VORT_w, DYN_VIS_ML_w, GRAD_TVIS_w, TVISGRADX_w, TVISGRADR_w, TVISGRADT_w;
    std::vector<R> REYNOLDS_w;

    void spal_loss() {
        const int NDAMP = 100000;
        if (NSTEP == 1 || NSTEP < NSTEPS_MAX / 4) {
            if (REYNO > R(100.)) {
                int J1 = F1(JLE, 1), J2 = F1(JTE, 1);
                if (F1(JLE, 1) > JM) J1 = 1;
                if (F1(JTE, 1) > JM) J2 = JM;
                R XCHORD = F2(SMERID, J2, KMID) - F2(SMERID, J1, KMID);
                R a = F3(ROVX, IMID, J2, KMID), b = F3(ROVR, IMID, J2, KMID), c = F3(ROWT, IMID, J2, KMID);
                VISLAM = XCHORD * om::sqrt(a * a + b * b + c * c) / REYNO;
            }
            if (REYNO > R(0.0) && REYNO < R(99.99)) VISLAM = REYNO / R(100000.);
            if (REYNO < R(0.0)) VISLAM = -REYNO * R(1.0E-5);
            TCOND = CP * VISLAM / PRANDTL;
            FTCOND = TCOND / VISLAM;
        }
        const size_t N = (size_t)IM * JM * KM;
        std::vector<R> TXR(N), TXX(N), TXT(N), TRR(N), TRT(N), TTT(N), QXX(N), QRR(N), QTT(N);
        if (ABS_VORT_w.size() != N) {
            ABS_VORT_w.assign(N, R(0)); TRANS_VORT_w.assign(N, R(0)); DYN_VIS_ML_w.assign(N, R(0));
            GRAD_TVIS_w.assign(N, R(0)); TVISGRADX_w.assign(N, R(0)); TVISGRADR_w.assign(N, R(0));
            TVISGRADT_w.assign(N, R(0));
            REYNOLDS_w.assign(NROWS, R(0));
        }
        if (FAC_PGRAD > R(0.001)) set_pwallgrad();
        R VORTICITY_FAC = R(0), PGRAD_FAC = R(0);   /* scalars: the last cell's values are used below */
        /* ---- DO 1000: strain rates, vorticity and the S-A viscosity ---- */
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j) {
                int NRW = F1(NROW, j), JTEDGE = F1(JTE, NRW);
                for (int i = 1; i <= IMM1; ++i) {
                    auto avg8 = [&](const std::vector<R> &A) {
                        return R(0.125) * (A3(A, i, j, k) + A3(A, i + 1, j, k) + A3(A, i + 1, j, k + 1) + A3(A, i, j, k + 1) +
                                           A3(A, i, j - 1, k) + A3(A, i + 1, j - 1, k) + A3(A, i + 1, j - 1, k + 1) +
                                           A3(A, i, j - 1, k + 1));
                    };
                    auto sum8 = [&](const std::vector<R> &A) {
                        return A3(A, i, j, k) + A3(A, i + 1, j, k) + A3(A, i + 1, j, k + 1) + A3(A, i, j, k + 1) +
                               A3(A, i, j - 1, k) + A3(A, i + 1, j - 1, k) + A3(A, i + 1, j - 1, k + 1) + A3(A, i, j - 1, k + 1);
                    };
                    R WTAVG = avg8(WT_v), ROAVG = F3(ROAVG_CELL, i, j, k), TSAVG = avg8(T_STATIC_v);
                    R RAVG = F2(RAVG_CELL, j, k);
                    R DVXDX, DVXDR, DVXDT, DVRDX, DVRDR, DVRDT, DWTDX, DWTDR, DWTDT, DTDX, DTDR, DTDT;
                    gradvel(i, j, k, VX_v, DVXDX, DVXDR, DVXDT);
                    gradvel(i, j, k, VR_v, DVRDX, DVRDR, DVRDT);
                    gradvel(i, j, k, WT_v, DWTDX, DWTDR, DWTDT);
                    gradvel(i, j, k, T_STATIC_v, DTDX, DTDR, DTDT);
                    size_t n = ijk(i, j, k);
                    TXR[n] = DVXDR + DVRDX;
                    TXX[n] = DVXDX;
                    TXT[n] = DWTDX + DVXDT;
                    TRR[n] = DVRDR;
                    TRT[n] = DWTDR + DVRDT - WTAVG / RAVG;
                    TTT[n] = DWTDT;
                    QXX[n] = DTDX;
                    QRR[n] = DTDR;
                    QTT[n] = DTDT;
                    R VORTX = DVRDT - DWTDR - WTAVG / RAVG, VORTR = DWTDX - DVXDT, VORTT = DVXDR - DVRDX;
                    R VORT = om::sqrt(VORTX * VORTX + VORTR * VORTR + VORTT * VORTT);
                    if (j == F1(JSTART, NRW)) VORT = R(0.0);
                    if (VORT > VORT_MAX) VORT = VORT_MAX;
                    if (F1(INDMIX, j) == 1) VORT = A3(ABS_VORT_w, i, j - 1, k);
                    A3(ABS_VORT_w, i, j, k) = VORT;
                    R WREL = R(0), VXAVG = R(0), VRAVG = R(0);
                    if (FAC_VORT > R(0.001) || FAC_PGRAD > R(0.001)) {
                        WTAVG = sum8(WT_v);
                        VXAVG = sum8(VX_v);
                        VRAVG = sum8(VR_v);
                        WREL = om::sqrt(VXAVG * VXAVG + VRAVG * VRAVG + WTAVG * WTAVG);
                    }
                    if (FAC_VORT > R(0.001)) {
                        R HELICITY = (VXAVG * VORTX + VRAVG * VORTR + WTAVG * VORTT) / (WREL * VORT);
                        VORTICITY_FAC = R(1.0) + FAC_VORT * om::tanh(R(3.0) * HELICITY * HELICITY);
                    }
                    if (FAC_PGRAD > R(0.001)) {
                        R a = F3(VX, IMID, j, k), b = F3(VR, IMID, j, k), c = F3(WT, IMID, j, k);
                        R WLIM = R(0.1) * om::sqrt(a * a + b * b + c * c);
                        if (WREL < WLIM) WREL = WLIM;
                        WREL = R(0.125) * WREL;
                        R PGRAD = F3(DPDS_CELL, i, j, k);
                        if (PGRAD < R(0.0)) PGRAD = R(0.0);
                        R PTERM = PGRAD * VISLAM / (ROAVG * ROAVG * WREL * WREL * WREL);
                        PTERM = PTERM * REYNOLDS_w[NRW - 1];
                        PGRAD_FAC = R(1.0) + FAC_PGRAD * om::tanh(PTERM * PTERM);
                    }
                    R TURBVIS_WALL = ROAVG * F3(XLENGTH, i, j, k) * VORT * FMIXUP;
                    if (REYNO < R(0.0001)) VISLAM = (om::fabs(REYNO) / R(100000.0)) * om::pow(TSAVG / R(288.0), R(0.62));
                    if (i == IMID && k == KMID && j == JTEDGE) {
                        R vx = F3(VX, i, j, k), vr = F3(VR, i, j, k), wt = F3(WT, i, j, k);
                        R WABS = om::sqrt(vx * vx + vr * vr + wt * wt);
                        R ROVEXIT = F3(RO, i, j, k) * WABS;
                        REYNOLDS_w[NRW - 1] = F1(CHORD, NRW) * ROVEXIT / VISLAM;
                    }
                    R VISTOT = VISLAM * (R(1) + F3(FST_RAT, i, j, k)) + TURBVIS_WALL;
                    R VISLIM = TURBVIS_LIM * VISLAM;
                    if (VISTOT > VISLIM) VISTOT = VISLIM;
                    R VISKLAM = VISLAM / ROAVG;
                    A3(DYN_VIS_ML_w, i, j, k) = VISTOT - VISLAM;
                    if (IF_RESTART == 0 && NSTEP == 1) F3(TRANS_DYN_VIS, i, j, k) = sa_transvis_in(VISLAM);
                    if (NSTEP == 1) F3(TRANS_KVIS, i, j, k) = F3(TRANS_DYN_VIS, i, j, k) / ROAVG;
                    R TRANSKVIS = F3(TRANS_KVIS, i, j, k);
                    R XI = TRANSKVIS / VISKLAM;
                    if (XI < R(1.1)) XI = R(1.1);
                    if (XI > TURBVIS_LIM) XI = TURBVIS_LIM;
                    R XI3 = XI * XI * XI;
                    R FV1 = XI3 / (XI3 + R(357.9));
                    R TRANSVISLIM = VISLIM / ROAVG / FV1;
                    if (TRANSKVIS > TRANSVISLIM) TRANSKVIS = TRANSVISLIM;
                    R VISTRU = TRANSKVIS * FV1 * ROAVG;
                    A3(TRANS_VORT_w, i, j, k) = A3(ABS_VORT_w, i, j, k);
                    VISTOT = VISTRU + VISLAM;
                    VISLIM = TURBVIS_LIM * VISLAM;
                    if (VISTOT > VISLIM) VISTOT = VISLIM;
                    F3(VISC_RAT, i, j, k) = VISTOT / VISLAM;
                    F3(VISC_LAM, i, j, k) = VISLAM;
                    F3(VISC_TURB, i, j, k) = VISTOT - VISLAM;
                }
            }
        /* ---- DO 1500: gradient of the kinematic transported viscosity ---- */
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JMM1; ++j) {
                int NRW = F1(NROW, j);
                for (int i = 1; i <= IMM1; ++i) {
                    R DX_, DR_, DT_;
                    gradcell(i, j, k, TRANS_KVIS_v, DX_, DR_, DT_);
                    A3(GRAD_TVIS_w, i, j, k) = DX_ * DX_ + DR_ * DR_ + DT_ * DT_;
                    R VISCEFF = F3(TRANS_KVIS, i, j, k) + F3(VISC_LAM, i, j, k);
                    A3(TVISGRADX_w, i, j, k) = VISCEFF * DX_;
                    A3(TVISGRADR_w, i, j, k) = VISCEFF * DR_;
                    A3(TVISGRADT_w, i, j, k) = VISCEFF * DT_;
                    if (j == F1(JSTART, NRW) || j == F1(JSTART, NRW) - 1) {
                        A3(GRAD_TVIS_w, i, j, k) = R(0.0);
                        A3(TVISGRADX_w, i, j, k) = R(0.0);
                        A3(TVISGRADR_w, i, j, k) = R(0.0);
                        A3(TVISGRADT_w, i, j, k) = R(0.0);
                    }
                }
            }
        /* ---- DO 1600: the source terms ---- */
        const R CW2 = R(0.3), SIGMA = R(0.6667), CB2 = R(0.622), CB1 = R(0.1355);
        const R CW1 = R(0.80607) + R(2.433);
        const R FST0 = FAC_ST0 * CB1, FST1 = FAC_ST1 / SIGMA, FST2 = FAC_ST2 * CB2 / SIGMA, FST3 = FAC_ST3 * CW1;
        const R FSTMIX = FAC_STMIX / R(NDAMP);
        const R RF_VIS1 = R(1.0) - RF_VIS;
        R FYPLUS = R(0);
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    FYPLUS = fyplus_of(F3(Y_PLUS, i, j, k), YPLAM, YPTURB, FYPLUS);
                    R TVISDDX, TVISDDR, TVISDDT, d1, d2;
                    gradcell(i, j, k, TVISGRADX_w, TVISDDX, d1, d2);
                    gradcell(i, j, k, TVISGRADR_w, d1, TVISDDR, d2);
                    gradcell(i, j, k, TVISGRADT_w, d1, d2, TVISDDT);
                    R ROAVG = F3(ROAVG_CELL, i, j, k);
                    R TVIS = F3(TRANS_KVIS, i, j, k);
                    R ST0 = FST0 * A3(TRANS_VORT_w, i, j, k) * TVIS;
                    if (FAC_VORT > R(0.001)) ST0 = ST0 * VORTICITY_FAC;
                    if (FAC_PGRAD > R(0.001)) ST0 = ST0 * PGRAD_FAC;
                    ST0 = ST0 * FYPLUS;
                    R ST1 = FST1 * (TVISDDX + TVISDDR + TVISDDT);
                    R ST2 = FST2 * A3(GRAD_TVIS_w, i, j, k);
                    R TAU = R(5.9488) * TVIS / A3(TRANS_VORT_w, i, j, k) / F3(DWALLSQ, i, j, k);
                    if (TAU > R(1.2)) TAU = R(1.2);
                    if (TAU < R(0.001)) TAU = R(0.001);
                    R G = TAU + CW2 * (TAU * TAU * TAU * TAU * TAU * TAU - TAU);
                    R G6CW6 = G * G * G * G * G * G / R(64.0);
                    R FW = G * om::pow((R(1) + R(0.015625)) / (R(1) + G6CW6), R(0.166667));
                    R ST3 = FST3 * FW * TVIS * TVIS / F3(DWALLSQ, i, j, k);
                    R ST_MIXL = FSTMIX * (A3(DYN_VIS_ML_w, i, j, k) - F3(VISC_TURB, i, j, k)) / F3(STEP, i, j, k);
                    F3(T_SOURCE, i, j, k) = RF_VIS1 * F3(T_SOURCE, i, j, k) +
                                            RF_VIS * (ROAVG * (ST0 + ST1 + ST2 - ST3) * F3(VOL, i, j, k) + ST_MIXL);
                    if (j > 2 && F1(INDMIX, j - 1) == 1) F3(T_SOURCE, i, j, k) = R(0.0);
                    if (j > 2 && F1(INDMIX, j - 2) == 1) F3(T_SOURCE, i, j, k) = R(0.0);
                }
        /* ---- DO 160: laminar regions pull the source towards a profile ---- */
        const int IEND1 = IMID / 2, IENDM = IMM1 - IEND1, KEND1 = KMID / 2, KENDM = KMM1 - KEND1;
        auto damp_to = [&](int i, int j, int k, R TVSPEC) {
            F3(T_SOURCE, i, j, k) = F3(T_SOURCE, i, j, k) - (F3(VISC_TURB, i, j, k) - TVSPEC) / F3(STEP, i, j, k) / R(NDAMP);
        };
        for (int j = 2; j <= JM; ++j) {
            int NRW = F1(NROW, j), J1 = F1(JSTART, NRW), JROW = j - J1 + 1;
            int JTRHUB = F1(JTRAN_K1, NRW), JTRTIP = F1(JTRAN_KM, NRW), JTRLOW = F1(JTRAN_I1, NRW),
                JTRUP = F1(JTRAN_IM, NRW), JLEROW = F1(JLE, NRW);
            for (int i = 1; i <= IMM1; ++i) {
                /* hub */
                if (!(JTRHUB <= 1 && FTRANS < R(0.1))) {
                    bool lam = JROW < JTRHUB;
                    if (!lam) {
                        R RMAX = R(0.0);
                        for (int k = 1; k <= KEND1; ++k)
                            if (!(F3(VISC_RAT, i, j, k) < RMAX)) RMAX = F3(VISC_RAT, i, j, k);
                        lam = !(RMAX > FTRANS);
                    }
                    if (lam) {
                        R TVEDGE = F3(VISC_TURB, i, j, KEND1);
                        for (int k = 1; k <= KEND1; ++k) {
                            R FK = R(KEND1 + 1 - k) / R(KEND1);
                            FK = FK * FK * (R(3) - R(2) * FK);
                            damp_to(i, j, k, FK * TVEDGE);
                        }
                    }
                }
                /* casing */
                if (!(JTRTIP <= 1 && FTRANS < R(0.1))) {
                    bool lam = JROW < JTRTIP;
                    if (!lam) {
                        R RMAX = R(0.0);
                        for (int k = KENDM; k <= KMM1; ++k)
                            if (!(F3(VISC_RAT, i, j, k) < RMAX)) RMAX = F3(VISC_RAT, i, j, k);
                        lam = !(RMAX > FTRANS);
                    }
                    if (lam) {
                        R TVEDGE = F3(VISC_TURB, i, j, KENDM);
                        for (int k = KENDM; k <= KMM1; ++k) {
                            R FK = R(k + 1 - KENDM) / R(KM - KENDM);
                            FK = FK * FK * (R(3) - R(2) * FK);
                            damp_to(i, j, k, FK * TVEDGE);
                        }
                    }
                }
            }
            for (int k = 1; k <= KMM1; ++k) {
                /* I = 1 surface */
                if (!(JTRLOW <= 1 && FTRANS < R(0.1)) && !(j <= JLEROW)) {
                    bool lam = JROW < JTRLOW || j < JLEROW;
                    if (!lam) {
                        R RMAX = R(0.0);
                        for (int i = 1; i <= IEND1; ++i)
                            if (!(F3(VISC_RAT, i, j, k) < RMAX)) RMAX = F3(VISC_RAT, i, j, k);
                        lam = !(RMAX > FTRANS);
                    }
                    if (lam) {
                        R TVEDGE = F3(VISC_TURB, IEND1, j, k);
                        for (int i = 1; i <= IEND1; ++i) {
                            R FI = R(IEND1 + 1 - i) / R(IEND1);
                            FI = FI * FI * (R(3) - R(2) * FI);
                            damp_to(i, j, k, FI * TVEDGE);
                        }
                    }
                }
                /* I = IM surface */
                if (!(JTRUP <= 1 && FTRANS < R(0.1)) && !(j <= JLEROW)) {
                    bool lam = JROW < JTRUP;
                    if (!lam) {
                        R RMAX = R(0.0);
                        for (int i = IENDM; i <= IMM1; ++i)
                            if (!(F3(VISC_RAT, i, j, k) < RMAX)) RMAX = F3(VISC_RAT, i, j, k);
                        lam = !(RMAX > FTRANS);
                    }
                    if (lam) {
                        R TVEDGE = F3(VISC_TURB, IENDM, j, k);
                        for (int i = IENDM; i <= IMM1; ++i) {
                            R FI = R(i + 1 - IENDM) / R(IM - IENDM);
                            FI = FI * FI * (R(3) - R(2) * FI);
                            damp_to(i, j, k, FI * TVEDGE);
                        }
                    }
                }
            }
        }
        /* ---- DO 190: stresses and heat flows with the final viscosity ---- */
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    size_t n = ijk(i, j, k);
                    VISLAM = F3(VISC_LAM, i, j, k);
                    R VISTOT = F3(VISC_RAT, i, j, k) * VISLAM;
                    R THCOND = CP * VISTOT / PRANDTL;
                    R VISTOT2 = R(2.0) * VISTOT;
                    TXR[n] = VISTOT * TXR[n];
                    TXX[n] = VISTOT2 * TXX[n];
                    TXT[n] = VISTOT * TXT[n];
                    TRR[n] = VISTOT2 * TRR[n];
                    TRT[n] = VISTOT * TRT[n];
                    TTT[n] = VISTOT2 * TTT[n];
                    QXX[n] = -THCOND * QXX[n];
                    QRR[n] = -THCOND * QRR[n];
                    QTT[n] = -THCOND * QTT[n];
                }
        viscous_walls_and_forces(TXR, TXX, TXT, TRR, TRT, TTT, QXX, QRR, QTT, true);
    }

    /* the transported viscosity's fluxes and source (LOOP 4279-4330), its
       TSTEP (NCALL = 2) and the floor and kinematic value after it
       (4340-4347) */
    void sa_transport() {
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 1; j <= JM; ++j) {
                int JP1 = j + 1;
                if (j == JM) JP1 = JM;
                if (j == 1) JP1 = 1;
                if (F1(INDMIX, j) == 1) JP1 = j;
                for (int i = 1; i <= IMM1; ++i)
                    A3(XFLUX, i, j, k) = A3(FLOWX, i, j, k) * (F3(TRANS_KVIS, i, j, k) + F3(TRANS_KVIS, i, JP1, k));
            }
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) A3(SOURCE, i, j, k) = R(-2.0) * F3(T_SOURCE, i, j, k);
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 2; i <= IMM1; ++i)
                    A3(TFLUX, i, j, k) = A3(FLOWT, i, j, k) * (F3(TRANS_KVIS, i - 1, j, k) + F3(TRANS_KVIS, i, j, k));
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j) {
                A3(TFLUX, 1, j, k) = A3(FLOWT, 1, j, k) * (F3(TRANS_KVIS, IMM1, j, k) + F3(TRANS_KVIS, 1, j, k));
                A3(TFLUX, IM, j, k) = A3(TFLUX, 1, j, k);
            }
        for (int k = 2; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i)
                    A3(RFLUX, i, j, k) = A3(FLOWR, i, j, k) * (F3(TRANS_KVIS, i, j, k - 1) + F3(TRANS_KVIS, i, j, k));
        for (int j = 2; j <= JM; ++j)
            for (int i = 1; i <= IMM1; ++i) {
                A3(RFLUX, i, j, 1) = R(0.0);
                A3(RFLUX, i, j, KM) = R(0.0);
            }
        tstep(TRANS_DYN_VIS_v, DEL_DYNVIS_v, 2);
        R TRANSVISMIN = R(0.1) * F3(VISC_LAM, IMID, 2, KMID);
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    if (F3(TRANS_DYN_VIS, i, j, k) < TRANSVISMIN) F3(TRANS_DYN_VIS, i, j, k) = TRANSVISMIN;
                    F3(TRANS_KVIS, i, j, k) = F3(TRANS_DYN_VIS, i, j, k) / F3(ROAVG_CELL, i, j, k);
                }
    }

    int loss_init() override {
        if (!committed) return fail(MGPU_E_STATE, "loss_init before commit");
        R save_rf = RF_VIS, save_fm = FMIXUP;
        int save_n = NSTEP;
        RF_VIS = R(1.0);
        FMIXUP = R(1.0);
        NSTEP = 1;
        // SETUP 7354-7356: no loss routine for an inviscid problem (ILOS = 0)
        if (ILOS >= 200) spal_loss();
        else if (ILOS >= 100) new_loss();
        else if (ILOS == 10) loss();
        RF_VIS = save_rf;
        FMIXUP = save_fm;
        NSTEP = save_n;
        return 0;
    }

    /* ================================================================== */
    /*  NEW_MIXPLAN   multall-open-18.3.f:14922-15251  (IFGAS=0, ITIMST=3) */
    /* ================================================================== */
    void new_mixplan() {
        R RFMIX1 = R(1.0) - RFMIX;
        std::vector<R> ALPHAA(IM + 1), GAMA(IM + 1), WREF_JP2(IM + 1), ROREF_JP2(IM + 1), PISENT(IM + 1),
            ROISENT(IM + 1), WMACH_JP2(IM + 1), TISENT(IM + 1), WIS_JP2(IM + 1);
        for (int nr = 1; nr <= NRWSM1; ++nr) {
            for (int k = 1; k <= KM; ++k) {
                int KSUB = (k == KM) ? KM - 1 : k;
                int j = F1(JMIX, nr);
                int JP1, JP2, JP3, JP4;
                R F_ANGLE;
                if (A3(FLOWX, IMID, j, KSUB) < R(0.0)) {
                    JP1 = j + 1; JP2 = j + 2; JP3 = j + 3; JP4 = j + 4;
                    F_ANGLE = FANGLE;
                } else {
                    j = F1(JMIX, nr) + 1;
                    JP1 = j - 1; JP2 = j - 2; JP3 = j - 3; JP4 = j - 4;
                    F_ANGLE = R(0.0);
                }
                (void)JP4;
                R F_ANGLE1 = R(1.0) - F_ANGLE;
                R RJP1 = F2(R, JP1, k);
                R UJP1 = F2(UBLADE, JP1, k);
                R ROMIX = F3(RO, IMID, JP1, k);
                R VXMIX = F3(ROVX, IMID, JP1, k) / ROMIX;
                R VRMIX = F3(ROVR, IMID, JP1, k) / ROMIX;
                R VTMIX = F3(RORVT, IMID, JP1, k) / ROMIX / RJP1;
                R ROEMIX = F3(ROE, IMID, JP1, k);
                R VMSQ = VXMIX * VXMIX + VRMIX * VRMIX;
                R VABSQ = VMSQ + VTMIX * VTMIX;
                R WTMIX = VTMIX - UJP1;
                R WMIXSQ = VMSQ + WTMIX * WTMIX;
                R WMIX = om::sqrt(WMIXSQ);
                R ALPHAMIX = om::asin(WTMIX / WMIX);
                R GAMAMIX = om::atan2(VRMIX, VXMIX);
                R TMIX = (ROEMIX / ROMIX - R(0.5) * VABSQ) / CV;
                R ROTHALPY = CP * TMIX + R(0.5) * (WMIXSQ - UJP1 * UJP1);
                R GAGAS = GA;
                R PMIX = ROMIX * RGAS * TMIX;
                int NMACH = 0;
                R RJP2 = F2(R, JP2, k), UNOWJP2 = F2(UBLADE, JP2, k);
                for (int i = 1; i <= IM; ++i) {
                    R ROJP2 = F3(RO, i, JP2, k);
                    R XVELJP2 = F3(ROVX, i, JP2, k) / ROJP2;
                    R RVELJP2 = F3(ROVR, i, JP2, k) / ROJP2;
                    R TVELJP2 = F3(RORVT, i, JP2, k) / RJP2 / ROJP2;
                    R WTJP2 = TVELJP2 - UNOWJP2;
                    R VMSQJP2 = XVELJP2 * XVELJP2 + RVELJP2 * RVELJP2;
                    R VELSQJP2 = VMSQJP2 + TVELJP2 * TVELJP2;
                    R WACT_SQ_JP2 = VMSQJP2 + WTJP2 * WTJP2;
                    R WACT_JP2 = om::sqrt(WACT_SQ_JP2);
                    R RO_ACT_JP2 = ROJP2;
                    R T_ACT_JP2 = (F3(ROE, i, JP2, k) / ROJP2 - R(0.5) * VELSQJP2) / CV;
                    R RJP3 = F2(R, JP3, k), UNOWJP3 = F2(UBLADE, JP3, k);
                    R ROJP3 = F3(RO, i, JP3, k);
                    R ROVXJP3 = F3(ROVX, i, JP3, k), ROVRJP3 = F3(ROVR, i, JP3, k);
                    R ROVTJP3 = F3(RORVT, i, JP3, k) / RJP3;
                    R ROWTJP3 = ROVTJP3 - UNOWJP3 * ROJP3;
                    R ROVMSQJP3 = ROVXJP3 * ROVXJP3 + ROVRJP3 * ROVRJP3;
                    R ROWRELSQJP3 = ROVMSQJP3 + ROWTJP3 * ROWTJP3;
                    R ROWRELJP3 = om::sqrt(ROWRELSQJP3);
                    R ALPHAJP3 = om::asin(ROWTJP3 / ROWRELJP3);
                    R GAMAJP3 = om::atan2(ROVRJP3, ROVXJP3);
                    R PSTAT = ROJP2 * RGAS * T_ACT_JP2;
                    R TISENT_JP2 = TMIX * om::pow(PSTAT / PMIX, FGA);
                    R WIS_SQ_JP2 = R(2) * (ROTHALPY - CP * TISENT_JP2 + R(0.5) * UNOWJP2 * UNOWJP2);
                    R ROISENT_JP2 = PSTAT / RGAS / TISENT_JP2;
                    ROISENT[i] = ROISENT_JP2;
                    PISENT[i] = PSTAT;
                    TISENT[i] = TISENT_JP2;
                    if (WIS_SQ_JP2 < R(1.0)) WIS_SQ_JP2 = R(1.0);
                    WIS_JP2[i] = om::sqrt(WIS_SQ_JP2);
                    WREF_JP2[i] = WACT_JP2;
                    ROREF_JP2[i] = RO_ACT_JP2;
                    WMACH_JP2[i] = WACT_JP2 / om::sqrt(GAGAS * RGAS * T_ACT_JP2);
                    if (WMACH_JP2[i] > R(1.0)) NMACH = NMACH + 1;
                    ALPHAA[i] = F_ANGLE1 * ALPHAMIX + F_ANGLE * ALPHAJP3;
                    GAMA[i] = F_ANGLE1 * GAMAMIX + F_ANGLE * GAMAJP3;
                }
                if (NMACH != 0) {
                    R FROTN = R(1.0);
                    if (WTMIX < R(0.0)) FROTN = R(-1.0);
                    for (int i = IMID + 1; i <= IM; ++i) {
                        int im1 = i - 1;
                        if (WMACH_JP2[i] > R(1.001) && WMACH_JP2[im1] > R(1.001)) {
                            R DELP = PISENT[i] - PISENT[im1];
                            R DELTAI = om::sqrt(WMACH_JP2[i] * WMACH_JP2[i] - R(1)) / (ROREF_JP2[i] * WREF_JP2[i] * WREF_JP2[i]);
                            R DELTAIM1 = om::sqrt(WMACH_JP2[im1] * WMACH_JP2[im1] - R(1)) /
                                         (ROREF_JP2[im1] * WREF_JP2[im1] * WREF_JP2[im1]);
                            ALPHAA[i] = ALPHAA[im1] + FROTN * DELP * R(0.5) * (DELTAI + DELTAIM1);
                            ++cnt_pm;
                        }
                    }
                    for (int i = IMID - 1; i >= 1; --i) {
                        int ip1 = i + 1;
                        if (WMACH_JP2[i] > R(1.001) && WMACH_JP2[ip1] > R(1.001)) {
                            R DELP = PISENT[i] - PISENT[ip1];
                            R DELTAI = om::sqrt(WMACH_JP2[i] * WMACH_JP2[i] - R(1)) / (ROREF_JP2[i] * WREF_JP2[i] * WREF_JP2[i]);
                            R DELTAIP1 = om::sqrt(WMACH_JP2[ip1] * WMACH_JP2[ip1] - R(1)) /
                                         (ROREF_JP2[ip1] * WREF_JP2[ip1] * WREF_JP2[ip1]);
                            ALPHAA[i] = ALPHAA[ip1] + FROTN * DELP * R(0.5) * (DELTAI + DELTAIP1);
                            ++cnt_pm;
                        }
                    }
                    R ROTN = ALPHAA[IM] - ALPHAA[1];
                    R SUMFP = R(0.0);
                    for (int i = 1; i <= IM; ++i) {
                        ALPHAA[i] = ALPHAA[i] - ROTN * (SUMFP - R(0.5));
                        SUMFP = SUMFP + (i <= IMM1 ? F1(FP, i) : R(0));
                    }
                }
                for (int i = 1; i <= IM; ++i) {
                    R RO_JP2 = ROISENT[i];
                    R WT_JP2 = WIS_JP2[i] * om::sin(ALPHAA[i]);
                    R VM_JP2 = WIS_JP2[i] * om::cos(ALPHAA[i]);
                    R VX_JP2 = VM_JP2 * om::cos(GAMA[i]);
                    R VR_JP2 = VM_JP2 * om::sin(GAMA[i]);
                    R VT_JP2 = WT_JP2 + UNOWJP2;
                    R V_JP2_SQ = VM_JP2 * VM_JP2 + VT_JP2 * VT_JP2;
                    R ROE_JP2 = ROISENT[i] * (CV * TISENT[i] + R(0.5) * V_JP2_SQ);
                    F3(RO, i, JP2, k) = RFMIX1 * F3(RO, i, JP2, k) + RFMIX * RO_JP2;
                    F3(ROVX, i, JP2, k) = RFMIX1 * F3(ROVX, i, JP2, k) + RFMIX * RO_JP2 * VX_JP2;
                    F3(ROVR, i, JP2, k) = RFMIX1 * F3(ROVR, i, JP2, k) + RFMIX * RO_JP2 * VR_JP2;
                    F3(RORVT, i, JP2, k) = RFMIX1 * F3(RORVT, i, JP2, k) + RFMIX * RO_JP2 * VT_JP2 * RJP2;
                    F3(ROE, i, JP2, k) = RFMIX1 * F3(ROE, i, JP2, k) + RFMIX * ROE_JP2;
                }
            }
        }
    }

    /* ================================================================== */
    /*  one LOOP iteration   multall-open-18.3.f:5000-5240 + tail 8000-    */
    /* ================================================================== */
    int step(int force_end, mgpu_monitors *mon) override {
        if (!committed) return fail(MGPU_E_STATE, "step before commit");
        cnt_dens = cnt_mach = cnt_pm = 0;
        IFPRINT = 0;
        NSTEP = NSTEP + 1;
        if (NSTEP == NSTEPS_MAX) IFEND = 1;
        if (EAVG < CONLIM && ECONT < R(0.01)) IFEND = 1;
        if (om::fabs(EMAX) < R(4) * CONLIM && ECONT < R(0.01)) IFEND = 1;
        if (force_end) IFEND = 1;

        if (!(IF_RESTART != 0 && NSTEP > 100)) {
            R FCHANGE = R(1.0) - R(NSTEP - 1) / R(NCHANGE);
            if (FCHANGE > R(0.0)) {
                SFT = SFTIN + R(0.02) * FCHANGE;
                SFX = SFXIN + R(0.02) * FCHANGE;
                DAMP = DAMPIN * (R(1.) - R(0.75) * FCHANGE);
            }
            SFT1 = R(1.0) - SFT;
            SFTH = R(0.5) * SFT;
            SFX1 = R(1.) - SFX;
            SFXH = R(0.5) * SFX;
            SFX15 = R(1.0) - R(1.5) * SFX;
            SFX14 = R(0.25) * SFX;
            SFXB = FSMTHB * SFX;
            SFXB1 = R(1.0) - SFXB;
            SFXBH = R(0.5) * SFXB;
            SFXHM1 = R(1.) - SFXH;
            FMIXUP = R(1.0) + (FACMIXUP - R(1.)) * R(NMIXUP - NSTEP) / R(NMIXUP);
            if (FMIXUP < R(1.0)) FMIXUP = R(1.0);
            FMIXUP = FMIXUP * FMIXUP;
        }
        /* primitive velocities 7450 */
        for (int k = 1; k <= KM; ++k)
            for (int j = 2; j <= JM; ++j) {
                R RRNOW = R(1) / F2(R, j, k);
                for (int i = 1; i <= IM; ++i) {
                    R RECIP = R(1.0) / F3(RO, i, j, k);
                    F3(VX, i, j, k) = F3(ROVX, i, j, k) * RECIP;
                    F3(VR, i, j, k) = F3(ROVR, i, j, k) * RECIP;
                    F3(ROVT, i, j, k) = F3(RORVT, i, j, k) * RRNOW;
                    F3(VT, i, j, k) = F3(ROVT, i, j, k) * RECIP;
                }
            }
        bool tail = (NSTEP % 5 == 0) || IFEND == 1;
        if (tail) {
            VRMS = R(0.0);
            VMAX = R(0.0);
            for (int k = 1; k <= KM; ++k)
                for (int j = 2; j <= JM; ++j)
                    for (int i = 1; i <= IM; ++i) {
                        R vr = F3(VR, i, j, k), wt = F3(WT, i, j, k), vx = F3(VX, i, j, k);
                        R EKE = vr * vr + wt * wt + vx * vx;
                        if (EKE > VMAX) {
                            VMAX = EKE;
                            IVMAX = i; JVMAX = j; KVMAX = k;
                        }
                        VRMS = VRMS + EKE;
                    }
            VMAX = om::sqrt(VMAX);
        }
        /* pressure, stagnation enthalpy, temperature 5900 */
        for (int k = 1; k <= KM; ++k)
            for (int j = 2; j <= JMM1; ++j)
                for (int i = 1; i <= IM; ++i) {
                    R RONOW = F3(RO, i, j, k);
                    R vr = F3(VR, i, j, k), vt = F3(VT, i, j, k), vx = F3(VX, i, j, k);
                    R EKE = R(.5) * (vr * vr + vt * vt + vx * vx);
                    R TSTATIC = (F3(ROE, i, j, k) / RONOW - EKE) / CV;
                    F3(P, i, j, k) = RONOW * RGAS * TSTATIC;
                    F3(HO, i, j, k) = CP * TSTATIC + EKE;
                    F3(T_STATIC, i, j, k) = TSTATIC;
                }
        if (ILOS == 10 && NSTEP % NLOS == 0 && !FROZEN) loss();
        if (ILOS >= 100 && ILOS < 200 && NSTEP % NLOS == 0 && !FROZEN) new_loss();
        if (ILOS >= 200 && NSTEP % NLOS == 0 && !FROZEN) spal_loss();
        mass_fluxes();
        tstep(RO_v, DRO_v);
        if (ILOS >= 100) roavg_cell();
        if (ILOS >= 200) sa_transport();
        energy_fluxes();
        tstep(ROE_v, DROE_v);
        boundary_conditions();
        if (IN_FLOW != 0) setflo();
        /* PEFF 4321 */
        for (int k = 1; k <= KM; ++k)
            for (int j = 1; j <= JM; ++j) {
                int jp1 = (j == JM) ? JM : j + 1;
                for (int i = 1; i <= IM; ++i)
                    F3(PEFF, i, j, k) = F3(P, i, j, k) - PREFF + F_PDOWN * (F3(P, i, jp1, k) - F3(P, i, j, k));
            }
        xmom_fluxes();
        tstep(ROVX_v, DROVX_v);
        rvt_fluxes();
        tstep(RORVT_v, DRORVT_v);
        rmom_fluxes();
        tstep(ROVR_v, DROVR_v);
        limiters();
        if (IFMIX > 0 && RFMIX > R(1.0E-3)) new_mixplan();
        cusp_separation();

        int rc = 0;
        if (mon) {
            memset(mon, 0, sizeof(*mon));
            mon->nstep = NSTEP;
        }
        if (tail) {
            int health = tail_monitors();
            if (!FROZEN) stepup(0.25);
            if (mon) {
                mon->tail_ran = 1;
                mon->emax = (float)EMAX; mon->imax = IMAXE; mon->jmax = JMAXE; mon->kmax = KMAXE;
                mon->eavg = (float)EAVG; mon->econt = (float)ECONT; mon->jcont = JCONT;
                mon->vref = (float)om::sqrt(VRMS * RIJKM);
                mon->vmax = (float)VMAX; mon->ivmax = IVMAX; mon->jvmax = JVMAX; mon->kvmax = KVMAX;
                mon->flow_in = (double)BLADE_FLOW[0];
                mon->flow_out = (double)BLADE_FLOW[JM - 1];
                mon->health = health;
            }
            if (health) rc = fail(MGPU_E_NONFINITE, "non-finite or non-positive density in the flow field");
        }
        if (mon) mon->ifend = IFEND;
        return rc;
    }

    /* mass fluxes 5020-5045 */
    void mass_fluxes() {
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 1; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    R AVGRVX = F3(ROVX, i, j, k) + F3(ROVX, i, j, k + 1) + F3(ROVX, i + 1, j, k) + F3(ROVX, i + 1, j, k + 1);
                    R AVGRVR = F3(ROVR, i, j, k) + F3(ROVR, i, j, k + 1) + F3(ROVR, i + 1, j, k) + F3(ROVR, i + 1, j, k + 1);
                    A3(FLOWX, i, j, k) = R(0.25) * (AVGRVX * F3(AQX, i, j, k) + AVGRVR * F3(AQR, i, j, k));
                    A3(SOURCE, i, j, k) = R(0.0);
                    A3(XFLUX, i, j, k) = A3(FLOWX, i, j, k);
                }
        for (int k = 1; k <= KM; ++k)
            for (int j = 1; j <= JM; ++j)
                for (int i = 1; i <= IM; ++i) {
                    F3(ROWT, i, j, k) = F3(ROVT, i, j, k) - F2(UBLADE, j, k) * F3(RO, i, j, k);
                    F3(WT, i, j, k) = F3(ROWT, i, j, k) / F3(RO, i, j, k);
                }
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IM; ++i) {
                    R AVGRVX = F3(ROVX, i, j, k) + F3(ROVX, i, j - 1, k) + F3(ROVX, i, j - 1, k + 1) + F3(ROVX, i, j, k + 1);
                    R AVGRVT = F3(ROWT, i, j, k) + F3(ROWT, i, j - 1, k) + F3(ROWT, i, j - 1, k + 1) + F3(ROWT, i, j, k + 1);
                    R AVGRVR = F3(ROVR, i, j, k) + F3(ROVR, i, j - 1, k) + F3(ROVR, i, j - 1, k + 1) + F3(ROVR, i, j, k + 1);
                    A3(FLOWT, i, j, k) = (AVGRVX * F3(ABX, i, j, k) + AVGRVT * F2(ABT, j, k) + AVGRVR * F3(ABR, i, j, k)) * R(0.25);
                    A3(TFLUX, i, j, k) = A3(FLOWT, i, j, k);
                }
        for (int j = 2; j <= JM; ++j) {
            if (F1(IND, j) == 1) continue;
            for (int k = 1; k <= KMM1; ++k) {
                R AVGFLUX = R(0.5) * (A3(FLOWT, 1, j, k) + A3(FLOWT, IM, j, k));
                A3(FLOWT, 1, j, k) = AVGFLUX;
                A3(FLOWT, IM, j, k) = AVGFLUX;
                A3(TFLUX, 1, j, k) = AVGFLUX;
                A3(TFLUX, IM, j, k) = AVGFLUX;
            }
        }
        for (int j = 2; j <= JM; ++j) {
            if (F1(IND, j) != 1) continue;
            int nr = F1(NROW, j);
            for (int k = F1(KS1, nr); k <= F1(KS2, nr); ++k) {
                A3(TFLUX, 1, j, k) = R(0.0);
                A3(TFLUX, IM, j, k) = R(0.0);
                A3(FLOWT, 1, j, k) = R(0.0);
                A3(FLOWT, IM, j, k) = R(0.0);
            }
        }
        for (int k = 2; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    R AVGRVX = F3(ROVX, i, j, k) + F3(ROVX, i, j - 1, k) + F3(ROVX, i + 1, j - 1, k) + F3(ROVX, i + 1, j, k);
                    R AVGRVR = F3(ROVR, i, j, k) + F3(ROVR, i, j - 1, k) + F3(ROVR, i + 1, j - 1, k) + F3(ROVR, i + 1, j, k);
                    A3(FLOWR, i, j, k) = R(0.25) * (AVGRVX * F3(ASX, i, j, k) + AVGRVR * F3(ASR, i, j, k));
                    A3(RFLUX, i, j, k) = A3(FLOWR, i, j, k);
                }
        for (int j = 2; j <= JM; ++j)
            for (int i = 1; i <= IMM1; ++i) {
                A3(FLOWR, i, j, 1) = R(0.0);
                A3(FLOWR, i, j, KM) = R(0.0);
                A3(RFLUX, i, j, 1) = R(0.0);
                A3(RFLUX, i, j, KM) = R(0.0);
            }
    }

    /* energy fluxes 5501-5503, 900 */
    void energy_fluxes() {
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 1; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    R AVGHO = F3(HO, i, j, k) + F3(HO, i, j, k + 1) + F3(HO, i + 1, j, k) + F3(HO, i + 1, j, k + 1);
                    A3(XFLUX, i, j, k) = A3(FLOWX, i, j, k) * AVGHO * R(0.25);
                }
        for (int j = 2; j <= JM; ++j)
            for (int k = 1; k <= KMM1; ++k)
                for (int i = 1; i <= IMM1; ++i) A3(SOURCE, i, j, k) = F3(QSOURCE, i, j, k);
        for (int k = 1; k <= KM; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    R AVGHO = R(0.25) * (F3(HO, i, j, k) + F3(HO, i, j - 1, k) + F3(HO, i + 1, j - 1, k) + F3(HO, i + 1, j, k));
                    A3(RFLUX, i, j, k) = A3(FLOWR, i, j, k) * AVGHO;
                }
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IM; ++i) {
                    R AVGHO = F3(HO, i, j, k) + F3(HO, i, j - 1, k) + F3(HO, i, j - 1, k + 1) + F3(HO, i, j, k + 1);
                    R AVGPB = F3(PEFF, i, j, k) + F3(PEFF, i, j - 1, k) + F3(PEFF, i, j - 1, k + 1) + F3(PEFF, i, j, k + 1);
                    A3(TFLUX, i, j, k) = (A3(FLOWT, i, j, k) * AVGHO + F2(WRABT, j, k) * AVGPB) * R(0.25);
                }
        periodic_tflux_avg();
    }

    void periodic_tflux_avg() {
        for (int j = 2; j <= JM; ++j) {
            if (F1(IND, j) == 1) continue;
            for (int k = 1; k <= KMM1; ++k) {
                A3(TFLUX, 1, j, k) = R(0.5) * (A3(TFLUX, 1, j, k) + A3(TFLUX, IM, j, k));
                A3(TFLUX, IM, j, k) = A3(TFLUX, 1, j, k);
            }
        }
    }

    /* inlet and exit boundary conditions 4476-4734 (ITIMST<5, IFGAS=0) */
    /* ================================================================== */
    /*  SETFLO   multall-open-18.3.f:8006-8052: relax the mass flow of     */
    /*  every J station towards FLOWIN (IN_FLOW=3) or towards the mean     */
    /*  flow (other nonzero IN_FLOW)                                        */
    /* ================================================================== */
    void setflo() {
        std::vector<R> FLOW((size_t)JM + 1, R(0));
        for (int j = 1; j <= JM; ++j) {
            FLOW[j] = R(0.0);
            for (int k = 1; k <= KMM1; ++k)
                for (int i = 1; i <= IMM1; ++i)
                    FLOW[j] = FLOW[j] - A3(FLOWX, i, j, k) * R(F1(NBLADE, j)) / R(F1(NBLADE, 1));
        }
        R AVFLOW = FLOWIN / R(F1(NBLADE, 1));
        if (IN_FLOW != 3) {
            AVFLOW = R(0.0);
            for (int j = 1; j <= JM; ++j) AVFLOW = AVFLOW + FLOW[j];
            AVFLOW = AVFLOW / R(JM);
        }
        for (int j = 1; j <= JM; ++j) {
            R a = F3(ROVX, IMID, j, KMID), b = F3(ROVR, IMID, j, KMID);
            R ROVMER = om::sqrt(a * a + b * b);
            R DELTA = (AVFLOW / FLOW[j] - R(1.0)) * ROVMER;
            DELTA = DELTA * RFLOW;
            for (int i = 1; i <= IM; ++i)
                for (int k = 1; k <= KM; ++k) {
                    R x = F3(ROVX, i, j, k), r = F3(ROVR, i, j, k);
                    R RM = om::sqrt(x * x + r * r);
                    if (x < R(0.0)) RM = -RM;
                    F3(ROVX, i, j, k) = x + x / RM * DELTA;
                    F3(ROVR, i, j, k) = r + r / RM * DELTA;
                    R RO_WT = F3(ROVT, i, j, k) - F2(UBLADE, j, k) * F3(RO, i, j, k);
                    F3(ROVT, i, j, k) = F3(ROVT, i, j, k) + RO_WT / RM * DELTA;
                }
        }
    }

    /* ================================================================== */
    /*  IF_CUSP = 2: forced trailing-edge separation, 5178-5233            */
    /* ================================================================== */
    void cusp_separation() {
        for (int nr = 1; nr <= NROWS; ++nr) {
            if (F1(IF_CUSP, nr) != 2) continue;
            int JTEDGE = F1(JTE, nr);
            int JSEP_I1 = JTEDGE - F1(NUP_I1, nr), JSEP_IM = JTEDGE - F1(NUP_IM, nr);
            int JTHIK = std::max(JSEP_I1, JSEP_IM);
            R FDRAG = F1(SEP_DRAG, nr);
            int NWKE = F1(N_WAKE, nr);
            auto force = [&](int i, int j, int k) {
                F3(ROVX, i, j, k) = FDRAG * F3(ROVX, i, j, k);
                F3(ROVR, i, j, k) = FDRAG * F3(ROVR, i, j, k);
                R RO_VBLADE = F3(RO, i, j, k) * F2(UBLADE, j, k);
                R RO_WT = F3(ROVT, i, j, k) - RO_VBLADE;
                R RO_VT = FDRAG * RO_WT + RO_VBLADE;
                F3(RORVT, i, j, k) = RO_VT * F2(R, j, k);
            };
            for (int k = 1; k <= KM; ++k) {
                R THIK_LIM = F1(SEP_THIK, nr) * F2(RT_THICK, JTHIK, k);
                R SSSLOPE = (F3(RTHETA, 1, JSEP_I1 + 1, k) - F3(RTHETA, 1, JSEP_I1 - 1, k)) /
                            (F2(X, JSEP_I1 + 1, k) - F2(X, JSEP_I1 - 1, k));
                R PSSLOPE = (F3(RTHETA, IM, JSEP_IM + 1, k) - F3(RTHETA, IM, JSEP_IM - 1, k)) /
                            (F2(X, JSEP_IM + 1, k) - F2(X, JSEP_IM - 1, k));
                for (int j = JSEP_I1; j <= JTEDGE + NWKE; ++j) {
                    R RTEXTRAP = F3(RTHETA, 1, JSEP_I1, k) + SSSLOPE * (F2(X, j, k) - F2(X, JSEP_I1, k));
                    for (int i = 1; i <= 6; ++i)
                        if ((RTEXTRAP - F3(RTHETA, i, j, k)) > THIK_LIM) force(i, j, k);
                }
                for (int j = JSEP_IM; j <= JTEDGE + NWKE; ++j) {
                    R RTEXTRAP = F3(RTHETA, IM, JSEP_IM, k) + PSSLOPE * (F2(X, j, k) - F2(X, JSEP_IM, k));
                    for (int i = IM - 6; i <= IM; ++i)
                        if ((F3(RTHETA, i, j, k) - RTEXTRAP) > THIK_LIM) force(i, j, k);
                }
            }
        }
    }

    void boundary_conditions() {
        // exit "plate loss" (4476-4484): pitchwise sums of ROV_m**2 at JM.  The
        // normalising statement after the loop runs once, with K = KM+1, so
        // the sums themselves are used below
        std::vector<R> ROVMSQ((size_t)KM + 2, R(0));
        if (PLATE_LOSS > R(0.001)) {
            for (int k = 1; k <= KM; ++k) {
                ROVMSQ[k] = R(0.0);
                for (int i = 1; i <= IM; ++i)
                    ROVMSQ[k] = ROVMSQ[k] + F3(ROVX, i, JM, k) * F3(VX, i, JM, k) + F3(ROVR, i, JM, k) * F3(VR, i, JM, k);
            }
            ROVMSQ[KM + 1] = R(0.5) * ROVMSQ[KM + 1] / R(IM);
        }
        // throttle exit condition (4488-4505)
        R PTHROTTLE = R(0.0), PDMID = R(0.0);
        if (NSTEP > 100 && THROTTLE_EXIT > R(0.001)) {
            R FFLOW = CHECK_FLOW[JM - 1] / THROTTLE_MAS;
            PTHROTTLE = THROTTLE_PRES * FFLOW * FFLOW;
            PDOWN_TIP = RFTHROTL1 * PDOWN_TIP + RFTHROTL * PTHROTTLE;
            PDOWN_HUB = RFTHROTL1 * PDOWN_HUB + RFTHROTL * PTHROTTLE;
            PDMID = PTHROTTLE - F1(PD, KMID);
            R RF_P = R(0.02) * RFTHROTL;
            THROTTLE_PRES = (R(1.) - RF_P) * THROTTLE_PRES + RF_P * PTHROTTLE;
        }
        R PDIFF = R(0.0);
        if (IPOUT == -1) PDIFF = PDOWN_TIP - F1(PD, KM);
        R SUMP = R(0);
        for (int k = 1; k <= KM; ++k) {
            R PAVG2 = R(0.0), PAVG3 = R(0.0), PAVGOUT = R(0.0), SUM = R(0.0);
            for (int i = 1; i <= IMM1; ++i) {
                PAVG2 = PAVG2 + R(0.5) * (F3(P, i, 2, k) + F3(P, i + 1, 2, k)) * F1(FP, i);
                PAVG3 = PAVG3 + R(0.5) * (F3(P, i, 3, k) + F3(P, i + 1, 3, k)) * F1(FP, i);
                PAVGOUT = PAVGOUT + R(0.5) * (F3(P, i, JMM1, k) + F3(P, i + 1, JMM1, k)) * F1(FP, i);
                SUM = SUM + R(0.5) * F1(FP, i) *
                                (F3(ROVT, i, JM, k) * F3(VT, i, JM, k) + F3(ROVT, i + 1, JM, k) * F3(VT, i + 1, JM, k)) /
                                F2(R, JM, k);
            }
            if (IPOUT <= 0) {
                F1(PD, 1) = PDOWN_HUB;
                if (k != 1) {
                    R DP = (SUM + SUMP) * R(0.5) * (F2(R, JM, k) - F2(R, JM, k - 1));
                    F1(PD, k) = R(0.9) * F1(PD, k) + R(0.1) * (F1(PD, k - 1) + DP);
                }
                SUMP = SUM;
                if (IPOUT == -1) F1(PD, k) = F1(PD, k) + PDIFF;
            }
            if (IPOUT >= 1 && THROTTLE_EXIT > R(0.001)) F1(PD, k) = F1(PD, k) + RFTHROTL * PDMID;
            if (PLATE_LOSS > R(0.001)) F1(PD, k) = F1(PD, k) + R(0.01) * PLATE_LOSS * (ROVMSQ[k] - ROVMSQ[KMID]);
            for (int i = 1; i <= IM; ++i) {
                R RO_STAG = F1(PO1, k) / RGAS / F1(TO1, k);
                R RO_IN = F3(RO, i, 1, k);
                if (RO_IN > R(0.9999) * RO_STAG) RO_IN = R(0.9999) * RO_STAG;
                R PNEW = F1(PO1, k) * om::pow(RO_IN / RO_STAG, GA);
                if (IN_PRESS == 0) F3(P, i, 1, k) = RFIN1 * F3(P, i, 1, k) + RFIN * PNEW;
                if (std::abs(IN_PRESS) == 1)
                    F3(P, i, 1, k) = RFIN1 * F3(P, i, 1, k) + RFIN2 * F3(P, i, 2, k) - RFIN * F3(P, i, 3, k);
                if (std::abs(IN_PRESS) == 3) F3(P, i, 1, k) = RFIN1 * F3(P, i, 1, k) + RFIN2 * PAVG2 - RFIN * PAVG3;
                if (std::abs(IN_PRESS) == 4)
                    F3(P, i, 1, k) = RFIN1 * F3(P, i, 1, k) + RFIN2 * F3(P, IMID, 2, KMID) - RFIN * F3(P, IMID, 3, KMID);
                if (F3(P, i, 1, k) > PLIM[k - 1]) F3(P, i, 1, k) = R(0.9) * F3(P, i, 1, k) + R(0.1) * PLIM[k - 1];
                if (F3(P, i, 1, k) > R(0.99999) * F1(PO1, k)) F3(P, i, 1, k) = F1(PO1, k) * R(0.99999);
                R TSTATIC = F1(TO1, k) * om::pow(F3(P, i, 1, k) * F1(RPO1, k), FGA);
                R VABSQ = R(2) * CP * (F1(TO1, k) - TSTATIC);
                F3(T_STATIC, i, 1, k) = TSTATIC;
                R VABS = om::sqrt(VABSQ);
                R VMER = R(0);
                if (IN_VTAN == 0) {
                    VMER = VABS * F1(BSCOS, k);
                    F3(VT, i, 1, k) = VABS * F1(BSSIN, k);
                }
                if (IN_VTAN == 1) {
                    R VMERSQ = VABSQ - F1(VTIN, k) * F1(VTIN, k);
                    if (VMERSQ < R(0.01)) VMERSQ = R(0.01);
                    VMER = om::sqrt(VMERSQ);
                    F3(VT, i, 1, k) = F1(VTIN, k);
                }
                if (IN_VTAN == 2) {
                    R WR = F2(UBLADE, 1, k);
                    R VRELSQ = VABSQ - WR * WR * F1(BSCOS, k) * F1(BSCOS, k);
                    if (VRELSQ < R(0.01)) VRELSQ = R(0.01);
                    R VREL = om::sqrt(VRELSQ) - WR * F1(BSSIN, k);
                    VMER = VREL * F1(BSCOS, k);
                    F3(VT, i, 1, k) = VREL * F1(BSSIN, k) + WR;
                }
                if (IN_VR > 0) F3(VX, i, 1, k) = VMER * F1(BRCOS, k);
                R VXSQ = VMER * VMER - F3(VR, i, 2, k) * F3(VR, i, 2, k);
                if (VXSQ < R(0.0000001) * F1(TO1, k) * CP) VXSQ = R(0.0000001) * F1(TO1, k) * CP;
                if (IN_VR <= 0) F3(VX, i, 1, k) = om::sqrt(VXSQ);
                if (IN_VR > 0) F3(VR, i, 1, k) = VMER * F1(BRSIN, k);
                if (IN_VR <= 0) F3(VR, i, 1, k) = F3(VR, i, 2, k);
                F3(RO, i, 1, k) = F3(P, i, 1, k) / (RGAS * TSTATIC);
                F3(ROVT, i, 1, k) = F3(RO, i, 1, k) * F3(VT, i, 1, k);
                F3(ROVR, i, 1, k) = F3(RO, i, 1, k) * F3(VR, i, 1, k);
                F3(RORVT, i, 1, k) = F3(ROVT, i, 1, k) * F2(R, 1, k);
                F3(ROVX, i, 1, k) = F3(RO, i, 1, k) * F3(VX, i, 1, k);
                F3(ROE, i, 1, k) = F3(P, i, 1, k) / GA1 + F3(RO, i, 1, k) * R(0.5) * VABSQ;
                F3(HO, i, 1, k) = CP * F1(TO1, k);
                if (ILOS >= 200) {
                    /* the transported viscosity at inlet (4679-4689); RO(IMID,1,KMID)
                       is the value this K, I loop has reached */
                    F3(TRANS_DYN_VIS, i, 1, k) = sa_transvis_in(F3(VISC_LAM, i, 2, k));
                    F3(TRANS_DYN_VIS, i, 2, k) = F3(TRANS_DYN_VIS, i, 1, k);
                    F3(TRANS_KVIS, i, 1, k) = F3(TRANS_DYN_VIS, i, 1, k) / F3(RO, IMID, 1, KMID);
                    F3(TRANS_KVIS, i, 2, k) = F3(TRANS_KVIS, i, 1, k);
                }
                /* exit */
                R vr = F3(VR, i, JM, k), vt = F3(VT, i, JM, k), vx = F3(VX, i, JM, k);
                R EKE = R(.5) * (vr * vr + vt * vt + vx * vx);
                F3(P, i, JM, k) = F1(PD, k) + FEXTRAP * (F3(P, i, JMM1, k) - PAVGOUT);
                F3(HO, i, JM, k) = R(2.0) * F3(HO, i, JMM1, k) - F3(HO, i, JM - 2, k);
                R TEXIT = (F3(HO, i, JM, k) - EKE) / CP;
                F3(RO, i, JM, k) = F3(P, i, JM, k) / RGAS / TEXIT;
                F3(ROE, i, JM, k) = F3(RO, i, JM, k) * (CV * TEXIT + EKE);
            }
        }
    }

    /* axial momentum fluxes 6100-6120, 6026 */
    void xmom_fluxes() {
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 1; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    A3(SOURCE, i, j, k) = F3(XFORCE, i, j, k);
                    R AVGP = F3(PEFF, i, j, k) + F3(PEFF, i, j, k + 1) + F3(PEFF, i + 1, j, k + 1) + F3(PEFF, i + 1, j, k);
                    R AVGVX = F3(VX, i, j, k) + F3(VX, i, j, k + 1) + F3(VX, i + 1, j, k + 1) + F3(VX, i + 1, j, k);
                    A3(XFLUX, i, j, k) = R(0.25) * (AVGP * F3(AQX, i, j, k) + A3(FLOWX, i, j, k) * AVGVX);
                }
        for (int k = 1; k <= KM; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    R AVGP = F3(PEFF, i, j, k) + F3(PEFF, i, j - 1, k) + F3(PEFF, i + 1, j - 1, k) + F3(PEFF, i + 1, j, k);
                    R AVGVX = F3(VX, i, j, k) + F3(VX, i, j - 1, k) + F3(VX, i + 1, j - 1, k) + F3(VX, i + 1, j, k);
                    A3(RFLUX, i, j, k) = R(0.25) * (AVGP * F3(ASX, i, j, k) + A3(FLOWR, i, j, k) * AVGVX);
                }
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IM; ++i) {
                    R AVGVX = F3(VX, i, j, k) + F3(VX, i, j - 1, k) + F3(VX, i, j - 1, k + 1) + F3(VX, i, j, k + 1);
                    R AVGP = F3(PEFF, i, j, k) + F3(PEFF, i, j - 1, k) + F3(PEFF, i, j - 1, k + 1) + F3(PEFF, i, j, k + 1);
                    A3(TFLUX, i, j, k) = R(0.25) * (A3(FLOWT, i, j, k) * AVGVX + F3(ABX, i, j, k) * AVGP);
                }
        for (int j = 2; j <= JM; ++j) {
            if (F1(IND, j) == 1) continue;
            for (int k = 1; k <= KMM1; ++k) {
                R AVGPCUSP = F3(PEFF, 1, j, k) + F3(PEFF, 1, j - 1, k) + F3(PEFF, 1, j, k + 1) + F3(PEFF, 1, j - 1, k + 1) +
                             F3(PEFF, IM, j, k) + F3(PEFF, IM, j - 1, k) + F3(PEFF, IM, j, k + 1) + F3(PEFF, IM, j - 1, k + 1);
                R AVGVXCUSP = F3(VX, 1, j, k) + F3(VX, 1, j - 1, k) + F3(VX, 1, j, k + 1) + F3(VX, 1, j - 1, k + 1) +
                              F3(VX, IM, j, k) + F3(VX, IM, j - 1, k) + F3(VX, IM, j, k + 1) + F3(VX, IM, j - 1, k + 1);
                A3(TFLUX, 1, j, k) = R(0.125) * (A3(FLOWT, 1, j, k) * AVGVXCUSP + AVGPCUSP * F3(ABX, 1, j, k));
                A3(TFLUX, IM, j, k) = R(0.125) * (A3(FLOWT, IM, j, k) * AVGVXCUSP + AVGPCUSP * F3(ABX, IM, j, k));
            }
        }
    }

    /* moment-of-momentum fluxes 6200-6230, 902 */
    void rvt_fluxes() {
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 1; j <= JM; ++j) {
                R AVGR = R(0.125) * (F2(R, j, k) + F2(R, j, k + 1));
                for (int i = 1; i <= IMM1; ++i) {
                    R AVGVT = F3(VT, i, j, k) + F3(VT, i, j, k + 1) + F3(VT, i + 1, j, k) + F3(VT, i + 1, j, k + 1);
                    A3(SOURCE, i, j, k) = F3(TFORCE, i, j, k);
                    A3(XFLUX, i, j, k) = A3(FLOWX, i, j, k) * AVGR * AVGVT;
                }
            }
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j) {
                R AVGR = R(0.25) * F2(RAVG_CELL, j, k);
                for (int i = 1; i <= IM; ++i) {
                    R AVGVT = F3(VT, i, j, k) + F3(VT, i, j - 1, k) + F3(VT, i, j - 1, k + 1) + F3(VT, i, j, k + 1);
                    R AVGP = F3(PEFF, i, j, k) + F3(PEFF, i, j - 1, k) + F3(PEFF, i, j - 1, k + 1) + F3(PEFF, i, j, k + 1);
                    A3(TFLUX, i, j, k) = (A3(FLOWT, i, j, k) * AVGVT + F2(ABT, j, k) * AVGP) * AVGR;
                }
            }
        for (int k = 1; k <= KM; ++k)
            for (int j = 2; j <= JM; ++j) {
                R AVGR = (F2(R, j, k) + F2(R, j - 1, k)) * R(0.125);
                for (int i = 1; i <= IMM1; ++i) {
                    R AVGVT = F3(VT, i, j, k) + F3(VT, i, j - 1, k) + F3(VT, i + 1, j - 1, k) + F3(VT, i + 1, j, k);
                    A3(RFLUX, i, j, k) = A3(FLOWR, i, j, k) * AVGVT * AVGR;
                }
            }
        periodic_tflux_avg();
    }

    /* radial momentum fluxes and source 6300-6330, 6260 */
    void rmom_fluxes() {
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 1; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    R AVGVR = F3(VR, i, j, k) + F3(VR, i, j, k + 1) + F3(VR, i + 1, j, k) + F3(VR, i + 1, j, k + 1);
                    R AVGP = F3(PEFF, i, j, k) + F3(PEFF, i, j, k + 1) + F3(PEFF, i + 1, j, k + 1) + F3(PEFF, i + 1, j, k);
                    A3(XFLUX, i, j, k) = R(0.25) * (A3(FLOWX, i, j, k) * AVGVR + F3(AQR, i, j, k) * AVGP);
                }
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IM; ++i) {
                    R AVGVR = F3(VR, i, j, k) + F3(VR, i, j - 1, k) + F3(VR, i, j - 1, k + 1) + F3(VR, i, j, k + 1);
                    R AVGP = F3(PEFF, i, j, k) + F3(PEFF, i, j - 1, k) + F3(PEFF, i, j - 1, k + 1) + F3(PEFF, i, j, k + 1);
                    A3(TFLUX, i, j, k) = R(.25) * (A3(FLOWT, i, j, k) * AVGVR + AVGP * F3(ABR, i, j, k));
                }
        for (int k = 1; k <= KM; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    R AVGVR = F3(VR, i, j, k) + F3(VR, i, j - 1, k) + F3(VR, i + 1, j - 1, k) + F3(VR, i + 1, j, k);
                    R AVGP = F3(PEFF, i, j, k) + F3(PEFF, i, j - 1, k) + F3(PEFF, i + 1, j - 1, k) + F3(PEFF, i + 1, j, k);
                    A3(RFLUX, i, j, k) = R(0.25) * (A3(FLOWR, i, j, k) * AVGVR + F3(ASR, i, j, k) * AVGP);
                }
        for (int k = 1; k <= KMM1; ++k)
            for (int j = 2; j <= JM; ++j)
                for (int i = 1; i <= IMM1; ++i) {
                    R AVGRVT = F3(ROVT, i, j, k) + F3(ROVT, i, j, k + 1) + F3(ROVT, i, j - 1, k) + F3(ROVT, i, j - 1, k + 1) +
                               F3(ROVT, i + 1, j, k) + F3(ROVT, i + 1, j, k + 1) + F3(ROVT, i + 1, j - 1, k) +
                               F3(ROVT, i + 1, j - 1, k + 1);
                    R AVGVT = R(0.125) * (F3(VT, i, j, k) + F3(VT, i, j - 1, k) + F3(VT, i, j - 1, k + 1) + F3(VT, i, j, k + 1) +
                                          F3(VT, i + 1, j, k) + F3(VT, i + 1, j - 1, k) + F3(VT, i + 1, j - 1, k + 1) +
                                          F3(VT, i + 1, j, k + 1));
                    R AVGP = F3(PEFF, i, j, k) + F3(PEFF, i, j - 1, k) + F3(PEFF, i, j - 1, k + 1) + F3(PEFF, i, j, k + 1) +
                             F3(PEFF, i + 1, j, k) + F3(PEFF, i + 1, j - 1, k) + F3(PEFF, i + 1, j - 1, k + 1) +
                             F3(PEFF, i + 1, j, k + 1);
                    A3(SOURCE, i, j, k) = F3(RFORCE, i, j, k) - (AVGRVT * AVGVT + AVGP) * F3(VOLOR, i, j, k);
                }
        for (int j = 2; j <= JM; ++j) {
            if (F1(IND, j) == 1) continue;
            for (int k = 1; k <= KMM1; ++k) {
                R AVGP1 = R(0.25) * (F3(PEFF, 1, j, k) + F3(PEFF, 1, j - 1, k) + F3(PEFF, 1, j, k + 1) + F3(PEFF, 1, j - 1, k + 1));
                R AVGPM = R(0.25) * (F3(PEFF, IM, j, k) + F3(PEFF, IM, j - 1, k) + F3(PEFF, IM, j, k + 1) +
                                     F3(PEFF, IM, j - 1, k + 1));
                R T1 = A3(TFLUX, 1, j, k) - AVGP1 * F3(ABR, 1, j, k);
                R T2 = A3(TFLUX, IM, j, k) - AVGPM * F3(ABR, IM, j, k);
                A3(TFLUX, 1, j, k) = R(0.5) * ((T1 + T2) + (AVGP1 + AVGPM) * F3(ABR, 1, j, k));
                A3(TFLUX, IM, j, k) = R(0.5) * ((T1 + T2) + (AVGP1 + AVGPM) * F3(ABR, IM, j, k));
            }
        }
    }

    /* density and Mach-number limiters 7200, 7250, 7100 */
    void limiters() {
        for (int k = 1; k <= KM; ++k)
            for (int j = 3; j <= JM - 3; ++j)
                for (int i = 1; i <= IM; ++i) {
                    R ROAVG = R(0.25) * (F3(RO, i, j - 2, k) + F3(RO, i, j - 1, k) + F3(RO, i, j + 1, k) + F3(RO, i, j + 2, k));
                    const R before = F3(RO, i, j, k);
                    if (F3(RO, i, j, k) < R(0.6) * ROAVG) F3(RO, i, j, k) = R(0.5) * (F3(RO, i, j, k) + R(0.6) * ROAVG);
                    if (F3(RO, i, j, k) > R(1.5) * ROAVG) F3(RO, i, j, k) = R(0.5) * (F3(RO, i, j, k) + R(1.5) * ROAVG);
                    if (F3(RO, i, j, k) < ROLIM) F3(RO, i, j, k) = R(0.5) * (F3(RO, i, j, k) + ROLIM);
                    if (!(F3(RO, i, j, k) == before)) ++cnt_dens;
                }
        R GM1 = GA - R(1.0);
        R TRATIO = R(1.0) + MACHLIM * MACHLIM * R(0.5) * GM1;
        R RFGM1 = R(1.0) / GM1;
        R RORATIO = om::pow(TRATIO, RFGM1);
        for (int nr = 1; nr <= NROWS; ++nr) {
            int JREF = F1(JLE, nr);
            R TREFL = F3(T_STATIC, IMID, JREF, KMID);
            R vx = F3(VX, IMID, JREF, KMID), vr = F3(VR, IMID, JREF, KMID), wt = F3(WT, IMID, JREF, KMID);
            R WREFSQ = vx * vx + vr * vr + wt * wt;
            R TOREL_REF = TREFL + R(0.5) * WREFSQ / CP;
            R TLIMIT = TOREL_REF / TRATIO;
            if (TLIMIT > TCOOL_MIN) TLIMIT = TCOOL_MIN;
            VLIMIT[nr - 1] = om::sqrt(R(2) * CP * (TOREL_REF - TLIMIT));
            R ROSTAG_REL = F3(RO, IMID, JREF, KMID) * om::pow(TOREL_REF / TREFL, RFGM1);
            ROLIMIT[nr - 1] = ROSTAG_REL / RORATIO;
        }
        for (int k = 1; k <= KM; ++k)
            for (int j = 1; j <= JM; ++j) {
                int nr = F1(NROW, j);
                R V_LIMIT = VLIMIT[nr - 1], RO_LIMIT = ROLIMIT[nr - 1];
                for (int i = 1; i <= IM; ++i) {
                    if (F3(RO, i, j, k) < RO_LIMIT) {
                        F3(RO, i, j, k) = RO_LIMIT;
                        ++cnt_mach;
                    }
                    R RONOW = F3(RO, i, j, k);
                    R vx = F3(VX, i, j, k), vr = F3(VR, i, j, k), wt = F3(WT, i, j, k);
                    R WRELSQ = vx * vx + vr * vr + wt * wt;
                    R WREL = om::sqrt(WRELSQ);
                    R FACSAFE = V_LIMIT / WREL;
                    if (FACSAFE < R(1.0)) {
                        ++cnt_mach;
                        F3(ROVX, i, j, k) = RONOW * vx * FACSAFE;
                        F3(ROVR, i, j, k) = RONOW * vr * FACSAFE;
                        R ROVTREL = RONOW * wt * FACSAFE;
                        F3(ROWT, i, j, k) = ROVTREL;
                        F3(ROVT, i, j, k) = ROVTREL + RONOW * F2(UBLADE, j, k);
                        F3(RORVT, i, j, k) = F3(ROVT, i, j, k) * F2(R, j, k);
                    }
                }
            }
    }

    /* every-5-step monitors 5264-5317; returns the health count */
    int tail_monitors() {
        for (int j = 1; j <= JM; ++j) {
            R SUMAS = R(0);
            int NB = F1(NBLADE, j);
            for (int i = 1; i <= IMM1; ++i)
                for (int k = 1; k <= KMM1; ++k) SUMAS = SUMAS - A3(FLOWX, i, j, k);
            BLADE_FLOW[j - 1] = SUMAS * R(NB);
            CHECK_FLOW[j - 1] = SUMAS * R(NB);
        }
        ECONT = R(0.0);
        for (int j = 1; j <= JM; ++j) {
            R RATIO = CHECK_FLOW[j - 1] / CHECK_FLOW[0];
            R EMASS = om::fabs(R(1.) - RATIO);
            if (EMASS > ECONT) {
                ECONT = EMASS;
                JCONT = j;
            }
        }
        EMAX = R(0.0);
        EAVG = R(0.0);
        R VREF = om::sqrt(VRMS * RIJKM);
        R RVEF = R(100.) / VREF;
        for (int k = 1; k <= KM; ++k)
            for (int j = 2; j <= JM; ++j) {
                R XD = F2(DX, j, k), RD = F2(DR, j, k), SD = F2(DS, j, k);
                for (int i = 1; i <= IM; ++i) {
                    R VM_START = (XD * F3(VX, i, j, k) + RD * F3(VR, i, j, k)) / SD;
                    R VM_END = (XD * F3(ROVX, i, j, k) + RD * F3(ROVR, i, j, k)) / SD / F3(RO, i, j, k);
                    R DVMER = (VM_END - VM_START) * RVEF;
                    A3(STORE, i, j, k) = DVMER;
                    EAVG = EAVG + om::fabs(DVMER);
                    if (om::fabs(DVMER) > om::fabs(EMAX)) {
                        EMAX = DVMER;
                        IMAXE = i; JMAXE = j; KMAXE = k;
                    }
                }
            }
        EAVG = EAVG / R(IM * JMM1 * KM);
        int bad = 0;
        size_t n3 = (size_t)IM * JM * KM;
        for (size_t q = 0; q < n3; ++q) {
            R ro = RO_v[q];
            if (!om::isfinite(ro) || !(ro > R(0)) || !om::isfinite(ROE_v[q]) || !om::isfinite(ROVX_v[q]) ||
                !om::isfinite(ROVR_v[q]) || !om::isfinite(RORVT_v[q]))
                ++bad;
        }
        return bad;
    }

    /* EFICOOL (IFCOOL=0) with SUMFLX: whole-machine efficiency */
    /* a REAL array from double values (finite-difference checks) */
    int set_array_f64(const char *n, const double *p, int64_t cnt) override {
        std::vector<R> *a = float_array(n);
        if (!a) return fail(MGPU_E_ARG, std::string("unknown array ") + n);
        if ((int64_t)a->size() != cnt) return fail(MGPU_E_ARG, std::string("size mismatch for ") + n);
        for (size_t q = 0; q < a->size(); ++q) (*a)[q] = R(p[q]);
        return 0;
    }
    /* ---- reverse mode ------------------------------------------------ */
    static constexpr bool is_ad = std::is_same<R, adt::AD>::value;
    adt::Tape tape_;
    std::vector<std::pair<std::string, std::vector<int32_t>>> ad_in_;
#define O_FA_INT32(nm)
#define O_FA_FLOAT32(nm) if (!strcmp(n, #nm)) return &nm##_v;
#define O_FA(nm, t, s, r) O_FA_##t(nm)
    std::vector<R> *float_array(const char *n) {
        MGPU_ARRAYS(O_FA)
        return nullptr;
    }
    int ad_begin() override {
        if constexpr (!is_ad) {
            return fail(MGPU_E_STATE, "not a differentiating oracle");
        } else {
            if (!committed) return fail(MGPU_E_STATE, "ad_begin before commit");
            tape_.clear();
            ad_in_.clear();
            adt::tape() = &tape_;
#define O_REG_INT32(nm)
#define O_REG_FLOAT32(nm)                                                   \
    {                                                                       \
        std::vector<int32_t> ids;                                           \
        for (auto &x : nm##_v) {                                            \
            x = adt::independent(x.v);                                      \
            ids.push_back(x.i);                                             \
        }                                                                   \
        ad_in_.emplace_back(#nm, std::move(ids));                           \
    }
#define O_REG(nm, t, s, r) O_REG_##t(nm)
            MGPU_ARRAYS(O_REG)
            return 0;
        }
    }
    int ad_zero() override {
        if constexpr (!is_ad) return fail(MGPU_E_STATE, "not a differentiating oracle");
        adt::tape() = nullptr;
        tape_.adj.assign(tape_.size(), 0.0);
        return 0;
    }
    int ad_seed(const char *n, const double *w, int64_t cnt) override {
        if constexpr (!is_ad) {
            return fail(MGPU_E_STATE, "not a differentiating oracle");
        } else {
            std::vector<R> *a = float_array(n);
            if (!a) return fail(MGPU_E_ARG, std::string("unknown array ") + n);
            if ((int64_t)a->size() != cnt) return fail(MGPU_E_ARG, std::string("size mismatch for ") + n);
            if (tape_.adj.size() != tape_.size()) ad_zero();
            for (size_t q = 0; q < a->size(); ++q)
                if ((*a)[q].i >= 0) tape_.adj[(size_t)(*a)[q].i] += w[q];
            return 0;
        }
    }
    int ad_reverse() override {
        if constexpr (!is_ad) return fail(MGPU_E_STATE, "not a differentiating oracle");
        if (tape_.adj.size() != tape_.size()) ad_zero();
        tape_.reverse();
        return 0;
    }
    int ad_grad(const char *n, double *out, int64_t cnt) override {
        if constexpr (!is_ad) return fail(MGPU_E_STATE, "not a differentiating oracle");
        for (auto &e : ad_in_)
            if (e.first == n) {
                if ((int64_t)e.second.size() != cnt) return fail(MGPU_E_ARG, std::string("size mismatch for ") + n);
                for (size_t q = 0; q < e.second.size(); ++q)
                    out[q] = (e.second[q] >= 0 && (size_t)e.second[q] < tape_.adj.size()) ? tape_.adj[(size_t)e.second[q]] : 0.0;
                return 0;
            }
        return fail(MGPU_E_ARG, std::string("array not registered: ") + n);
    }
    int64_t ad_tape_size() override { return (int64_t)tape_.size(); }

    /* EFICOOL's mass averages per J station (10662-10849, IFCOOL = 0) */
    void per_j_sums(std::vector<R> &BF, std::vector<R> &SPO, std::vector<R> &STO, std::vector<R> &SPS) {
        size_t n3 = (size_t)IM * JM * KM;
        std::vector<R> ST2(n3), T1(n3), T2(n3), T3(n3), T4(n3);
        R TO1M = F1(TO1, KMID), PO1M = F1(PO1, KMID);
        for (int k = 1; k <= KM; ++k)
            for (int j = 1; j <= JM; ++j)
                for (int i = 1; i <= IM; ++i) {
                    R vx = F3(VX, i, j, k), vt = F3(VT, i, j, k), vr = F3(VR, i, j, k);
                    R EKE = R(0.5) * (vx * vx + vt * vt + vr * vr);
                    R TS = (F3(HO, i, j, k) - EKE) * RCP;
                    R TSTAG = F3(HO, i, j, k) * RCP;
                    if (TSTAG < R(0.1) * TO1M) TSTAG = R(0.1) * TO1M;
                    if (TS < R(0.1) * TO1M) TS = R(0.1) * TO1M;
                    R PSTAT = F3(P, i, j, k);
                    if (PSTAT < R(0.02) * PO1M) PSTAT = R(0.02) * PO1M;
                    R PSTAG = PSTAT * om::pow(TSTAG / TS, RFGA);
                    R TRAT = TS / TO1M, PRAT = PSTAT / PO1M;
                    R ENTRPY = R(0.0);
                    bool skip = (PRAT > R(0.99999) && PRAT < R(1.00001)) || (TRAT > R(0.99999) && TRAT < R(1.00001));
                    if (!skip) ENTRPY = CP * om::log(TRAT) - RGAS * om::log(PRAT);
                    A3(ST2, i, j, k) = TS;
                    A3(T1, i, j, k) = TSTAG;
                    A3(T2, i, j, k) = PSTAG / PO1M;
                    A3(T3, i, j, k) = F3(RORVT, i, j, k) / F3(RO, i, j, k);
                    A3(T4, i, j, k) = ENTRPY;
                }
        BF.assign(JM, R(0)); SPO.assign(JM, R(0)); STO.assign(JM, R(0)); SPS.assign(JM, R(0));
        for (int j = 1; j <= JM; ++j) {
            R bf = 0, spo = 0, sto = 0, sps = 0;
            for (int k = 1; k <= KMM1; ++k)
                for (int i = 1; i <= IMM1; ++i) {
                    R DFLOW = -A3(FLOWX, i, j, k) * R(F1(NBLADE, j));
                    bf = bf + DFLOW;
                    R DFLOW4 = R(0.25) * DFLOW;
                    spo = spo + DFLOW4 * (A3(T2, i, j, k) + A3(T2, i + 1, j, k) + A3(T2, i + 1, j, k + 1) + A3(T2, i, j, k + 1));
                    sto = sto + DFLOW4 * (A3(T1, i, j, k) + A3(T1, i + 1, j, k) + A3(T1, i + 1, j, k + 1) + A3(T1, i, j, k + 1));
                    sps = sps + DFLOW4 * (F3(P, i, j, k) + F3(P, i + 1, j, k) + F3(P, i + 1, j, k + 1) + F3(P, i, j, k + 1));
                }
            BF[j - 1] = bf;
            SPO[j - 1] = spo / bf;
            STO[j - 1] = sto / bf;
            SPS[j - 1] = sps / bf;
        }
    }

    /* EFICOOL's stage table (11253-11420, IFCOOL = 0) with the stations of
       the reader's JSTG_START / JSTG_END (1522-1536) */
    int stage_performance(int nstg, mgpu_stage *out) override {
        if (!committed) return fail(MGPU_E_STATE, "stage performance before commit");
        if (!NSTAGE_set) return fail(MGPU_E_STATE, "bind the row array NSTAGE for the stage table");
        const int NSTGP1 = NSTAGES == 1 ? 1 : NSTAGES + 1;
        if (nstg < 1 || nstg > NSTGP1) return fail(MGPU_E_ARG, "stage number out of range");
        std::vector<int> JSTG_START(NSTAGES + 2, 0), JSTG_END(NSTAGES + 2, 0);
        JSTG_START[1] = 1;
        for (int n = 1; n <= NROWS; ++n) {
            const int s0 = NSTAGE_v[n - 1], s1 = n < NROWS ? NSTAGE_v[n] : NSTAGES + 1;
            if (s0 != s1) {
                JSTG_END[s0] = JMIX_v[n - 1];
                if (s1 <= NSTAGES) JSTG_START[s1] = JSTART_v[n];
            }
        }
        const bool whole = NSTGP1 > 1 && nstg == NSTGP1;
        int J1, J2, J2M1, JMS;
        if (!whole) {
            J1 = JSTG_START[nstg];
            J2 = JSTG_END[nstg] + 1;
            J2M1 = nstg == NSTAGES ? JM - 1 : J2;
            JMS = JMIX_v[NROW_v[J1] - 1];
        } else {
            J1 = 2; J2 = JM; J2M1 = JM - 1; JMS = (J1 + J2) / 2;
        }
        out->j1 = J1; out->j2m1 = J2M1; out->jmix = JMS; out->has_reaction = !whole;
        out->reac_hub = out->reac_mid = out->reac_tip = 0.0;
        if (!whole) {
            const int KM2 = KM / 2;
            auto pline = [&](int j, int k) {
                R s = R(0);
                for (int i = 1; i <= IMM1; ++i) s = s + R(0.5) * (F3(P, i, j, k) + F3(P, i + 1, j, k)) * F1(FP, i);
                return s;
            };
            const int ks[3] = {1, KM2, KM};
            const R pmi = pline(J1, KM2), pmo = pline(J2M1, KM2);
            double rr[3];
            for (int q = 0; q < 3; ++q) {
                R r = (pline(JMS, ks[q]) - pline(J2M1, ks[q])) / (pline(J1, ks[q]) - pline(J2M1, ks[q]));
                if (pmo > pmi) r = R(1.0) - r;
                rr[q] = (double)r;
            }
            out->reac_hub = rr[0]; out->reac_mid = rr[1]; out->reac_tip = rr[2];
        }
        std::vector<R> BF, SPO, STO, SPS;
        per_j_sums(BF, SPO, STO, SPS);
        const R PO1M = F1(PO1, KMID);
        R POIN = SPO[J1 - 1] * PO1M, PO2 = SPO[J2M1 - 1] * PO1M, PSOUT = SPS[J2M1 - 1];
        R TO_IN = STO[J1 - 1], TO_OUT = STO[J2M1 - 1];
        R TORAT = TO_OUT / TO_IN, DELTO = TO_OUT - TO_IN, PORAT = PO2 / POIN, PSRAT = PSOUT / POIN;
        if (PORAT < R(0.01)) PORAT = R(0.01);
        R TO2IS = om::pow(PORAT, FGA) * TO_IN, TSTAT2_IS = om::pow(PSRAT, FGA) * TO_IN;
        R DELTOIS = TO2IS - TO_IN, DELT_TOT_STAT = TSTAT2_IS - TO_IN;
        R ETAIS = R(1.0), ETATS = R(1.0);
        if (DELTO > R(0.0)) { ETAIS = DELTOIS / DELTO; ETATS = DELT_TOT_STAT / DELTO; }
        if (DELTO < R(0.0)) { ETAIS = DELTO / DELTOIS; ETATS = DELTO / DELT_TOT_STAT; }
        R EPOLY = om::log(TORAT) / om::log(PORAT) / FGA;
        if (TORAT > R(1.0)) EPOLY = R(1.0) / EPOLY;
        out->mass_flow_in = (double)BF[J1 - 1];
        out->mass_flow_out = (double)BF[J2M1 - 1];
        out->po_ratio = (double)PORAT; out->to_ratio = (double)TORAT; out->delta_to = (double)DELTO;
        out->eta_tt = (double)ETAIS; out->eta_ts = (double)ETATS; out->eta_poly = (double)EPOLY;
        return 0;
    }

    int integrals(mgpu_integrals *out) override {
        if (!committed) return fail(MGPU_E_STATE, "integrals before commit");
        std::vector<R> BF, SPO, STO, SPS;
        per_j_sums(BF, SPO, STO, SPS);
        R PO1M = F1(PO1, KMID);
        int J1, J2M1;
        if (NSTAGES == 1) { J1 = 1; J2M1 = JM - 1; }
        else { J1 = 2; J2M1 = JM - 1; }
        R POIN = SPO[J1 - 1] * PO1M, PO2 = SPO[J2M1 - 1] * PO1M;
        R PSOUT = SPS[J2M1 - 1];
        R TO_IN = STO[J1 - 1], TO_OUT = STO[J2M1 - 1];
        R TORAT = TO_OUT / TO_IN, DELTO = TO_OUT - TO_IN, PORAT = PO2 / POIN, PSRAT = PSOUT / POIN;
        if (PORAT < R(0.01)) PORAT = R(0.01);
        R TO2IS = om::pow(PORAT, FGA) * TO_IN;
        R TSTAT2_IS = om::pow(PSRAT, FGA) * TO_IN;
        R DELTOIS = TO2IS - TO_IN, DELT_TOT_STAT = TSTAT2_IS - TO_IN;
        R ETAIS = R(1.0);
        if (DELTO > R(0.0)) ETAIS = DELTOIS / DELTO;
        if (DELTO < R(0.0)) ETAIS = DELTO / DELTOIS;
        R ETATS = R(1.0);
        if (DELTO > R(0.0)) ETATS = DELT_TOT_STAT / DELTO;
        if (DELTO < R(0.0)) ETATS = DELTO / DELT_TOT_STAT;
        out->mass_flow_in = (double)BF[J1 - 1];
        out->mass_flow_out = (double)BF[J2M1 - 1];
        out->eta_tt = (double)ETAIS;
        out->eta_ts = (double)ETATS;
        out->po_ratio = (double)PORAT;
        out->to_ratio = (double)TORAT;
        out->j1 = J1;
        out->j2m1 = J2M1;
        return 0;
    }
};

} /* namespace */

/* ---------------------------------------------------------------------- */
/*  C entry points used by the test harness (ctypes)                       */
/* ---------------------------------------------------------------------- */
extern "C" {

void *oref_create(int32_t im, int32_t jm, int32_t km, int32_t nrows, int32_t use_double) {
    if (im < 3 || jm < 8 || km < 3 || nrows < 1) {
        g_err = "bad dimensions";
        return nullptr;
    }
    if (use_double == 2) return (OracleBase *)new Oracle<adt::AD>(im, jm, km, nrows);
    if (use_double) return (OracleBase *)new Oracle<double>(im, jm, km, nrows);
    return (OracleBase *)new Oracle<float>(im, jm, km, nrows);
}
void oref_destroy(void *h) { delete (OracleBase *)h; }
const char *oref_last_error(void) { return g_err.c_str(); }
int32_t oref_set_int(void *h, const char *n, int32_t v) { return ((OracleBase *)h)->set_int(n, v); }
int32_t oref_set_real(void *h, const char *n, double v) { return ((OracleBase *)h)->set_real(n, v); }
int32_t oref_get_real(void *h, const char *n, double *v) { return ((OracleBase *)h)->get_real(n, v); }
int32_t oref_get_int(void *h, const char *n, int32_t *v) { return ((OracleBase *)h)->get_int(n, v); }
int32_t oref_set_array(void *h, const char *n, const void *p, int64_t nb) { return ((OracleBase *)h)->set_array(n, p, nb); }
int32_t oref_get_array(void *h, const char *n, void *p, int64_t nb, int32_t as_double) {
    return ((OracleBase *)h)->get_array(n, p, nb, as_double);
}
int32_t oref_commit(void *h) { return ((OracleBase *)h)->commit(); }
int32_t oref_stepup(void *h, double relax) { return ((OracleBase *)h)->stepup(relax); }
int32_t oref_loss_init(void *h) { return ((OracleBase *)h)->loss_init(); }
int32_t oref_step(void *h, int32_t force_end, mgpu_monitors *mon) { return ((OracleBase *)h)->step(force_end, mon); }
int32_t oref_integrals(void *h, mgpu_integrals *out) { return ((OracleBase *)h)->integrals(out); }
int32_t oref_stage_performance(void *h, int32_t nstg, mgpu_stage *out) {
    return ((OracleBase *)h)->stage_performance(nstg, out);
}
int32_t oref_set_array_f64(void *h, const char *n, const double *p, int64_t cnt) {
    return ((OracleBase *)h)->set_array_f64(n, p, cnt);
}
int32_t oref_ad_begin(void *h) { return ((OracleBase *)h)->ad_begin(); }
int32_t oref_ad_zero(void *h) { return ((OracleBase *)h)->ad_zero(); }
int32_t oref_ad_seed(void *h, const char *n, const double *w, int64_t cnt) { return ((OracleBase *)h)->ad_seed(n, w, cnt); }
int32_t oref_ad_reverse(void *h) { return ((OracleBase *)h)->ad_reverse(); }
int32_t oref_ad_grad(void *h, const char *n, double *out, int64_t cnt) { return ((OracleBase *)h)->ad_grad(n, out, cnt); }
int64_t oref_ad_tape_size(void *h) { return ((OracleBase *)h)->ad_tape_size(); }
int32_t oref_write_flow_out(void *h, const char *path, const float *rosub) {
    return ((OracleBase *)h)->write_flow_out(path, rosub);
}
int32_t oref_write_grid_out(void *h, const char *path) { return ((OracleBase *)h)->write_grid_out(path); }
int32_t oref_read_flow_out(void *h, const char *path, int32_t *nstep) {
    return ((OracleBase *)h)->read_flow_out(path, nstep);
}

} /* extern "C" */
