// mgpu_io.cu -- the combined restart/plotting file "flow_out" written from the
// device state (OUTPUT, multall-open-18.3.f:5942-5978) and read back as
// SETUP's IF_RESTART branch reads it (6920-6992), so that a run can
// checkpoint and resume through the C ABI without a Fortran round trip.
//
// The file is what gfortran writes for WRITE(7) on a sequential unformatted
// unit: each record is its payload between two copies of its length in
// bytes, as 4-byte little-endian integers.  Records: NSTEP (INTEGER), then
// RO, ROVX, ROVR, ROVT, ROE, ROSUB, DPDS_CELL*1.0E-6 (TRANS_DYN_VIS with the
// Spalart-Allmaras model) and PEFF+PREFF, each
// IM*JM*KM REAL*4 values in Fortran order (I fastest).
//
// Both directions run on the host.  Writing reads the arrays back from the
// device; reading forms the secondary variables in REAL*4 with the
// reference's expressions and uploads them with mgpu_set_array, before
// mgpu_commit, whose LOOP prologue then starts from the restarted flow.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mgpu_internal.cuh"

using namespace mgpu;

namespace {

struct FileCloser {
    FILE *f = nullptr;
    ~FileCloser() {
        if (f) fclose(f);
    }
};

bool put_record(FILE *f, const void *p, uint32_t n) {
    return fwrite(&n, 4, 1, f) == 1 && (n == 0 || fwrite(p, 1, n, f) == n) && fwrite(&n, 4, 1, f) == 1;
}

// Reads one record of exactly n bytes into p (p == nullptr: skip it).
bool get_record(FILE *f, void *p, uint32_t n) {
    uint32_t a = 0, b = 0;
    if (fread(&a, 4, 1, f) != 1 || a != n) return false;
    if (p) {
        if (fread(p, 1, n, f) != n) return false;
    } else if (fseek(f, (long)n, SEEK_CUR) != 0) {
        return false;
    }
    return fread(&b, 4, 1, f) == 1 && b == n;
}

struct Dims {
    int IM, JM, KM;
    size_t N;
};

Dims dims_of(const HandleView &hv) {
    return Dims{hv.d->IM, hv.d->JM, hv.d->KM, (size_t)hv.d->IM * hv.d->JM * hv.d->KM};
}

}  // namespace

extern "C" {

int32_t mgpu_write_flow_out(mgpu_handle *h, const char *path, const float *rosub) {
    if (!h || !path) return api_fail(MGPU_E_ARG, "null argument to mgpu_write_flow_out");
    const HandleView hv = handle_view(h);
    if (!hv.committed) return api_fail(MGPU_E_STATE, "mgpu_write_flow_out before mgpu_commit");
    const Dims g = dims_of(hv);
    int rc = 0;
    const size_t N = g.N;
    const int64_t nb = (int64_t)(N * sizeof(float));
    std::vector<float> ro(N), rovx(N), rovr(N), rovt(N), roe(N), dpds(N), peff(N), p(N);
    if ((rc = mgpu_get_array(h, "RO", ro.data(), nb)) || (rc = mgpu_get_array(h, "ROVX", rovx.data(), nb)) ||
        (rc = mgpu_get_array(h, "ROVR", rovr.data(), nb)) || (rc = mgpu_get_array(h, "ROVT", rovt.data(), nb)) ||
        (rc = mgpu_get_array(h, "ROE", roe.data(), nb)) || (rc = mgpu_get_array(h, "DPDS_CELL", dpds.data(), nb)) ||
        (rc = mgpu_get_array(h, "PEFF", peff.data(), nb)) || (rc = mgpu_get_array(h, "P", p.data(), nb)))
        return rc;
    int32_t nstep = 0;
    if ((rc = mgpu_get_int(h, "NSTEP", &nstep))) return rc;
    // OUTPUT's own PREFF (5950), from the current pressures
    const int IMID = hv.d->IMID, KMID = hv.d->KMID;
    auto at = [&](const std::vector<float> &v, int i, int j, int k) {
        return v[(size_t)(i - 1) + (size_t)g.IM * ((size_t)(j - 1) + (size_t)g.JM * (size_t)(k - 1))];
    };
    const float PREFF = 0.5f * (at(p, IMID, 1, KMID) + at(p, IMID, g.JM, KMID));
    // the seventh array is the transported viscosity with the Spalart-
    // Allmaras model, else DPDS_CELL * 1.0E-6 for plotting (5966-5972)
    const bool sa = hv.d->ILOS >= 200;
    if (sa && (rc = mgpu_get_array(h, "TRANS_DYN_VIS", dpds.data(), nb))) return rc;
    for (size_t n = 0; n < N; ++n) {
        if (!sa) dpds[n] = dpds[n] * 1.0e-6f;
        peff[n] = peff[n] + PREFF;
    }
    FileCloser fc;
    fc.f = fopen(path, "wb");
    if (!fc.f) return api_fail(MGPU_E_ARG, (std::string("cannot open for writing: ") + path).c_str());
    const uint32_t rb = (uint32_t)(N * sizeof(float));
    const float *recs[] = {ro.data(), rovx.data(), rovr.data(), rovt.data(), roe.data(), rosub ? rosub : ro.data(),
                           dpds.data(), peff.data()};
    bool ok = put_record(fc.f, &nstep, 4);
    for (const float *r : recs) ok = ok && put_record(fc.f, r, rb);
    if (!ok || fflush(fc.f) != 0) return api_fail(MGPU_E_ARG, (std::string("write failed: ") + path).c_str());
    return 0;
}

int32_t mgpu_write_grid_out(mgpu_handle *h, const char *path) {
    if (!h || !path) return api_fail(MGPU_E_ARG, "null argument to mgpu_write_grid_out");
    const HandleView hv = handle_view(h);
    const Dims g = dims_of(hv);
    const size_t njk = (size_t)g.JM * g.KM;
    int32_t nrows = hv.d->NROWS, nsmax = 0;
    float CP = 0.0f, GA = 0.0f;
    std::vector<float> X(njk), R(njk), RT(g.N), WRAD(g.JM);
    std::vector<int32_t> INDLE(g.JM), NBLADE(g.JM), JTE(nrows);
    int rc = 0;
    if ((rc = mgpu_get_int(h, "NSTEPS_MAX", &nsmax)) || (rc = mgpu_get_real(h, "CP", &CP)) ||
        (rc = mgpu_get_real(h, "GA", &GA)) || (rc = mgpu_get_array(h, "X", X.data(), (int64_t)njk * 4)) ||
        (rc = mgpu_get_array(h, "R", R.data(), (int64_t)njk * 4)) ||
        (rc = mgpu_get_array(h, "RTHETA", RT.data(), (int64_t)g.N * 4)) ||
        (rc = mgpu_get_array(h, "WRAD", WRAD.data(), (int64_t)g.JM * 4)) ||
        (rc = mgpu_get_array(h, "INDLE", INDLE.data(), (int64_t)g.JM * 4)) ||
        (rc = mgpu_get_array(h, "NBLADE", NBLADE.data(), (int64_t)g.JM * 4)) ||
        (rc = mgpu_get_array(h, "JTE", JTE.data(), (int64_t)nrows * 4)))
        return rc;
    // INDLETE (6307-6309): 1 on the leading- and trailing-edge planes
    std::vector<int32_t> INDLETE(g.JM, 0);
    for (int j = 1; j <= g.JM; ++j)
        if (INDLE[j - 1] == 1) INDLETE[j - 1] = 1;
    for (int nr = 0; nr < nrows; ++nr)
        if (JTE[nr] >= 1 && JTE[nr] <= g.JM) INDLETE[JTE[nr] - 1] = 1;
    FileCloser fc;
    fc.f = fopen(path, "wb");
    if (!fc.f) return api_fail(MGPU_E_ARG, (std::string("cannot open for writing: ") + path).c_str());
    // 6587-6597
    const int32_t dims[3] = {g.IM, g.JM, g.KM};
    const float gas[2] = {CP, GA};
    const uint32_t nj = (uint32_t)g.JM * 4;
    bool ok = put_record(fc.f, &nsmax, 4) && put_record(fc.f, dims, 12) && put_record(fc.f, gas, 8) &&
              put_record(fc.f, INDLETE.data(), nj) && put_record(fc.f, WRAD.data(), nj) &&
              put_record(fc.f, NBLADE.data(), nj);
    std::vector<float> rec((size_t)g.IM + 2);
    for (int j = 1; j <= g.JM && ok; ++j)
        for (int k = 1; k <= g.KM && ok; ++k) {
            const size_t jk = (size_t)(j - 1) + (size_t)g.JM * (size_t)(k - 1);
            rec[0] = X[jk];
            rec[1] = R[jk];
            for (int i = 1; i <= g.IM; ++i) rec[(size_t)i + 1] = RT[(size_t)(i - 1) + (size_t)g.IM * jk];
            ok = put_record(fc.f, rec.data(), (uint32_t)rec.size() * 4);
        }
    if (!ok || fflush(fc.f) != 0) return api_fail(MGPU_E_ARG, (std::string("write failed: ") + path).c_str());
    return 0;
}

int32_t mgpu_read_flow_out(mgpu_handle *h, const char *path, int32_t *nstep) {
    if (!h || !path) return api_fail(MGPU_E_ARG, "null argument to mgpu_read_flow_out");
    const HandleView hv = handle_view(h);
    if (hv.committed) return api_fail(MGPU_E_STATE, "mgpu_read_flow_out after mgpu_commit (SETUP reads the restart file)");
    const Dims g = dims_of(hv);
    int rc = 0;
    const size_t N = g.N;
    const int64_t nb = (int64_t)(N * sizeof(float));
    const uint32_t rb = (uint32_t)nb;
    std::vector<float> ro(N), rovx(N), rovr(N), rovt(N), roe(N), tdv(N);
    int32_t ns = 0;
    {
        FileCloser fc;
        fc.f = fopen(path, "rb");
        if (!fc.f) return api_fail(MGPU_E_ARG, (std::string("cannot open: ") + path).c_str());
        // 6927-6934: NSTEP, the five variables, ROSUB (unused by the
        // covered schemes) and TRANS_DYN_VIS, read whatever the model
        const bool ok = get_record(fc.f, &ns, 4) && get_record(fc.f, ro.data(), rb) &&
                        get_record(fc.f, rovx.data(), rb) && get_record(fc.f, rovr.data(), rb) &&
                        get_record(fc.f, rovt.data(), rb) && get_record(fc.f, roe.data(), rb) &&
                        get_record(fc.f, nullptr, rb) && get_record(fc.f, tdv.data(), rb);
        if (!ok)
            return api_fail(MGPU_E_ARG, (std::string("not a flow_out file of this grid: ") + path).c_str());
    }
    float CP = 0.0f, GA = 0.0f;
    int32_t IPOUT = 0;
    if ((rc = mgpu_get_real(h, "CP", &CP)) || (rc = mgpu_get_real(h, "GA", &GA)) ||
        (rc = mgpu_get_int(h, "IPOUT", &IPOUT)))
        return rc;
    // SETUP 6459-6468
    const float CV = CP / GA, RGAS = CP - CV;
    std::vector<float> R((size_t)g.JM * g.KM), FP(g.IM), PD(g.KM);
    if ((rc = mgpu_get_array(h, "R", R.data(), (int64_t)R.size() * 4)) ||
        (rc = mgpu_get_array(h, "FP", FP.data(), (int64_t)FP.size() * 4)) ||
        (rc = mgpu_get_array(h, "PD", PD.data(), (int64_t)PD.size() * 4)))
        return rc;
    // 3900: the secondary variables (IFGAS = 0, ITIMST < 5)
    std::vector<float> vx(N), vr(N), vt(N), rorvt(N), ts(N), ho(N), p(N);
    for (int k = 1; k <= g.KM; ++k)
        for (int j = 1; j <= g.JM; ++j)
            for (int i = 1; i <= g.IM; ++i) {
                const size_t n = (size_t)(i - 1) + (size_t)g.IM * ((size_t)(j - 1) + (size_t)g.JM * (size_t)(k - 1));
                vx[n] = rovx[n] / ro[n];
                vr[n] = rovr[n] / ro[n];
                vt[n] = rovt[n] / ro[n];
                rorvt[n] = rovt[n] * R[(size_t)(j - 1) + (size_t)g.JM * (size_t)(k - 1)];
                const float EKE = 0.5f * (vx[n] * vx[n] + vr[n] * vr[n] + vt[n] * vt[n]);
                const float TSTATIC = (roe[n] / ro[n] - EKE) / CV;
                ts[n] = TSTATIC;
                ho[n] = CP * TSTATIC + EKE;
                p[n] = ro[n] * RGAS * TSTATIC;
            }
    // 3902-3903: the exit pressures, shifted to keep PD(1) (IPOUT = 0) or
    // PD(KM) (IPOUT = -1)
    if (IPOUT <= 0) {
        std::vector<float> PDOWN(g.KM);
        for (int k = 1; k <= g.KM; ++k) {
            float s = 0.0f;
            for (int i = 1; i <= g.IM - 1; ++i) {
                const size_t a = (size_t)(i - 1) + (size_t)g.IM * ((size_t)(g.JM - 1) + (size_t)g.JM * (size_t)(k - 1));
                s = s + FP[i - 1] * 0.5f * (p[a] + p[a + 1]);
            }
            PDOWN[k - 1] = s;
        }
        const float PDIFF = IPOUT == 0 ? PD[0] - PDOWN[0] : PD[g.KM - 1] - PDOWN[g.KM - 1];
        for (int k = 0; k < g.KM; ++k) PD[k] = PDOWN[k] + PDIFF;
    }
    struct {
        const char *name;
        const std::vector<float> *v;
    } up[] = {{"RO", &ro}, {"ROVX", &rovx}, {"ROVR", &rovr}, {"ROVT", &rovt}, {"ROE", &roe},
              {"RORVT", &rorvt}, {"VX", &vx}, {"VR", &vr}, {"VT", &vt}, {"T_STATIC", &ts},
              {"HO", &ho}, {"P", &p}, {"PEFF", &p},      // PEFF = P here (6977)
              {"TRANS_DYN_VIS", &tdv}};
    for (auto &u : up)
        if ((rc = mgpu_set_array(h, u.name, u.v->data(), nb))) return rc;
    if ((rc = mgpu_set_array(h, "PD", PD.data(), (int64_t)PD.size() * 4))) return rc;
    if (nstep) *nstep = ns;
    return 0;
}

}  // extern "C"
