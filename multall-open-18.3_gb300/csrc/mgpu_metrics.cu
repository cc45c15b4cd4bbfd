// mgpu_metrics.cu -- SETUP's face areas and volumes on the device
// (multall-open-18.3.f:6490-6502 THETA, 6528-6540 DS, 6570-6578 the theta
// extrapolated onto the upstream side of each mixing plane, 6605-6711 the
// quasi-orthogonal, bladewise and streamwise face areas, the volumes and
// VOLOR), in float or double.
//
// Each value is formed by the reference's expression in its order of
// operations; with the library's --fmad=false and IEEE division and square
// root, the float instance gives SETUP's REAL*4 values bit for bit.  One
// thread per node; a node thread also writes the copies SETUP makes onto the
// last I and K planes (AQX(IM,J,K) = AQX(IMM1,J,K), ...), by evaluating the
// copied value's expression itself.
#include "mgpu_internal.cuh"

namespace mgpu {

namespace {

template <typename T>
struct Geo {
    int IM, JM, KM;
    MetricArgs<T> a;
    __device__ T X(int j, int k) const { return a.X[(j - 1) + JM * (k - 1)]; }
    __device__ T R(int j, int k) const { return a.R[(j - 1) + JM * (k - 1)]; }
    __device__ int n3(int i, int j, int k) const { return (i - 1) + IM * ((j - 1) + JM * (k - 1)); }
    __device__ T TH(int i, int j, int k) const { return a.THETA[n3(i, j, k)]; }
    __device__ T RT(int i, int j, int k) const { return a.RTHETA[n3(i, j, k)]; }
    __device__ T T1(int i, int j, int k) const { return a.TEMP1[n3(i, j, k)]; }
    __device__ T T2(int i, int j, int k) const { return a.TEMP2[n3(i, j, k)]; }
    __device__ bool mix(int j) const { return a.INDMIX[j - 1] == 1; }
    // DS(J,K), SETUP 6534 (J >= 2)
    __device__ T DS(int j, int k) const {
        T dr = R(j, k) - R(j - 1, k);
        T dx = X(j, k) - X(j - 1, k);
        return sqrt(dr * dr + dx * dx);
    }
};

template <typename T>
__global__ void k_met_theta(Geo<T> g) {
    const int N = g.IM * g.JM * g.KM;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        g.a.THETA[n] = g.a.RTHETA[n] / g.a.R[n / g.IM];         // 6502: R(J,K) of node n
    }
}

// TEMP1, TEMP2 on the planes J with INDMIX(J) = 1 (3025)
template <typename T>
__global__ void k_met_temp(Geo<T> g) {
    const int N = g.IM * g.JM * g.KM;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const int i = n % g.IM + 1, j = (n / g.IM) % g.JM + 1, k = n / (g.IM * g.JM) + 1;
        if (!g.mix(j) || j + 2 > g.JM) continue;
        const T FAC = g.DS(j + 1, k) / g.DS(j + 2, k);
        const T t1 = g.TH(i, j + 1, k) + FAC * (g.TH(i, j + 1, k) - g.TH(i, j + 2, k));
        g.a.TEMP1[n] = t1;
        g.a.TEMP2[n] = g.R(j, k) * t1;
    }
}

// the quasi-orthogonal face of (i, j, k), i <= IMM1, k <= KMM1 (3015)
template <typename T>
__device__ inline void aq_face(const Geo<T> &g, int i, int j, int k, T &ax, T &ar) {
    const T X1 = g.X(j, k + 1) - g.X(j, k), X2 = X1;
    const T R1 = g.R(j, k + 1) - g.R(j, k), R2 = R1;
    const T T1 = g.R(j, k + 1) * (g.TH(i + 1, j, k + 1) - g.TH(i, j, k));
    const T T2 = g.R(j, k + 1) * (g.TH(i, j, k + 1) - g.TH(i, j, k)) - g.R(j, k) * (g.TH(i + 1, j, k) - g.TH(i, j, k));
    ax = T(-0.5) * (R2 * T1 - R1 * T2);
    ar = T(-0.5) * (X1 * T2 - X2 * T1);
}

template <typename T>
__global__ void k_met_faces(Geo<T> g) {
    const int IM = g.IM, JM = g.JM, KM = g.KM, IMM1 = IM - 1, KMM1 = KM - 1;
    const int N = IM * JM * KM;
    MetricArgs<T> a = g.a;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const int i = n % IM + 1, j = (n / IM) % JM + 1, k = n / (IM * JM) + 1;
        // quasi-orthogonal faces, with the copies onto K = KM and I = IM (3030-3031)
        {
            const int ii = i == IM ? IMM1 : i, kk = k == KM ? KMM1 : k;
            T ax, ar;
            aq_face(g, ii, j, kk, ax, ar);
            a.AQX[n] = ax;
            a.AQR[n] = ar;
        }
        if (j < 2 || k > KMM1) continue;
        // bladewise faces and volumes (3040)
        const T X1 = g.X(j - 1, k + 1) - g.X(j, k);
        const T X2 = g.X(j, k + 1) - g.X(j - 1, k);
        const T R1 = g.R(j - 1, k + 1) - g.R(j, k);
        const T R2 = g.R(j, k + 1) - g.R(j - 1, k);
        const T ABT = T(-0.5) * (X1 * R2 - X2 * R1);
        if (i == 1) {
            a.ABT[(j - 1) + JM * (k - 1)] = ABT;
            a.WRABT[(j - 1) + JM * (k - 1)] =
                T(a.WRAD[j - 1]) * T(0.25) * (g.R(j, k) + g.R(j - 1, k) + g.R(j - 1, k + 1) + g.R(j, k + 1)) * ABT;
        }
        const bool mx = g.mix(j - 1);
        T T1, T2;
        if (!mx) {
            T1 = g.R(j - 1, k + 1) * (g.TH(i, j - 1, k + 1) - g.TH(i, j, k));
            T2 = g.R(j, k + 1) * (g.TH(i, j, k + 1) - g.TH(i, j, k)) - g.R(j - 1, k) * (g.TH(i, j - 1, k) - g.TH(i, j, k));
        } else {
            T1 = g.R(j - 1, k + 1) * (g.T1(i, j - 1, k + 1) - g.TH(i, j, k));
            T2 = g.R(j, k + 1) * (g.TH(i, j, k + 1) - g.TH(i, j, k)) - g.R(j - 1, k) * (g.T1(i, j - 1, k) - g.TH(i, j, k));
        }
        a.ABX[n] = T(-0.5) * (R1 * T2 - R2 * T1);
        a.ABR[n] = T(-0.5) * (X2 * T1 - X1 * T2);
        if (i < IM) {
            if (!mx)
                a.VOL[n] = ABT * T(0.25) *
                           (g.RT(i + 1, j, k) + g.RT(i + 1, j - 1, k) + g.RT(i + 1, j - 1, k + 1) + g.RT(i + 1, j, k + 1) -
                            g.RT(i, j, k) - g.RT(i, j - 1, k) - g.RT(i, j - 1, k + 1) - g.RT(i, j, k + 1));
            else
                a.VOL[n] = ABT * T(0.25) *
                           (g.RT(i + 1, j, k) + g.T2(i + 1, j - 1, k) + g.T2(i + 1, j - 1, k + 1) + g.RT(i + 1, j, k + 1) -
                            g.RT(i, j, k) - g.T2(i, j - 1, k) - g.T2(i, j - 1, k + 1) - g.RT(i, j, k + 1));
        }
    }
    // streamwise faces (3050): every K, i <= IMM1, j >= 2
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const int i = n % IM + 1, j = (n / IM) % JM + 1, k = n / (IM * JM) + 1;
        if (j < 2 || i > IMM1) continue;
        const T X1 = g.X(j - 1, k) - g.X(j, k), X2 = X1;
        const T R1 = g.R(j - 1, k) - g.R(j, k), R2 = R1;
        T T1, T2;
        if (!g.mix(j - 1)) {
            T1 = g.R(j - 1, k) * (g.TH(i, j - 1, k) - g.TH(i, j, k)) - g.R(j, k) * (g.TH(i + 1, j, k) - g.TH(i, j, k));
            T2 = g.R(j - 1, k) * (g.TH(i + 1, j - 1, k) - g.TH(i, j, k));
        } else {
            T1 = g.R(j - 1, k) * (g.T1(i, j - 1, k) - g.TH(i, j, k)) - g.R(j, k) * (g.TH(i + 1, j, k) - g.TH(i, j, k));
            T2 = g.R(j - 1, k) * (g.T1(i + 1, j - 1, k) - g.TH(i, j, k));
        }
        a.ASX[n] = T(0.5) * (R1 * T2 - R2 * T1);
        a.ASR[n] = T(0.5) * (X2 * T1 - X1 * T2);
    }
}

// VOLOR (4045): i <= IMM1, j >= 2, k <= KMM1
template <typename T>
__global__ void k_met_volor(Geo<T> g) {
    const int IM = g.IM, JM = g.JM, KM = g.KM;
    const int N = IM * JM * KM;
    MetricArgs<T> a = g.a;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const int i = n % IM + 1, j = (n / IM) % JM + 1, k = n / (IM * JM) + 1;
        if (j < 2 || i > IM - 1 || k > KM - 1) continue;
        const T RAREA = a.ABR[n] - a.ABR[n + 1] + a.AQR[n] - a.AQR[n - IM] + a.ASR[n] - a.ASR[n + IM * JM];
        a.VOLOR[n] = T(-0.125) * RAREA;
    }
}

// ---------------------------------------------------------------------
// SETUP's grid from a deck's blade sections: NEW_INTPOL (7493-7613), the
// circumferential alignment of the rows at mid-span (6442-6448), the
// pinched-tip thickness (6452-6459) and RTHETA (6490-6501), in REAL*4 in
// the reference's order of operations.
// ---------------------------------------------------------------------
constexpr int MAX_SECS = 32;

// INTP (7801-7872): Lagrange interpolation through four neighbouring table
// points (all n when n < 4); xn, yn 0-based here
__device__ float intp_dev(int n, const float *xn, const float *yn, float x) {
    const float span = xn[n - 1] - xn[0];
    int L = 1, nm = n;
    if (n >= 4) {
        nm = 4;
        for (;;) {
            if ((span > 0.0f && x < xn[L - 1]) || (span < 0.0f && x > xn[L - 1])) {
                L = L > 2 ? (L != n ? L - 2 : n - 3) : 1;
                break;
            }
            if (L == n) {
                L = n - 3;
                break;
            }
            ++L;
        }
    }
    float y = 0.0f;
    for (int l1 = 1; l1 <= nm; ++l1) {
        float co = 1.0f;
        for (int l2 = 1; l2 <= nm; ++l2) {
            float temp = 1.0f;
            if (l1 != l2) temp = (x - xn[L + l2 - 2]) / (xn[L + l1 - 2] - xn[L + l2 - 2]);
            co = co * temp;
        }
        y = y + co * yn[L + l1 - 2];
    }
    return y;
}

// SMERID of each input section (7500-7506), one thread per section
__global__ void k_geo_smerid(GeoArgs g) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.NS) return;
    const float *xs = g.sec + (size_t)s * g.JM, *rs = g.sec + (size_t)(g.NS + s) * g.JM;
    float *sm = g.SMERID + (size_t)s * g.JM;
    sm[0] = 0.0f;
    for (int j = 2; j <= g.JM; ++j) {
        const float xd = xs[j - 1] - xs[j - 2], rd = rs[j - 1] - rs[j - 2];
        sm[j - 1] = sm[j - 2] + sqrtf(xd * xd + rd * rd);
    }
}

// NEW_INTPOL, one thread per J: the KM stream surfaces of plane J
__global__ void k_geo_intpol(GeoArgs g) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > g.JM) return;
    const int JM = g.JM, NS = g.NS;
    const int nr = g.NROW[j - 1];
    const int j1 = g.JSTART[nr - 1], jl = g.JLE[nr - 1], jt = g.JTE[nr - 1], je = g.JMIX[nr - 1];
    const int kts = g.KTIPS[nr - 1], kte = g.KTIPE[nr - 1], ks1 = g.KS1[nr - 1], ks2 = g.KS2[nr - 1];
    // the tip-gap grid (FRMOD, 7519-7560): FAC, TIPGAP, TIPSPACE and SUMFR
    // are DOUBLE PRECISION there
    double fac = 1.0, tipgap = 0.0, tipspace = 0.0, sumfr = 0.0;
    const bool tip = kts > 0;
    if (tip) {
        const int ktip = kts == 1 ? 1 : NS;
        const float *sm = g.SMERID + (size_t)(ktip - 1) * JM;
        const float f1 = g.FRACTIP[2 * (nr - 1)], f2 = g.FRACTIP[2 * (nr - 1) + 1];
        if (j >= j1 && j < jl) {
            fac = (double)((sm[j - 1] - sm[j1 - 1]) / (sm[jl - 1] - sm[j1 - 1]));
            tipgap = (double)f1;
        }
        if (j >= jl && j <= jt) {
            fac = 1.0;
            const float frac = (sm[j - 1] - sm[jl - 1]) / (sm[jt - 1] - sm[jl - 1]);
            tipgap = (double)(f1 + frac * (f2 - f1));
        }
        if (j > jt && j <= je) {
            fac = (double)((sm[je - 1] - sm[j - 1]) / (sm[je - 1] - sm[jt - 1]));
            tipgap = (double)f2;
        }
        for (int k = kts; k <= kte - 1; ++k) sumfr = sumfr + (double)g.FR[k - 1];
        tipspace = tipgap / (double)(kte - kts);
    }
    float xi[MAX_SECS], yi[MAX_SECS], ru[MAX_SECS], rt[MAX_SECS], qod[MAX_SECS];
    for (int s = 0; s < NS; ++s) {
        xi[s] = g.sec[(size_t)s * JM + (j - 1)];
        yi[s] = g.sec[(size_t)(NS + s) * JM + (j - 1)];
        ru[s] = g.sec[(size_t)(2 * NS + s) * JM + (j - 1)];
        rt[s] = g.sec[(size_t)(3 * NS + s) * JM + (j - 1)];
        if (s == 0) {
            qod[0] = 0.0f;
        } else {
            const float rd = yi[s] - yi[s - 1], xd = xi[s] - xi[s - 1];
            qod[s] = qod[s - 1] + sqrtf(xd * xd + rd * rd);
        }
    }
    const float qospan = qod[NS - 1];
    float xarg = 0.0f;
    for (int k = 1; k <= g.KM; ++k) {
        const int o = (j - 1) + JM * (k - 1);
        g.X[o] = intp_dev(NS, qod, xi, xarg);
        g.R[o] = intp_dev(NS, qod, yi, xarg);
        g.RTU[o] = intp_dev(NS, qod, ru, xarg);
        g.RTT[o] = intp_dev(NS, qod, rt, xarg);
        float frmod = g.FR[k - 1];
        if (tip && k >= kts && k <= kte - 1) frmod = (float)(tipspace * fac + (1.0 - fac) * (double)g.FR[k - 1]);
        if (tip && k >= ks1 && k <= ks2)
            frmod = (float)((double)g.FR[k - 1] * ((1.0 - tipgap) / (1.0 - sumfr) * fac + (1.0 - fac)));
        xarg = xarg + frmod * qospan;
    }
}

// the alignment shifts along J (6442-6448): each plane after a mixing plane
// is turned so that its mid-span I = 1 line continues the previous plane's;
// sequential in J, one thread
__global__ void k_geo_shift(GeoArgs g) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int JM = g.JM, km = g.KMID;
    float SHIFT = 0.0f, prev = g.RTU[1 + JM * (km - 1)];    // RT_UPP(2, KMID), not moved
    g.SH[0] = g.SH[1] = 0.0f;
    for (int j = 3; j <= JM; ++j) {
        const float rtu = g.RTU[(j - 1) + JM * (km - 1)], r = g.R[(j - 1) + JM * (km - 1)];
        if (g.INDMIX[j - 2] == 1) SHIFT = (prev - rtu) / r;
        g.SH[j - 1] = SHIFT;
        prev = rtu + SHIFT * r;
    }
}

// the shift and the pinched-tip thickness of node line (J, K), then its
// RTHETA(I) (6490-6501)
__global__ void k_geo_rtheta(GeoArgs g) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.JM * g.KM) return;
    const int j = t % g.JM + 1, k = t / g.JM + 1;
    const float R = g.R[t];
    float rtu = g.RTU[t], rtt = g.RTT[t];
    if (j >= 3) rtu = rtu + g.SH[j - 1] * R;
    const int nr = g.NROW[j - 1];
    const float RTMID = rtu - 0.5f * rtt;
    const float THICK = g.FTHICK[(size_t)(nr - 1) * g.KM + (k - 1)] * rtt;
    rtu = RTMID + 0.5f * THICK;
    rtt = THICK;
    g.RTU[t] = rtu;
    g.RTT[t] = rtt;
    const float PI = 3.14159265f;
    const float PITCH = 2.0f * PI / (float)g.NBLADE[j - 1];
    const float GAP = PITCH * R - rtt;
    float *rth = g.RTHETA + (size_t)(j - 1) * g.IM + (size_t)(k - 1) * g.IM * g.JM;
    float v = rtu;
    rth[0] = v;
    for (int i = 2; i <= g.IM; ++i) {
        v = v + g.FP[i - 2] * GAP;
        rth[i - 1] = v;
    }
}

}  // namespace

cudaError_t launch_setup_geometry(const GeoArgs &g, cudaStream_t s) {
    if (g.NS < 2 || g.NS > MAX_SECS) return cudaErrorInvalidValue;
    k_geo_smerid<<<1, 32, 0, s>>>(g);
    k_geo_intpol<<<(g.JM + 127) / 128, 128, 0, s>>>(g);
    k_geo_shift<<<1, 1, 0, s>>>(g);
    k_geo_rtheta<<<(g.JM * g.KM + 255) / 256, 256, 0, s>>>(g);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_setup_metrics(int IM, int JM, int KM, const MetricArgs<T> &a, cudaStream_t s) {
    Geo<T> g{IM, JM, KM, a};
    const int N = IM * JM * KM;
    const unsigned grid = (unsigned)((N + 255) / 256);
    k_met_theta<T><<<grid, 256, 0, s>>>(g);
    k_met_temp<T><<<grid, 256, 0, s>>>(g);
    k_met_faces<T><<<grid, 256, 0, s>>>(g);
    k_met_volor<T><<<grid, 256, 0, s>>>(g);
    return cudaGetLastError();
}

template cudaError_t launch_setup_metrics<float>(int, int, int, const MetricArgs<float> &, cudaStream_t);
template cudaError_t launch_setup_metrics<double>(int, int, int, const MetricArgs<double> &, cudaStream_t);

}  // namespace mgpu
