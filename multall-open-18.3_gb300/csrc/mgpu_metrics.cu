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

}  // namespace

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
