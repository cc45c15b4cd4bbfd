// mgpu_sa.cu -- the Spalart-Allmaras turbulence model (ILOS 200-299) on the
// GPU: SPAL_LOSS (multall-open-18.3.f:13586-14832, with GRADCELL 13516-13585)
// and the transport of its cell-centred turbulent viscosity TRANS_DYN_VIS
// through the loop (fluxes 4279-4330, TSTEP's NCALL = 2 branch 5736-5777,
// the floor and kinematic value 4340-4347, the inlet value 4679-4689).
//
// The transported viscosity is a sixth TSTEP variable (d.var[V_SA]): its
// flux sum, SCREE update, multigrid and negative feedback's row means run
// in TSTEP's own kernels (launch_tstep_cells_prolong); the branch that
// differs runs here: the damped change is added to the cell, the last plane
// of each row is carried across the mixing plane with the decay
// TURBVIS_DAMP, one SMOOTH_RESID pass smooths it, and the periodic, tip-gap
// and mixing-plane averages close the step.
//
// SPAL_LOSS shares the wall shear stresses, the face stresses and the force
// update with NEW_LOSS (k_nl_walls, k_nl_forces); its own kernels form the
// S-A viscosity of every cell, the gradient of the kinematic viscosity, the
// source term of the transport equation and its damping in laminar regions.
// Every expression keeps the reference's evaluation order.  Two reference
// scalars are reproduced as the reference leaves them: VORTICITY_FAC and
// PGRAD_FAC are the last cell's values of DO 1000 when DO 1600 reads them,
// and PTERM of that cell uses the laminar viscosity of the cell before it.
#include "mgpu_internal.cuh"

namespace mgpu {

namespace {

constexpr int SA_BS = 256;

// node-array slices of the work buffer
enum { SAW_ABS_VORT = 0, SAW_DYN_VIS_ML = 1, SAW_GRAD_TVIS = 2, SAW_TVGX = 3, SAW_TVGR = 4, SAW_TVGT = 5 };
__device__ inline float *saw(const Dev &d, int which) { return d.SAW + (size_t)which * d.IM * d.JM * d.KM; }
// REYNOLDS(NR) at [NR-1], then VORTICITY_FAC [64], PGRAD_FAC [65], RO_OLD [66]
__device__ inline float *saw_scalars(const Dev &d) { return d.SAW + sa_work_node_floats(d); }

__device__ inline bool sa_cell(const Dev &d, int t, int &i, int &j, int &k) {
    const int IMM1 = d.IMM1, JC = d.JM - 1;
    if (t >= IMM1 * JC * d.KMM1) return false;
    i = t % IMM1 + 1;
    const int q = t / IMM1;
    j = q % JC + 2;
    k = q / JC + 1;
    return true;
}

// the free-stream transported viscosity (13832-13838, 4681-4684)
__device__ inline float transvis_in(const Dev &d, float vislam) {
    const float fs = A1(d.FSTURB, 1);
    if (fs < 1.0f) return 4.35f * vislam * powf(fs, 0.25f);
    return vislam * (3.5f + fs * 0.85f);
}

__device__ inline float fyplus_sa(float yp, float yplam, float ypturb) {
    float f = 0.0f;
    if (yp > yplam) {
        float XFAC = (yp - yplam) / (ypturb - yplam);
        if (XFAC > 1.0f) XFAC = 1.0f;
        f = XFAC * XFAC * (3.0f - 2.0f * XFAC);
    }
    return f;
}

// the face areas and volume of one cell, for GRADVEL (13468-13508)
struct CellGeo {
    float RVOL, aqx0, aqx1, abx0, abx1, asx0, asx1, aqr0, aqr1, abr0, abr1, asr0, asr1, abt, RAVG;
};

__device__ inline CellGeo cell_geo(const Dev &d, int n, int j, int k) {
    const int sJ = d.IM, sK = d.IM * d.JM;
    CellGeo g;
    g.RVOL = 0.25f / d.VOL[n];
    g.aqx0 = d.AQX[n]; g.aqx1 = d.AQX[n - sJ]; g.abx0 = d.ABX[n]; g.abx1 = d.ABX[n + 1];
    g.asx0 = d.ASX[n]; g.asx1 = d.ASX[n + sK];
    g.aqr0 = d.AQR[n]; g.aqr1 = d.AQR[n - sJ]; g.abr0 = d.ABR[n]; g.abr1 = d.ABR[n + 1];
    g.asr0 = d.ASR[n]; g.asr1 = d.ASR[n + sK];
    g.abt = A2(d.ABT, j, k);
    g.RAVG = A2(d.RAVG_CELL, j, k);
    return g;
}

// GRADVEL of the node quantity V at the cell whose first corner is n
__device__ inline void gradvel(const Dev &d, const CellGeo &g, int n, const float *V, float &dx, float &dr,
                               float &dt) {
    const int sJ = d.IM, sK = d.IM * d.JM;
    const int o000 = n, o100 = n + 1, o0m0 = n - sJ, o1m0 = n + 1 - sJ;
    const int o001 = n + sK, o101 = n + 1 + sK, o0m1 = n - sJ + sK, o1m1 = n + 1 - sJ + sK;
    const float VAVGJ1 = V[o0m0] + V[o1m0] + V[o1m1] + V[o0m1];
    const float VAVGJ2 = V[o000] + V[o100] + V[o101] + V[o001];
    const float VAVGI1 = V[o000] + V[o0m0] + V[o0m1] + V[o001];
    const float VAVGI2 = V[o100] + V[o1m0] + V[o1m1] + V[o101];
    const float VAVGK1 = V[o000] + V[o100] + V[o1m0] + V[o0m0];
    const float VAVGK2 = V[o001] + V[o101] + V[o1m1] + V[o0m1];
    const float VAVGCELL = 0.125f * (VAVGJ1 + VAVGJ2);
    dx = -((VAVGJ2 * g.aqx0 - VAVGJ1 * g.aqx1 + VAVGI1 * g.abx0 - VAVGI2 * g.abx1 + VAVGK1 * g.asx0 -
            VAVGK2 * g.asx1) * g.RVOL);
    dr = -((VAVGJ2 * g.aqr0 - VAVGJ1 * g.aqr1 + VAVGI1 * g.abr0 - VAVGI2 * g.abr1 + VAVGK1 * g.asr0 -
            VAVGK2 * g.asr1) * g.RVOL) - VAVGCELL / g.RAVG;
    dt = -((VAVGI1 - VAVGI2) * g.abt * g.RVOL);
}

// GRADCELL (13516-13585) of the cell quantity V at cell (i, j, k); planes
// past J = JM are the never-written slots of a COMMON array: zero
__device__ inline void gradcell(const Dev &d, int i, int j, int k, const float *V, float &dx, float &dr, float &dt) {
    int ip1 = i + 1, im1 = i - 1, kp1 = k + 1, km1 = k - 1;
    if (i == 1) im1 = d.IMM1;
    if (i == d.IMM1) ip1 = 1;
    if (k == 1) km1 = 1;
    if (k == d.KMM1) kp1 = d.KMM1;
    const int n = ix3(d, i, j, k);
    const float v0 = V[n];
    const float vjm = V[ix3(d, i, j - 1, k)];
    const float vjp = j + 1 > d.JM ? 0.0f : V[ix3(d, i, j + 1, k)];
    const float RVOL = 0.5f / d.VOL[n];
    const float VAVGJ1 = v0 + vjm;
    const float VAVGJ2 = v0 + vjp;
    float VAVGI1 = v0 + V[ix3(d, im1, j, k)];
    float VAVGI2 = v0 + V[ix3(d, ip1, j, k)];
    float VAVGK1 = v0 + V[ix3(d, i, j, km1)];
    float VAVGK2 = v0 + V[ix3(d, i, j, kp1)];
    if (A1(d.IND, j) == 1) {
        if (i == 1) VAVGI1 = 0.0f;
        if (i == d.IMM1) VAVGI2 = 0.0f;
    }
    if (k == 1 && (d.IBOUND == 0 || d.IBOUND == 2)) VAVGK1 = 0.0f;
    if (k == d.KMM1 && d.IBOUND <= 1) VAVGK2 = 0.0f;
    const int sJ = d.IM, fi = ix3(d, ip1, j, k), fk = ix3(d, i, j, kp1);
    dx = -((VAVGJ2 * d.AQX[n] - VAVGJ1 * d.AQX[n - sJ] + VAVGI1 * d.ABX[n] - VAVGI2 * d.ABX[fi] +
            VAVGK1 * d.ASX[n] - VAVGK2 * d.ASX[fk]) * RVOL);
    dr = -((VAVGJ2 * d.AQR[n] - VAVGJ1 * d.AQR[n - sJ] + VAVGI1 * d.ABR[n] - VAVGI2 * d.ABR[fi] +
            VAVGK1 * d.ASR[n] - VAVGK2 * d.ASR[fk]) * RVOL) - v0 / A2(d.RAVG_CELL, j, k);
    dt = -((VAVGI1 - VAVGI2) * A2(d.ABT, j, k) * RVOL);
}

// the velocity and temperature gradients of DO 1000 at one cell
struct CellGrad {
    float DVXDX, DVXDR, DVXDT, DVRDX, DVRDR, DVRDT, DWTDX, DWTDR, DWTDT, DTDX, DTDR, DTDT, WTAVG;
};

__device__ inline CellGrad cell_grad(const Dev &d, int i, int j, int k) {
    const int n = ix3(d, i, j, k);
    const CellGeo g = cell_geo(d, n, j, k);
    CellGrad c;
    gradvel(d, g, n, d.VX, c.DVXDX, c.DVXDR, c.DVXDT);
    gradvel(d, g, n, d.VR, c.DVRDX, c.DVRDR, c.DVRDT);
    gradvel(d, g, n, d.WT, c.DWTDX, c.DWTDR, c.DWTDT);
    gradvel(d, g, n, d.T_STATIC, c.DTDX, c.DTDR, c.DTDT);
    const int sJ = d.IM, sK = d.IM * d.JM;
    const float *A = d.WT;
    c.WTAVG = 0.125f * (A[n] + A[n + 1] + A[n + 1 + sK] + A[n + sK] + A[n - sJ] + A[n + 1 - sJ] + A[n + 1 - sJ + sK] +
                        A[n - sJ + sK]);
    (void)i;
    return c;
}

// the vorticity of DO 1000 before the mixing-plane copy: zero on a row's
// first plane, at most VORT_MAX
__device__ inline float cell_vort(const Dev &d, const CellGrad &c, int j, float RAVG, float &VORTX, float &VORTR,
                                  float &VORTT) {
    VORTX = c.DVRDT - c.DWTDR - c.WTAVG / RAVG;
    VORTR = c.DWTDX - c.DVXDT;
    VORTT = c.DVXDR - c.DVRDX;
    float VORT = sqrtf(VORTX * VORTX + VORTR * VORTR + VORTT * VORTT);
    if (j == A1(d.JSTART, A1(d.NROW, j))) VORT = 0.0f;
    if (VORT > d.VORT_MAX) VORT = d.VORT_MAX;
    return VORT;
}

// ---------------------------------------------------------------------
// DO 1000: strain rates, vorticity and the S-A viscosity of every cell
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(SA_BS) k_sa_cells(const __grid_constant__ Dev d, int init_call) {
    pdl_wait();
    const DevCtl *c = d.ctl;
    if (!init_call && !c->do_loss) return;
    int i, j, k;
    if (!sa_cell(d, blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const int n = ix3(d, i, j, k);
    const int nstep = init_call ? 1 : c->nstep;
    const float FMIXUP = init_call ? 1.0f : c->FMIXUP;
    float VISLAM = c->VISLAM;
    const CellGrad g = cell_grad(d, i, j, k);
    const float RAVG = A2(d.RAVG_CELL, j, k);
    const size_t N = (size_t)d.IM * d.JM * d.KM;
    float *W = d.NLS;
    W[n] = g.DVXDR + g.DVRDX;                        // TXR
    W[N + n] = g.DVXDX;                              // TXX
    W[2 * N + n] = g.DWTDX + g.DVXDT;                // TXT
    W[3 * N + n] = g.DVRDR;                          // TRR
    W[4 * N + n] = g.DWTDR + g.DVRDT - g.WTAVG / RAVG;   // TRT
    W[5 * N + n] = g.DWTDT;                          // TTT
    W[6 * N + n] = g.DTDX;                           // QXX
    W[7 * N + n] = g.DTDR;                           // QRR
    W[8 * N + n] = g.DTDT;                           // QTT
    float VX_, VR_, VT_;
    float VORT = cell_vort(d, g, j, RAVG, VX_, VR_, VT_);
    if (A1(d.INDMIX, j) == 1) {
        // the mixing plane's cell takes the vorticity of the cell upstream
        const CellGrad gm = cell_grad(d, i, j - 1, k);
        VORT = cell_vort(d, gm, j - 1, A2(d.RAVG_CELL, j - 1, k), VX_, VR_, VT_);
    }
    saw(d, SAW_ABS_VORT)[n] = VORT;
    const float ROAVG = d.ROAVG_CELL[n];
    const float TURBVIS_WALL = ROAVG * d.XLENGTH[n] * VORT * FMIXUP;
    if (d.REYNO < 0.0001f) {
        const int sJ = d.IM, sK = d.IM * d.JM;
        const float *A = d.T_STATIC;
        const float TSAVG = 0.125f * (A[n] + A[n + 1] + A[n + 1 + sK] + A[n + sK] + A[n - sJ] + A[n + 1 - sJ] +
                                      A[n + 1 - sJ + sK] + A[n - sJ + sK]);
        VISLAM = (fabsf(d.REYNO) / 100000.0f) * powf(TSAVG / 288.0f, 0.62f);
    }
    const int NRW = A1(d.NROW, j);
    if (i == d.IMID && k == d.KMID && j == A1(d.JTE, NRW)) {
        const float vx = d.VX[n], vr = d.VR[n], wt = d.WT[n];
        const float WABS = sqrtf(vx * vx + vr * vr + wt * wt);
        const float ROVEXIT = d.RO[n] * WABS;
        saw_scalars(d)[NRW - 1] = A1(d.CHORD, NRW) * ROVEXIT / VISLAM;
    }
    float VISTOT = VISLAM * (1.0f + d.FST_RAT[n]) + TURBVIS_WALL;
    float VISLIM = d.TURBVIS_LIM * VISLAM;
    if (VISTOT > VISLIM) VISTOT = VISLIM;
    const float VISKLAM = VISLAM / ROAVG;
    saw(d, SAW_DYN_VIS_ML)[n] = VISTOT - VISLAM;
    if (d.IF_RESTART == 0 && nstep == 1) d.TRANS_DYN_VIS[n] = transvis_in(d, VISLAM);
    if (nstep == 1) d.TRANS_KVIS[n] = d.TRANS_DYN_VIS[n] / ROAVG;
    float TRANSKVIS = d.TRANS_KVIS[n];
    float XI = TRANSKVIS / VISKLAM;
    if (XI < 1.1f) XI = 1.1f;
    if (XI > d.TURBVIS_LIM) XI = d.TURBVIS_LIM;
    const float XI3 = XI * XI * XI;
    const float FV1 = XI3 / (XI3 + 357.9f);
    const float TRANSVISLIM = VISLIM / ROAVG / FV1;
    if (TRANSKVIS > TRANSVISLIM) TRANSKVIS = TRANSVISLIM;
    const float VISTRU = TRANSKVIS * FV1 * ROAVG;
    VISTOT = VISTRU + VISLAM;
    VISLIM = d.TURBVIS_LIM * VISLAM;
    if (VISTOT > VISLIM) VISTOT = VISLIM;
    d.VISC_RAT[n] = VISTOT / VISLAM;
    d.VISC_LAM[n] = VISLAM;
    d.VISC_TURB[n] = VISTOT - VISLAM;
}

// DO 1500: gradient of the kinematic transported viscosity (J = 2..JM-1)
__global__ void __launch_bounds__(SA_BS) k_sa_grad(const __grid_constant__ Dev d, int init_call) {
    pdl_wait();
    if (!init_call && !d.ctl->do_loss) return;
    int i, j, k;
    if (!sa_cell(d, blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    if (j > d.JMM1) return;
    const int n = ix3(d, i, j, k);
    float DX_, DR_, DT_;
    gradcell(d, i, j, k, d.TRANS_KVIS, DX_, DR_, DT_);
    float g = DX_ * DX_ + DR_ * DR_ + DT_ * DT_;
    const float VISCEFF = d.TRANS_KVIS[n] + d.VISC_LAM[n];
    float gx = VISCEFF * DX_, gr = VISCEFF * DR_, gt = VISCEFF * DT_;
    const int J1 = A1(d.JSTART, A1(d.NROW, j));
    if (j == J1 || j == J1 - 1) g = gx = gr = gt = 0.0f;
    saw(d, SAW_GRAD_TVIS)[n] = g;
    saw(d, SAW_TVGX)[n] = gx;
    saw(d, SAW_TVGR)[n] = gr;
    saw(d, SAW_TVGT)[n] = gt;
}

// The helicity and pressure-gradient factors of DO 1000 are scalars in the
// reference: DO 1600 reads the values of the loop's last cell (IMM1, JM,
// KMM1).  PTERM there uses the laminar viscosity as the loop left it on the
// cell before (IMM1-1, JM, KMM1).
__global__ void k_sa_lastcell(const __grid_constant__ Dev d, int init_call) {
    pdl_wait();
    const DevCtl *c = d.ctl;
    if (!init_call && !c->do_loss) return;
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int i = d.IMM1, j = d.JM, k = d.KMM1;
    const int n = ix3(d, i, j, k);
    const CellGrad g = cell_grad(d, i, j, k);
    float VORTX, VORTR, VORTT;
    float VORT = cell_vort(d, g, j, A2(d.RAVG_CELL, j, k), VORTX, VORTR, VORTT);
    if (A1(d.INDMIX, j) == 1) VORT = saw(d, SAW_ABS_VORT)[ix3(d, i, j - 1, k)];
    const int sJ = d.IM, sK = d.IM * d.JM;
    auto sum8 = [&](const float *A) {
        return A[n] + A[n + 1] + A[n + 1 + sK] + A[n + sK] + A[n - sJ] + A[n + 1 - sJ] + A[n + 1 - sJ + sK] + A[n - sJ + sK];
    };
    const float WTAVG = sum8(d.WT), VXAVG = sum8(d.VX), VRAVG = sum8(d.VR);
    float WREL = sqrtf(VXAVG * VXAVG + VRAVG * VRAVG + WTAVG * WTAVG);
    float *sc = saw_scalars(d);
    if (d.FAC_VORT > 0.001f) {
        const float HELICITY = (VXAVG * VORTX + VRAVG * VORTR + WTAVG * VORTT) / (WREL * VORT);
        sc[64] = 1.0f + d.FAC_VORT * tanhf(3.0f * HELICITY * HELICITY);
    }
    if (d.FAC_PGRAD > 0.001f) {
        const float a = A3(d.VX, d.IMID, j, k), b = A3(d.VR, d.IMID, j, k), cc = A3(d.WT, d.IMID, j, k);
        const float WLIM = 0.1f * sqrtf(a * a + b * b + cc * cc);
        if (WREL < WLIM) WREL = WLIM;
        WREL = 0.125f * WREL;
        float PGRAD = d.DPDS_CELL[n];
        if (PGRAD < 0.0f) PGRAD = 0.0f;
        const float VISLAM = d.REYNO < 0.0001f ? d.VISC_LAM[ix3(d, i - 1, j, k)] : c->VISLAM;
        const float ROAVG = d.ROAVG_CELL[n];
        float PTERM = PGRAD * VISLAM / (ROAVG * ROAVG * WREL * WREL * WREL);
        PTERM = PTERM * sc[A1(d.NROW, j) - 1];
        sc[65] = 1.0f + d.FAC_PGRAD * tanhf(PTERM * PTERM);
    }
}

// DO 1600: the source term of the transport equation, relaxed by RF_VIS
__global__ void __launch_bounds__(SA_BS) k_sa_source(const __grid_constant__ Dev d, int init_call) {
    pdl_wait();
    const DevCtl *c = d.ctl;
    if (!init_call && !c->do_loss) return;
    int i, j, k;
    if (!sa_cell(d, blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const int n = ix3(d, i, j, k);
    const float CW2 = 0.3f, SIGMA = 0.6667f, CB2 = 0.622f, CB1 = 0.1355f;
    const float CW1 = 0.80607f + 2.433f;
    const float FST0 = d.FAC_ST0 * CB1, FST1 = d.FAC_ST1 / SIGMA, FST2 = d.FAC_ST2 * CB2 / SIGMA;
    const float FST3 = d.FAC_ST3 * CW1;
    const float FSTMIX = d.FAC_STMIX / 100000.0f;
    const float RF_VIS = init_call ? 1.0f : d.RF_VIS;
    const float RF_VIS1 = 1.0f - RF_VIS;
    const float FYPLUS = fyplus_sa(d.Y_PLUS[n], d.YPLAM, d.YPTURB);
    float TVISDDX, TVISDDR, TVISDDT, d1, d2;
    gradcell(d, i, j, k, saw(d, SAW_TVGX), TVISDDX, d1, d2);
    gradcell(d, i, j, k, saw(d, SAW_TVGR), d1, TVISDDR, d2);
    gradcell(d, i, j, k, saw(d, SAW_TVGT), d1, d2, TVISDDT);
    const float ROAVG = d.ROAVG_CELL[n];
    const float TVIS = d.TRANS_KVIS[n];
    const float TVORT = saw(d, SAW_ABS_VORT)[n];
    float ST0 = FST0 * TVORT * TVIS;
    const float *sc = saw_scalars(d);
    if (d.FAC_VORT > 0.001f) ST0 = ST0 * sc[64];
    if (d.FAC_PGRAD > 0.001f) ST0 = ST0 * sc[65];
    ST0 = ST0 * FYPLUS;
    const float ST1 = FST1 * (TVISDDX + TVISDDR + TVISDDT);
    const float ST2 = FST2 * saw(d, SAW_GRAD_TVIS)[n];
    const float DW = d.DWALLSQ[n];
    float TAU = 5.9488f * TVIS / TVORT / DW;
    if (TAU > 1.2f) TAU = 1.2f;
    if (TAU < 0.001f) TAU = 0.001f;
    const float G = TAU + CW2 * (TAU * TAU * TAU * TAU * TAU * TAU - TAU);
    const float G6CW6 = G * G * G * G * G * G / 64.0f;
    const float FW = G * powf((1.0f + 0.015625f) / (1.0f + G6CW6), 0.166667f);
    const float ST3 = FST3 * FW * TVIS * TVIS / DW;
    const float ST_MIXL = FSTMIX * (saw(d, SAW_DYN_VIS_ML)[n] - d.VISC_TURB[n]) / d.STEP[n];
    float ts = RF_VIS1 * d.T_SOURCE[n] + RF_VIS * (ROAVG * (ST0 + ST1 + ST2 - ST3) * d.VOL[n] + ST_MIXL);
    if (j > 2 && A1(d.INDMIX, j - 1) == 1) ts = 0.0f;
    if (j > 2 && A1(d.INDMIX, j - 2) == 1) ts = 0.0f;
    d.T_SOURCE[n] = ts;
}

// DO 160: in laminar regions the source pulls the turbulent viscosity
// towards a profile rising from the wall.  One CTA per J plane: the hub and
// casing columns of every I first, then the I = 1 and I = IM lines of every
// K, as the reference orders them.
__global__ void __launch_bounds__(128) k_sa_transition(const __grid_constant__ Dev d, int init_call) {
    pdl_wait();
    DevCtl *c = d.ctl;
    if (!init_call && !c->do_loss) return;
    const int j = blockIdx.x + 2;
    const int NRW = A1(d.NROW, j);
    const int JROW = j - A1(d.JSTART, NRW) + 1;
    const int IMID = d.IMID, KMID = d.KMID, IMM1 = d.IMM1, KMM1 = d.KMM1, IM = d.IM, KM = d.KM;
    const int IEND1 = IMID / 2, IENDM = IMM1 - IEND1, KEND1 = KMID / 2, KENDM = KMM1 - KEND1;
    const float FTRANS = d.FTRANS;
    const bool ftr = FTRANS < 0.1f;
    const float *VR = d.VISC_RAT, *VT = d.VISC_TURB, *ST = d.STEP;
    float *TS = d.T_SOURCE;
    auto damp = [&](int n, float TVSPEC) { TS[n] = TS[n] - (VT[n] - TVSPEC) / ST[n] / 100000.0f; };
    auto laminar = [&](bool upstream, int n0, int stride, int cnt) {
        if (upstream) return true;
        float RMAX = 0.0f;
        for (int q = 0; q < cnt; ++q) {
            const float r = VR[n0 + q * stride];
            if (!(r < RMAX)) RMAX = r;
        }
        return !(RMAX > FTRANS);
    };
    const int sK = d.IM * d.JM;
    const int JTRHUB = A1(d.JTRAN_K1, NRW), JTRTIP = A1(d.JTRAN_KM, NRW);
    for (int i = threadIdx.x + 1; i <= IMM1; i += blockDim.x) {
        if (!(JTRHUB <= 1 && ftr) && laminar(JROW < JTRHUB, ix3(d, i, j, 1), sK, KEND1)) {
            const float TVEDGE = VT[ix3(d, i, j, KEND1)];
            for (int k = 1; k <= KEND1; ++k) {
                float FK = (float)(KEND1 + 1 - k) / (float)KEND1;
                FK = FK * FK * (3.0f - 2.0f * FK);
                damp(ix3(d, i, j, k), FK * TVEDGE);
            }
        }
        if (!(JTRTIP <= 1 && ftr) && laminar(JROW < JTRTIP, ix3(d, i, j, KENDM), sK, KMM1 - KENDM + 1)) {
            const float TVEDGE = VT[ix3(d, i, j, KENDM)];
            for (int k = KENDM; k <= KMM1; ++k) {
                float FK = (float)(k + 1 - KENDM) / (float)(KM - KENDM);
                FK = FK * FK * (3.0f - 2.0f * FK);
                damp(ix3(d, i, j, k), FK * TVEDGE);
            }
        }
    }
    __syncthreads();
    const int JTRLOW = A1(d.JTRAN_I1, NRW), JTRUP = A1(d.JTRAN_IM, NRW), JLEROW = A1(d.JLE, NRW);
    for (int k = threadIdx.x + 1; k <= KMM1; k += blockDim.x) {
        if (!(JTRLOW <= 1 && ftr) && !(j <= JLEROW) &&
            laminar(JROW < JTRLOW || j < JLEROW, ix3(d, 1, j, k), 1, IEND1)) {
            const float TVEDGE = VT[ix3(d, IEND1, j, k)];
            for (int i = 1; i <= IEND1; ++i) {
                float FI = (float)(IEND1 + 1 - i) / (float)IEND1;
                FI = FI * FI * (3.0f - 2.0f * FI);
                damp(ix3(d, i, j, k), FI * TVEDGE);
            }
        }
        if (!(JTRUP <= 1 && ftr) && !(j <= JLEROW) &&
            laminar(JROW < JTRUP, ix3(d, IENDM, j, k), 1, IMM1 - IENDM + 1)) {
            const float TVEDGE = VT[ix3(d, IENDM, j, k)];
            for (int i = IENDM; i <= IMM1; ++i) {
                float FI = (float)(i + 1 - IENDM) / (float)(IM - IENDM);
                FI = FI * FI * (3.0f - 2.0f * FI);
                damp(ix3(d, i, j, k), FI * TVEDGE);
            }
        }
    }
    // the COMMON VISLAM leaves DO 190 as the last cell's laminar viscosity
    if (blockIdx.x == 0 && threadIdx.x == 0 && d.REYNO < 0.0001f) c->VISLAM = A3(d.VISC_LAM, IMM1, d.JM, KMM1);
}

// ---------------------------------------------------------------------
// transport of the turbulent viscosity (LOOP 4279-4347, TSTEP 5736-5777)
// ---------------------------------------------------------------------
// fluxes and source, doubled for a larger effective time step (4279-4330)
__global__ void __launch_bounds__(SA_BS) k_sa_fluxes(const __grid_constant__ Dev d) {
    pdl_wait();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.IMM1 * d.JM * d.KMM1) return;
    const int i = t % d.IMM1 + 1, q = t / d.IMM1, j = q % d.JM + 1, k = q / d.JM + 1;
    const VarSet &V = d.var[V_SA];
    const float *TK = d.TRANS_KVIS;
    const int n = ix3(d, i, j, k);
    int JP1 = j + 1;
    if (j == d.JM) JP1 = d.JM;
    if (j == 1) JP1 = 1;
    if (A1(d.INDMIX, j) == 1) JP1 = j;
    V.XF[n] = d.FLOWX[n] * (TK[n] + TK[ix3(d, i, JP1, k)]);
    if (j < 2) return;
    V.SR[n] = -2.0f * d.T_SOURCE[n];
    if (i >= 2) {
        V.TF[n] = d.FLOWT[n] * (TK[n - 1] + TK[n]);
    } else {
        const float tf = d.FLOWT[n] * (TK[ix3(d, d.IMM1, j, k)] + TK[n]);
        V.TF[n] = tf;
        V.TF[ix3(d, d.IM, j, k)] = tf;
    }
    const int sK = d.IM * d.JM;
    V.RF[n] = k >= 2 ? d.FLOWR[n] * (TK[n - sK] + TK[n]) : 0.0f;
    if (k == d.KMM1) V.RF[n + sK] = 0.0f;
}

// the negative feedback's damping and the cell-centred update D += STORE
// (1525, 1600); one CTA per J plane, the row means formed as k_ts_update does
__global__ void __launch_bounds__(SA_BS) k_sa_update(const __grid_constant__ Dev d) {
    pdl_wait();
    const VarSet &V = d.var[V_SA];
    __shared__ float s_blk[64];
    __shared__ float chg[64];
    const int j = blockIdx.x + 2;
    const int IMM1 = d.IMM1, KMM1 = d.KMM1;
    const DevCtl *ctl = d.ctl;
    const int damp_on = ctl->damp_on;
    const float DAMP = ctl->DAMP;
    if (damp_on) {
        if (d.REDUCE_ORDER == 1) {
            for (int r = threadIdx.x; r < d.NROWS; r += SA_BS) s_blk[r] = V.AVG_BLK[r];
        } else {
            const int ro = d.REDUCE_ORDER;
            const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
            for (int nr = w + 1; nr <= d.NROWS; nr += SA_BS / 32) {
                const int JST = A1(d.JSTART, nr) + 1, JEN = A1(d.JMIX, nr) - 1;
                df s = df_of(0.0f);
                for (int jj = JST + l; jj <= JEN; jj += 32) s = dacc(ro, s, V.pabs[jj - 1]);
                for (int o = 16; o > 0; o >>= 1) s = dacc(ro, s, df_shfl_down(s, o));
                if (l == 0) chg[nr - 1] = df_val(s) / (float)(IMM1 * KMM1 * (JEN - JST + 1));
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                const int NROWS = d.NROWS;
                if (NROWS == 1) s_blk[0] = chg[0];
                if (NROWS == 2) {
                    s_blk[1] = 0.5f * (chg[0] + chg[1]);
                    s_blk[0] = s_blk[1];
                }
                if (NROWS > 2) {
                    for (int nr = 2; nr <= NROWS - 1; ++nr)
                        s_blk[nr - 1] = 0.25f * (chg[nr - 2] + chg[nr]) + 0.5f * chg[nr - 1];
                    s_blk[NROWS - 1] = 0.5f * (chg[NROWS - 2] + chg[NROWS - 1]);
                    s_blk[0] = 0.5f * (chg[0] + chg[1]);
                }
            }
        }
        __syncthreads();
    }
    const float blk = damp_on ? s_blk[A1(d.NROW, j) - 1] : 1.0f;
    for (int t = threadIdx.x; t < IMM1 * KMM1; t += SA_BS) {
        const int i = t % IMM1 + 1, k = t / IMM1 + 1;
        const int n = ix3(d, i, j, k);
        float v = V.ST[n];
        if (damp_on) {
            const float FDAMP = fabsf(v) / blk;
            v = v / (1.0f + FDAMP / DAMP);
        }
        V.D[n] = V.D[n] + v;
    }
}

// the row's last plane carried across each mixing plane with the decay
// TURBVIS_DAMP (1560-1591): one thread per (row interface, K)
__global__ void k_sa_mixtransfer(const __grid_constant__ Dev d) {
    pdl_wait();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (d.NROWS - 1) * d.KMM1) return;
    const int nr = t / d.KMM1 + 1, k = t % d.KMM1 + 1;
    float *D = d.var[V_SA].D;
    const int j = A1(d.JMIX, nr);
    const float FMULT = A1(d.TURBVIS_DAMP, nr);
    float AVG;
    if (d.REDUCE_ORDER != 0) {
        AVG = 0.0f;
        for (int i = 1; i <= d.IMM1; ++i) AVG = AVG + A1(d.FP, i) * A3(D, i, j, k);
    } else {
        double s = 0.0;
        for (int i = 1; i <= d.IMM1; ++i) s += (double)(A1(d.FP, i) * A3(D, i, j, k));
        AVG = (float)s;
    }
    for (int jav = j + 1; jav <= j + 2; ++jav)
        for (int i = 1; i <= d.IMM1; ++i) A3(D, i, jav, k) = FMULT * AVG;
}

// one SMOOTH_RESID pass (14852-14910) of the transported viscosity with
// SFTVIS = FAC_SFVIS * SFT: along J (dir 0), I (1) or K (2), src -> dst;
// cells outside every row are copied, and dir 3 copies every cell
__global__ void __launch_bounds__(SA_BS) k_sa_resid(const __grid_constant__ Dev d, int dir, int d_to_tm) {
    pdl_wait();
    const VarSet &V = d.var[V_SA];
    const float *__restrict__ src = d_to_tm ? V.D : V.TM;
    float *__restrict__ dst = d_to_tm ? V.TM : V.D;
    int i, j, k;
    if (!sa_cell(d, blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const int n = ix3(d, i, j, k);
    const float smfac = d.FAC_SFVIS * d.ctl->SFT;
    const float SFAC1 = 1.0f - smfac, SFACH = 0.5f * smfac;
    const int nr = A1(d.NROW, j);
    const int J1P1 = A1(d.JSTART, nr) + 1, J1P2 = J1P1 + 1, J2 = A1(d.JMIX, nr), J2M1 = J2 - 1;
    float v = src[n];
    if (j < J1P1 || j > J2) {
        dst[n] = v;
        return;
    }
#define S(ii, jj, kk) A3(src, ii, jj, kk)
    if (dir == 0) {
        if (j >= J1P2 && j <= J2M1) v = SFAC1 * v + SFACH * (S(i, j + 1, k) + S(i, j - 1, k));
        if (j == J1P1) v = S(i, J1P1, k) + SFACH * (S(i, J1P2, k) - S(i, J1P1, k));
        if (j == J2) v = S(i, J2, k) + SFACH * (S(i, J2M1, k) - S(i, J2, k));
    } else if (dir == 1) {
        const int IMM1 = d.IMM1, IMM2 = d.IMM2;
        if (i >= 2 && i <= IMM2) v = SFAC1 * v + SFACH * (S(i + 1, j, k) + S(i - 1, j, k));
        if (i == 1) v = S(1, j, k) + SFACH * (S(2, j, k) - S(1, j, k));
        if (i == IMM1) v = S(IMM1, j, k) + SFACH * (S(IMM2, j, k) - S(IMM1, j, k));
    } else if (dir == 2) {
        const int KMM1 = d.KMM1, KMM2 = d.KMM2;
        if (k >= 2 && k <= KMM2) v = SFAC1 * v + SFACH * (S(i, j, k + 1) + S(i, j, k - 1));
        if (k == 1) v = S(i, j, 1) + SFACH * (S(i, j, 2) - S(i, j, 1));
        if (k == KMM1) v = S(i, j, KMM1) + SFACH * (S(i, j, KMM2) - S(i, j, KMM1));
    }
#undef S
    dst[n] = v;
}

// the periodic (8000, ILAST = IM-1), tip-gap (510) and mixing-plane (100)
// averages of every (J, K) line of the transported viscosity
__global__ void __launch_bounds__(SA_BS) k_sa_fix(const __grid_constant__ Dev d) {
    pdl_wait();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.JM * d.KM) return;
    const int j = t % d.JM + 1, k = t / d.JM + 1;
    float *D = d.var[V_SA].D;
    const int IM = d.IM, KM = d.KM, ILAST = d.IMM1;
    const int n1 = ix3(d, 1, j, k), nl = ix3(d, ILAST, j, k);
    if (!(A1(d.IND, j) == 1 || A1(d.INDLE, j) == 1)) {
        const float v = 0.5f * (D[n1] + D[nl]);
        D[n1] = v;
        D[nl] = v;
    }
    const int nr = A1(d.NROW, j);
    if (KM != 2 && A1(d.KTIPS, nr) > 0) {
        int K1 = A1(d.KTIPS, nr), K2 = A1(d.KTIPE, nr);
        if (K1 == 1) K2 = K2 - 1;
        if (K2 == KM) K1 = K1 + 1;
        if (k >= K1 && k <= K2) {
            const float v = 0.5f * (D[n1] + D[nl]);
            D[n1] = v;
            D[nl] = v;
        }
    }
    if (d.IFMIX == 0) return;
    for (int r = 1; r <= d.NRWSM1; ++r) {
        const int jx = A1(d.JMIX, r);
        if (j != jx && j != jx + 1) continue;
        float s;
        if (d.REDUCE_ORDER != 0) {
            s = 0.0f;
            for (int i = 1; i <= d.IMM1; ++i) s = s + A1(d.FP, i) * (A3(D, i, j, k) + A3(D, i + 1, j, k));
        } else {
            double s64 = 0.0;
            for (int i = 1; i <= d.IMM1; ++i) s64 += (double)(A1(d.FP, i) * (A3(D, i, j, k) + A3(D, i + 1, j, k)));
            s = (float)s64;
        }
        s = 0.5f * s;
        for (int i = 1; i <= IM; ++i) A3(D, i, j, k) = s;
        break;
    }
}

// the floor on the transported viscosity and its kinematic value (4340-4347)
__global__ void __launch_bounds__(SA_BS) k_sa_floor(const __grid_constant__ Dev d) {
    pdl_wait();
    int i, j, k;
    if (!sa_cell(d, blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const int n = ix3(d, i, j, k);
    const float TRANSVISMIN = 0.1f * A3(d.VISC_LAM, d.IMID, 2, d.KMID);
    float v = d.TRANS_DYN_VIS[n];
    if (v < TRANSVISMIN) v = TRANSVISMIN;
    d.TRANS_DYN_VIS[n] = v;
    d.TRANS_KVIS[n] = v / d.ROAVG_CELL[n];
}

// the transported viscosity at inlet (4679-4689), after the inlet condition:
// each (I, K) divides by RO(IMID,1,KMID) as the reference's K, I loop has
// reached it, the value from before the condition for the points before
// (IMID, KMID)
__global__ void __launch_bounds__(SA_BS) k_sa_inlet(const __grid_constant__ Dev d) {
    pdl_wait();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.IM * d.KM) return;
    const int i = t % d.IM + 1, k = t / d.IM + 1;
    const float ro_old = saw_scalars(d)[66];
    const float ro = (k < d.KMID || (k == d.KMID && i < d.IMID)) ? ro_old : A3(d.RO, d.IMID, 1, d.KMID);
    const float tv = transvis_in(d, A3(d.VISC_LAM, i, 2, k));
    A3(d.TRANS_DYN_VIS, i, 1, k) = tv;
    A3(d.TRANS_DYN_VIS, i, 2, k) = tv;
    const float tk = tv / ro;
    A3(d.TRANS_KVIS, i, 1, k) = tk;
    A3(d.TRANS_KVIS, i, 2, k) = tk;
}

}  // namespace

size_t sa_work_floats(const Dev &d) { return sa_work_node_floats(d) + 64 + 8; }

void launch_sa_transport(const Dev &d, Launch L) {
    const unsigned nc = (unsigned)((d.IMM1 * (d.JM - 1) * d.KMM1 + SA_BS - 1) / SA_BS);
    const unsigned nf = (unsigned)((d.IMM1 * d.JM * d.KMM1 + SA_BS - 1) / SA_BS);
    launchk(L, k_sa_fluxes, dim3(nf), dim3(SA_BS), 0, d);
    mark(L, "k_sa_fluxes");
    launch_tstep_cells_prolong(d, L, V_SA, 1);
    launchk(L, k_sa_update, dim3(d.JM - 1), dim3(SA_BS), 0, d);
    mark(L, "k_sa_update");
    if (d.NROWS > 1) {
        launchk(L, k_sa_mixtransfer, dim3((unsigned)(((d.NROWS - 1) * d.KMM1 + 63) / 64)), dim3(64), 0, d);
        mark(L, "k_sa_mixtransfer");
    }
    // SMOOTH_RESID: J pass D -> TMP, I pass TMP -> D, K pass D -> TMP, and
    // the copy TMP -> D
    const int dirs[4][2] = {{0, 1}, {1, 0}, {2, 1}, {3, 0}};
    for (auto &p : dirs) {
        launchk(L, k_sa_resid, dim3(nc), dim3(SA_BS), 0, d, p[0], p[1]);
        mark(L, "k_sa_resid");
    }
    launchk(L, k_sa_fix, dim3((unsigned)((d.JM * d.KM + SA_BS - 1) / SA_BS)), dim3(SA_BS), 0, d);
    mark(L, "k_sa_fix");
    launchk(L, k_sa_floor, dim3(nc), dim3(SA_BS), 0, d);
    mark(L, "k_sa_floor");
}

void launch_sa_inlet(const Dev &d, Launch L) {
    launchk(L, k_sa_inlet, dim3((unsigned)((d.IM * d.KM + SA_BS - 1) / SA_BS)), dim3(SA_BS), 0, d);
    mark(L, "k_sa_inlet");
}

void launch_spal_loss(const Dev &d, Launch L, bool init_call) {
    const int ic = init_call ? 1 : 0;
    const unsigned nc = (unsigned)((d.IMM1 * (d.JM - 1) * d.KMM1 + SA_BS - 1) / SA_BS);
    launch_loss_prologue(d, L, init_call);
    launchk(L, k_sa_cells, dim3(nc), dim3(SA_BS), 0, d, ic);
    mark(L, "k_sa_cells");
    launchk(L, k_sa_grad, dim3(nc), dim3(SA_BS), 0, d, ic);
    mark(L, "k_sa_grad");
    if (d.FAC_PGRAD > 0.001f || d.YPLUSWALL < -10.0f) launch_pwallgrad(d, L, init_call);
    if (d.FAC_VORT > 0.001f || d.FAC_PGRAD > 0.001f) {
        launchk(L, k_sa_lastcell, dim3(1), dim3(32), 0, d, ic);
        mark(L, "k_sa_lastcell");
    }
    launchk(L, k_sa_source, dim3(nc), dim3(SA_BS), 0, d, ic);
    mark(L, "k_sa_source");
    launchk(L, k_sa_transition, dim3(d.JM - 1), dim3(128), 0, d, ic);
    mark(L, "k_sa_transition");
    launch_viscous_walls_and_forces(d, L, init_call);
}

}  // namespace mgpu
