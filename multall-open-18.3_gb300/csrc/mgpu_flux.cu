// mgpu_flux.cu -- per-step node kernels of the time-marching loop:
// step control, primitive recovery, the face fluxes of the five
// conservation equations, inlet/exit boundary conditions, PEFF, the density
// and Mach limiters and the mixing-plane relaxation.
//
// Each kernel restates one sweep of SUBROUTINE LOOP
// (multall-open-18.3.f:3664-5463) with one thread per node and the
// reference's floating-point expression order, so that (built without FMA
// contraction, as the reference is) the results match REAL*4 arithmetic.
// Periodic fix-ups that couple I=1 and I=IM are done by both end threads
// from the same raw values, so no thread waits on another.
#include "mgpu_internal.cuh"

namespace mgpu {

static inline unsigned grid_for(size_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

// ---------------------------------------------------------------------
// step control: NSTEP, the end test, the smoothing/damping ramp and FMIXUP
// (multall-open-18.3.f:3759-3815), and the viscosity update LOSS makes on
// entry (8088-8112).
// ---------------------------------------------------------------------
__global__ void k_step_begin(Dev d) {
    pdl_wait();
    DevCtl *c = d.ctl;
    int n = c->nstep + 1;
    c->nstep = n;
    int ifend = c->ifend;
    if (n == d.NSTEPS_MAX) ifend = 1;
    if (c->EAVG < d.CONLIM && c->ECONT < 0.01f) ifend = 1;
    if (fabsf(c->EMAX) < 4.0f * d.CONLIM && c->ECONT < 0.01f) ifend = 1;
    if (c->force_end) ifend = 1;
    c->ifend = ifend;
    if (!(d.IF_RESTART != 0 && n > 100)) {
        float FCHANGE = 1.0f - (float)(n - 1) / (float)d.NCHANGE;
        if (FCHANGE > 0.0f) {
            c->SFT = d.SFTIN + 0.02f * FCHANGE;
            c->SFX = d.SFXIN + 0.02f * FCHANGE;
            c->DAMP = d.DAMPIN * (1.0f - 0.75f * FCHANGE);
        }
        float SFT = c->SFT, SFX = c->SFX;
        c->SFT1 = 1.0f - SFT;
        c->SFTH = 0.5f * SFT;
        c->SFX1 = 1.0f - SFX;
        c->SFXH = 0.5f * SFX;
        c->SFX14 = 0.25f * SFX;
        c->SFXB = d.FSMTHB * SFX;
        c->SFXB1 = 1.0f - c->SFXB;
        c->SFXBH = 0.5f * c->SFXB;
        c->SFXHM1 = 1.0f - c->SFXH;
        float FM = 1.0f + (d.FACMIXUP - 1.0f) * (float)(d.NMIXUP - n) / (float)d.NMIXUP;
        if (FM < 1.0f) FM = 1.0f;
        c->FMIXUP = FM * FM;
    }
    c->do_tail = (n % 5 == 0) || ifend == 1;
    c->do_loss = (d.ILOS == 10 || (d.ILOS >= 100 && d.ILOS < 300)) && (n % d.NLOS == 0) && !d.FROZEN;
    c->damp_on = !(c->DAMP < 2.0f || c->DAMP > 100.0f);
    if (d.use_cond) {
        if (d.ILOS != 0) cudaGraphSetConditional((cudaGraphConditionalHandle)d.cond_loss, c->do_loss ? 1u : 0u);
        cudaGraphSetConditional((cudaGraphConditionalHandle)d.cond_tail, c->do_tail ? 1u : 0u);
    }
    if (c->do_tail) {
        c->mon.vrms = 0.0;
        c->mon.vmax_key = 0ull;
        c->mon.eavg_sum = 0.0;
        c->mon.emax_key = 0ull;
        c->mon.health = 0;
    }
}

void launch_step_begin(const Dev &d, Launch L) {
    launchk(L, k_step_begin, dim3(1), dim3(1), 0, d);
    mark(L, "k_step_begin");
}

// ---------------------------------------------------------------------
// primitive variables (7450) and P, HO, T (5900); with the 5-step tail
// also the sum and the maximum of |W|^2 (5910, uses the previous WT).
// ---------------------------------------------------------------------
template <int BS>
__device__ inline void block_reduce_sum_key(int order, double s, unsigned long long key, double *out_s,
                                            unsigned long long *out_k) {
    __shared__ double ss[BS / 32];
    __shared__ unsigned long long sk[BS / 32];
    for (int o = 16; o > 0; o >>= 1) {
        s = racc(order, s, __shfl_down_sync(0xffffffffu, s, o));
        unsigned long long ok = __shfl_down_sync(0xffffffffu, key, o);
        key = ok > key ? ok : key;
    }
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        ss[w] = s;
        sk[w] = key;
    }
    __syncthreads();
    if (w == 0) {
        s = l < BS / 32 ? ss[l] : 0.0;
        key = l < BS / 32 ? sk[l] : 0ull;
        for (int o = 16; o > 0; o >>= 1) {
            s = racc(order, s, __shfl_down_sync(0xffffffffu, s, o));
            unsigned long long ok = __shfl_down_sync(0xffffffffu, key, o);
            key = ok > key ? ok : key;
        }
        if (l == 0) {
            *out_s = s;
            *out_k = key;
        }
    }
}

constexpr int PRIM_BS = 256;

__global__ void __launch_bounds__(PRIM_BS) k_prim(Dev d) {
    pdl_wait();
    size_t n = (size_t)blockIdx.x * PRIM_BS + threadIdx.x;
    size_t N = (size_t)d.IM * d.JM * d.KM;
    int do_tail = d.ctl->do_tail;
    double eke_s = 0.0;
    unsigned long long key = 0ull;
    if (n < N) {
        int i, j, k;
        node_ijk(d, n, i, j, k);
        if (j >= 2) {
            // every load before the first store (a store through one Dev
            // pointer keeps later loads through another behind it)
            const bool thermo = j <= d.JMM1;
            const float rr = A2(d.R, j, k), RONOW = d.RO[n], rovx = d.ROVX[n], rovr = d.ROVR[n];
            const float rorvt = d.RORVT[n], roe = thermo ? d.ROE[n] : 0.0f, wt = do_tail ? d.WT[n] : 0.0f;
            float RRNOW = 1.0f / rr;
            float RECIP = 1.0f / RONOW;
            float vx = rovx * RECIP;
            float vr = rovr * RECIP;
            float rovt = rorvt * RRNOW;
            float vt = rovt * RECIP;
            d.VX[n] = vx;
            d.VR[n] = vr;
            d.ROVT[n] = rovt;
            d.VT[n] = vt;
            if (do_tail) {
                float EKE = vr * vr + wt * wt + vx * vx;
                eke_s = (double)EKE;
                key = max_key(EKE, n);
            }
            if (thermo) {
                float EKE = 0.5f * (vr * vr + vt * vt + vx * vx);
                float TSTATIC = (roe / RONOW - EKE) / d.CV;
                d.P[n] = RONOW * d.RGAS * TSTATIC;
                d.HO[n] = d.CP * TSTATIC + EKE;
                d.T_STATIC[n] = TSTATIC;
            }
        }
    }
    if (do_tail)
        block_reduce_sum_key<PRIM_BS>(d.REDUCE_ORDER, eke_s, key, &d.part_sum[blockIdx.x], &d.part_key[blockIdx.x]);
}

void launch_prim(const Dev &d, Launch L) {
    size_t N = (size_t)d.IM * d.JM * d.KM;
    launchk(L, k_prim, dim3(grid_for(N, PRIM_BS)), dim3(PRIM_BS), 0, d);
    mark(L, "k_prim");
}

// ---------------------------------------------------------------------
// mass fluxes FLOWX/FLOWT/FLOWR, ROWT and WT (5020-5045)
// ---------------------------------------------------------------------
__device__ inline float rowt_at(const Dev &d, int i, int j, int k) {
    return A3(d.ROVT, i, j, k) - A2(d.UBLADE, j, k) * A3(d.RO, i, j, k);
}

__device__ inline float flowt_raw(const Dev &d, int i, int j, int k) {
    float AVGRVX = A3(d.ROVX, i, j, k) + A3(d.ROVX, i, j - 1, k) + A3(d.ROVX, i, j - 1, k + 1) + A3(d.ROVX, i, j, k + 1);
    float AVGRVT = rowt_at(d, i, j, k) + rowt_at(d, i, j - 1, k) + rowt_at(d, i, j - 1, k + 1) + rowt_at(d, i, j, k + 1);
    float AVGRVR = A3(d.ROVR, i, j, k) + A3(d.ROVR, i, j - 1, k) + A3(d.ROVR, i, j - 1, k + 1) + A3(d.ROVR, i, j, k + 1);
    return (AVGRVX * A3(d.ABX, i, j, k) + AVGRVT * A2(d.ABT, j, k) + AVGRVR * A3(d.ABR, i, j, k)) * 0.25f;
}

// energy flux of the blade-wise face (I, J, K) whose mass flux is flowt
__device__ inline float tflux_energy_at(const Dev &d, float flowt, int i, int j, int k) {
    float AVGHO = A3(d.HO, i, j, k) + A3(d.HO, i, j - 1, k) + A3(d.HO, i, j - 1, k + 1) + A3(d.HO, i, j, k + 1);
    float AVGPB = A3(d.PEFF, i, j, k) + A3(d.PEFF, i, j - 1, k) + A3(d.PEFF, i, j - 1, k + 1) + A3(d.PEFF, i, j, k + 1);
    return (flowt * AVGHO + A2(d.WRABT, j, k) * AVGPB) * 0.25f;
}

__global__ void k_flux_mass_energy(Dev d) {
    pdl_wait();
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, (size_t)n, i, j, k);
    const VarSet &V = d.var[V_ROE];
    // results are kept in registers and stored at the end, so that no store
    // orders the loads of a later section behind it
    const bool hx = i < d.IM && k < d.KM, ht = j >= 2 && k < d.KM, hr = i < d.IM && j >= 2;
    const bool hs = hx && j >= 2;
    float fx = 0.0f, ft = 0.0f, fr = 0.0f;
    float xf = 0.0f, src = 0.0f, rf = 0.0f, tf = 0.0f;
    // mass fluxes (5020-5045)
    if (hx) {
        float AVGRVX = A3(d.ROVX, i, j, k) + A3(d.ROVX, i, j, k + 1) + A3(d.ROVX, i + 1, j, k) + A3(d.ROVX, i + 1, j, k + 1);
        float AVGRVR = A3(d.ROVR, i, j, k) + A3(d.ROVR, i, j, k + 1) + A3(d.ROVR, i + 1, j, k) + A3(d.ROVR, i + 1, j, k + 1);
        fx = 0.25f * (AVGRVX * A3(d.AQX, i, j, k) + AVGRVR * A3(d.AQR, i, j, k));
    }
    const float ro = d.RO[n];
    const float rowt = d.ROVT[n] - A2(d.UBLADE, j, k) * ro;
    const float wt = rowt / ro;
    bool tbal = false;          // periodic I = 1 / IM face: FLOWT there is the balanced value ft at both
    if (ht) {
        ft = flowt_raw(d, i, j, k);
        if (i == 1 || i == d.IM) {
            if (A1(d.IND, j) != 1) {
                float f1 = (i == 1) ? ft : flowt_raw(d, 1, j, k);
                float fm = (i == d.IM) ? ft : flowt_raw(d, d.IM, j, k);
                ft = 0.5f * (f1 + fm);
                tbal = true;
            } else {
                int nr = A1(d.NROW, j);
                if (k >= A1(d.KS1, nr) && k <= A1(d.KS2, nr)) ft = 0.0f;
            }
        }
    }
    if (hr) {
        if (k >= 2 && k <= d.KMM1) {
            float AVGRVX = A3(d.ROVX, i, j, k) + A3(d.ROVX, i, j - 1, k) + A3(d.ROVX, i + 1, j - 1, k) + A3(d.ROVX, i + 1, j, k);
            float AVGRVR = A3(d.ROVR, i, j, k) + A3(d.ROVR, i, j - 1, k) + A3(d.ROVR, i + 1, j - 1, k) + A3(d.ROVR, i + 1, j, k);
            fr = 0.25f * (AVGRVX * A3(d.ASX, i, j, k) + AVGRVR * A3(d.ASR, i, j, k));
        }
    }
    // energy fluxes (5501-5503) from this node's mass fluxes, and their
    // periodic balance (900): with IND(J) != 1 the mass flux of both edge
    // faces is the balanced ft, so the two edge energy fluxes are formed here
    if (hx) {
        float AVGHO = A3(d.HO, i, j, k) + A3(d.HO, i, j, k + 1) + A3(d.HO, i + 1, j, k) + A3(d.HO, i + 1, j, k + 1);
        xf = fx * AVGHO * 0.25f;
        if (hs) src = d.QSOURCE[n];
    }
    if (hr) {
        float AVGHO = 0.25f * (A3(d.HO, i, j, k) + A3(d.HO, i, j - 1, k) + A3(d.HO, i + 1, j - 1, k) + A3(d.HO, i + 1, j, k));
        rf = fr * AVGHO;
    }
    if (ht) {
        tf = tflux_energy_at(d, ft, i, j, k);
        if (tbal) {
            float t1 = (i == 1) ? tf : tflux_energy_at(d, ft, 1, j, k);
            float tm = (i == d.IM) ? tf : tflux_energy_at(d, ft, d.IM, j, k);
            tf = 0.5f * (t1 + tm);
        }
    }
    if (hx) d.FLOWX[n] = fx;
    d.ROWT[n] = rowt;
    d.WT[n] = wt;
    if (ht) d.FLOWT[n] = ft;
    if (hr) d.FLOWR[n] = fr;
    if (hx) V.XF[n] = xf;
    if (hs) V.SR[n] = src;
    if (hr) V.RF[n] = rf;
    if (ht) V.TF[n] = tf;
}

void launch_flux_mass_energy(const Dev &d, Launch L) {
    size_t N = (size_t)d.IM * d.JM * d.KM;
    launchk(L, k_flux_mass_energy, dim3(grid_for(N, 256)), dim3(256), 0, d);
    mark(L, "k_flux_mass_energy");
}


// ---------------------------------------------------------------------
// inlet and exit boundary conditions (4476-4734).  k_bc_sums: one warp per
// K line forms the pitchwise sums in the reference's sequential order (the
// lanes load, lane 0 adds in I order), then one thread runs the radial-
// equilibrium recurrence for PD(K) (4533-4541).  k_bc_apply: one thread per
// (I,K) sets the inlet and exit states.
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_bc_sums(Dev d) {
    pdl_wait();
    // per warp: the four pitchwise terms of one K line, [4][IMM1], and with
    // PLATE_LOSS the two ROV_m**2 terms at JM, [2][IM]
    extern __shared__ float bsm[];
    __shared__ float s_sum[512], s_pd[512], s_r[512], s_rov[514];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int IM = d.IM, IMM1 = d.IMM1, KM = d.KM;
    const bool plate = d.PLATE_LOSS > 0.001f;
    float *tt = bsm + (size_t)w * (4 * IMM1 + 2 * IM);
    for (int k = w + 1; k <= KM; k += nw) {
        const float RJM = A2(d.R, d.JM, k);
        for (int i = l + 1; i <= IMM1; i += 32) {
            float fp = A1(d.FP, i);
            tt[i - 1] = 0.5f * (A3(d.P, i, 2, k) + A3(d.P, i + 1, 2, k)) * fp;
            tt[IMM1 + i - 1] = 0.5f * (A3(d.P, i, 3, k) + A3(d.P, i + 1, 3, k)) * fp;
            tt[2 * IMM1 + i - 1] = 0.5f * (A3(d.P, i, d.JMM1, k) + A3(d.P, i + 1, d.JMM1, k)) * fp;
            tt[3 * IMM1 + i - 1] = 0.5f * fp *
                                   (A3(d.ROVT, i, d.JM, k) * A3(d.VT, i, d.JM, k) +
                                    A3(d.ROVT, i + 1, d.JM, k) * A3(d.VT, i + 1, d.JM, k)) /
                                   RJM;
        }
        if (plate)
            for (int i = l + 1; i <= IM; i += 32) {
                tt[4 * IMM1 + i - 1] = A3(d.ROVX, i, d.JM, k) * A3(d.VX, i, d.JM, k);
                tt[4 * IMM1 + IM + i - 1] = A3(d.ROVR, i, d.JM, k) * A3(d.VR, i, d.JM, k);
            }
        __syncwarp();
        // lanes 0..3 each add one term over I in the reference's order; lane 4
        // forms ROVMSQ(K) = sum of ROVX*VX + ROVR*VR (4476-4482)
        if (l < 4) {
            const float *t = tt + l * IMM1;
            float sum = 0.0f;
            for (int i = 0; i < IMM1; ++i) sum = sum + t[i];
            if (l < 3) d.BCBUF[l * KM + k - 1] = sum;   // PAVG2, PAVG3, PAVGOUT
            else s_sum[k - 1] = sum;
        } else if (l == 4 && plate) {
            const float *a = tt + 4 * IMM1, *b = a + IM;
            float sum = 0.0f;
            for (int i = 0; i < IM; ++i) {
                sum = sum + a[i];
                sum = sum + b[i];
            }
            s_rov[k] = sum;
        }
        __syncwarp();
    }
    // the recurrence runs on shared copies of PD and R(JM, K): one thread,
    // no global round trip per K
    for (int k = threadIdx.x; k < KM; k += blockDim.x) {
        s_pd[k] = d.PD[k];
        s_r[k] = A2(d.R, d.JM, k + 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        DevCtl *c = d.ctl;
        // throttle exit condition (4488-4505): the exit pressures follow the
        // exit mass flow of the last tail
        const bool throttle = d.THROTTLE_EXIT > 0.001f;
        float PTHROTTLE = 0.0f, PDMID = 0.0f;
        if (c->nstep > 100 && throttle) {
            float FFLOW = c->CHECK_FLOW_JM / d.THROTTLE_MAS;
            PTHROTTLE = c->THROTTLE_PRES * FFLOW * FFLOW;
            c->PDOWN_TIP = d.RFTHROTL1 * c->PDOWN_TIP + d.RFTHROTL * PTHROTTLE;
            c->PDOWN_HUB = d.RFTHROTL1 * c->PDOWN_HUB + d.RFTHROTL * PTHROTTLE;
            PDMID = PTHROTTLE - s_pd[d.KMID - 1];
            float RF_P = 0.02f * d.RFTHROTL;
            c->THROTTLE_PRES = (1.0f - RF_P) * c->THROTTLE_PRES + RF_P * PTHROTTLE;
        }
        const float PDOWN_HUB = c->PDOWN_HUB;
        float PDIFF = 0.0f;
        if (d.IPOUT == -1) PDIFF = c->PDOWN_TIP - s_pd[KM - 1];
        float SUMP = 0.0f;
        for (int k = 1; k <= KM; ++k) {
            if (d.IPOUT <= 0) {
                s_pd[0] = PDOWN_HUB;
                if (k != 1) {
                    float DP = (s_sum[k - 1] + SUMP) * 0.5f * (s_r[k - 1] - s_r[k - 2]);
                    s_pd[k - 1] = 0.9f * s_pd[k - 1] + 0.1f * (s_pd[k - 2] + DP);
                }
                SUMP = s_sum[k - 1];
                if (d.IPOUT == -1) s_pd[k - 1] = s_pd[k - 1] + PDIFF;
            }
            if (d.IPOUT >= 1 && throttle) s_pd[k - 1] = s_pd[k - 1] + d.RFTHROTL * PDMID;
            if (plate) s_pd[k - 1] = s_pd[k - 1] + 0.01f * d.PLATE_LOSS * (s_rov[k] - s_rov[d.KMID]);
            // the exit update of this K uses PD(K) as it is now; PD(1) is reset
            // again at the next K
            d.BCBUF[3 * KM + k - 1] = s_pd[k - 1];
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < KM; k += blockDim.x) d.PD[k] = s_pd[k];
}

__global__ void k_bc_apply(Dev d) {
    pdl_wait();
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.IM * d.KM) return;
    int i = t % d.IM + 1, k = t / d.IM + 1;
    float PO1 = A1(d.PO1, k), TO1 = A1(d.TO1, k);
    // inlet, isentropic from the stagnation state
    float RO_STAG = PO1 / d.RGAS / TO1;
    float RO_IN = A3(d.RO, i, 1, k);
    if (d.ADJ_ROIN) d.ADJ_ROIN[t] = RO_IN;
    // the Spalart-Allmaras inlet value divides by RO(IMID,1,KMID) as the
    // reference's K, I loop finds it: the inlet points before (IMID, KMID)
    // see this value from before the update (k_sa_inlet)
    if (d.SAW && i == d.IMID && k == d.KMID) d.SAW[sa_work_node_floats(d) + 64 + 2] = RO_IN;
    if (RO_IN > 0.9999f * RO_STAG) RO_IN = 0.9999f * RO_STAG;
    float PNEW = PO1 * powf(RO_IN / RO_STAG, d.GA);
    float p1 = A3(d.P, i, 1, k);
    int ip = d.IN_PRESS < 0 ? -d.IN_PRESS : d.IN_PRESS;
    if (d.IN_PRESS == 0) p1 = d.RFIN1 * p1 + d.RFIN * PNEW;
    if (ip == 1) p1 = d.RFIN1 * p1 + d.RFIN2 * A3(d.P, i, 2, k) - d.RFIN * A3(d.P, i, 3, k);
    if (ip == 3) p1 = d.RFIN1 * p1 + d.RFIN2 * d.BCBUF[k - 1] - d.RFIN * d.BCBUF[d.KM + k - 1];
    if (ip == 4) p1 = d.RFIN1 * p1 + d.RFIN2 * A3(d.P, d.IMID, 2, d.KMID) - d.RFIN * A3(d.P, d.IMID, 3, d.KMID);
    float plim = A1(d.PLIM, k);
    if (p1 > plim) p1 = 0.9f * p1 + 0.1f * plim;
    if (p1 > 0.99999f * PO1) p1 = PO1 * 0.99999f;
    A3(d.P, i, 1, k) = p1;
    float TSTATIC = TO1 * powf(p1 * A1(d.RPO1, k), d.FGA);
    float VABSQ = 2.0f * d.CP * (TO1 - TSTATIC);
    A3(d.T_STATIC, i, 1, k) = TSTATIC;
    float VABS = sqrtf(VABSQ);
    float VMER = 0.0f;
    float vt1 = A3(d.VT, i, 1, k);
    if (d.IN_VTAN == 0) {
        VMER = VABS * A1(d.BSCOS, k);
        vt1 = VABS * A1(d.BSSIN, k);
    }
    if (d.IN_VTAN == 1) {
        float VMERSQ = VABSQ - A1(d.VTIN, k) * A1(d.VTIN, k);
        if (VMERSQ < 0.01f) VMERSQ = 0.01f;
        VMER = sqrtf(VMERSQ);
        vt1 = A1(d.VTIN, k);
    }
    if (d.IN_VTAN == 2) {
        float WR = A2(d.UBLADE, 1, k);
        float VRELSQ = VABSQ - WR * WR * A1(d.BSCOS, k) * A1(d.BSCOS, k);
        if (VRELSQ < 0.01f) VRELSQ = 0.01f;
        float VREL = sqrtf(VRELSQ) - WR * A1(d.BSSIN, k);
        VMER = VREL * A1(d.BSCOS, k);
        vt1 = VREL * A1(d.BSSIN, k) + WR;
    }
    A3(d.VT, i, 1, k) = vt1;
    float vx1 = A3(d.VX, i, 1, k), vr1 = A3(d.VR, i, 1, k);
    float vr2 = A3(d.VR, i, 2, k);
    if (d.IN_VR > 0) vx1 = VMER * A1(d.BRCOS, k);
    float VXSQ = VMER * VMER - vr2 * vr2;
    if (VXSQ < 0.0000001f * TO1 * d.CP) VXSQ = 0.0000001f * TO1 * d.CP;
    if (d.IN_VR <= 0) vx1 = sqrtf(VXSQ);
    if (d.IN_VR > 0) vr1 = VMER * A1(d.BRSIN, k);
    if (d.IN_VR <= 0) vr1 = vr2;
    A3(d.VX, i, 1, k) = vx1;
    A3(d.VR, i, 1, k) = vr1;
    float ro1 = p1 / (d.RGAS * TSTATIC);
    float rovt1 = ro1 * vt1;
    A3(d.RO, i, 1, k) = ro1;
    A3(d.ROVT, i, 1, k) = rovt1;
    A3(d.ROVR, i, 1, k) = ro1 * vr1;
    A3(d.RORVT, i, 1, k) = rovt1 * A2(d.R, 1, k);
    A3(d.ROVX, i, 1, k) = ro1 * vx1;
    A3(d.ROE, i, 1, k) = p1 / d.GA1 + ro1 * 0.5f * VABSQ;
    A3(d.HO, i, 1, k) = d.CP * TO1;
    // exit: pitchwise pressure variation extrapolated from upstream
    float vr = A3(d.VR, i, d.JM, k), vt = A3(d.VT, i, d.JM, k), vx = A3(d.VX, i, d.JM, k);
    float EKE = 0.5f * (vr * vr + vt * vt + vx * vx);
    float pe = d.BCBUF[3 * d.KM + k - 1] + d.FEXTRAP * (A3(d.P, i, d.JMM1, k) - d.BCBUF[2 * d.KM + k - 1]);
    float hoe = 2.0f * A3(d.HO, i, d.JMM1, k) - A3(d.HO, i, d.JM - 2, k);
    float TEXIT = (hoe - EKE) / d.CP;
    float roe_ = pe / d.RGAS / TEXIT;
    A3(d.P, i, d.JM, k) = pe;
    A3(d.HO, i, d.JM, k) = hoe;
    A3(d.RO, i, d.JM, k) = roe_;
    A3(d.ROE, i, d.JM, k) = roe_ * (d.CV * TEXIT + EKE);
}

static size_t bc_sums_smem(const Dev &d) { return (size_t)32 * (4 * d.IMM1 + 2 * d.IM) * sizeof(float); }

cudaError_t configure_flux_kernels(const Dev &d) {
    return raise_smem((const void *)k_bc_sums, bc_sums_smem(d));
}

void launch_bc_sums(const Dev &d, Launch L) {
    launchk(L, k_bc_sums, dim3(1), dim3(1024), bc_sums_smem(d), d);
    mark(L, "k_bc_sums");
}

void launch_bc_apply(const Dev &d, Launch L) {
    launchk(L, k_bc_apply, dim3((d.IM * d.KM + 127) / 128), dim3(128), 0, d);
    mark(L, "k_bc_apply");
}

// ---------------------------------------------------------------------
// SETFLO (8006-8052), IN_FLOW != 0: relax the mass flow of every J station
// towards FLOWIN (IN_FLOW = 3) or the mean flow.  k_setflo_flow forms FLOW(J)
// (one CTA per J; REDUCE_ORDER = 1: one thread in the reference's K, I
// order, otherwise an FP64 tree of the same terms); k_setflo_apply scales
// ROVX, ROVR and ROVT of plane J.
// ---------------------------------------------------------------------
constexpr int SF_BS = 256;

__global__ void __launch_bounds__(SF_BS) k_setflo_flow(Dev d) {
    pdl_wait();
    const int j = blockIdx.x + 1;
    const int IMM1 = d.IMM1, KMM1 = d.KMM1;
    const float NBJ = (float)A1(d.NBLADE, j), NB1 = (float)A1(d.NBLADE, 1);
    if (d.REDUCE_ORDER == 1) {
        if (threadIdx.x == 0) {
            float f = 0.0f;
            for (int k = 1; k <= KMM1; ++k)
                for (int i = 1; i <= IMM1; ++i) f = f - A3(d.FLOWX, i, j, k) * NBJ / NB1;
            d.FLOWJ[j - 1] = f;
        }
        return;
    }
    const int ro = d.REDUCE_ORDER;
    double s = 0.0;
    for (int c = threadIdx.x; c < IMM1 * KMM1; c += SF_BS) {
        int i = c % IMM1 + 1, k = c / IMM1 + 1;
        s = racc(ro, s, (double)(A3(d.FLOWX, i, j, k) * NBJ / NB1));
    }
    __shared__ double sh[SF_BS / 32];
    for (int o = 16; o > 0; o >>= 1) s = racc(ro, s, __shfl_down_sync(0xffffffffu, s, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < SF_BS / 32; ++w) t = racc(ro, t, sh[w]);
        d.FLOWJ[j - 1] = (float)(-t);
    }
}

__global__ void __launch_bounds__(SF_BS) k_setflo_apply(Dev d) {
    pdl_wait();
    const int j = blockIdx.x + 1;
    __shared__ float s_delta;
    if (threadIdx.x == 0) {
        float AVFLOW = d.FLOWIN / (float)A1(d.NBLADE, 1);
        if (d.IN_FLOW != 3) {
            if (d.REDUCE_ORDER == 1) {
                float a = 0.0f;
                for (int jj = 1; jj <= d.JM; ++jj) a = a + d.FLOWJ[jj - 1];
                AVFLOW = a / (float)d.JM;
            } else {
                double a = 0.0;
                for (int jj = 1; jj <= d.JM; ++jj) a = racc(d.REDUCE_ORDER, a, (double)d.FLOWJ[jj - 1]);
                AVFLOW = d.REDUCE_ORDER == 2 ? (float)a / (float)d.JM : (float)(a / (double)d.JM);
            }
        }
        float a = A3(d.ROVX, d.IMID, j, d.KMID), b = A3(d.ROVR, d.IMID, j, d.KMID);
        float ROVMER = sqrtf(a * a + b * b);
        float DELTA = (AVFLOW / d.FLOWJ[j - 1] - 1.0f) * ROVMER;
        s_delta = DELTA * d.RFLOW;
    }
    __syncthreads();
    const float DELTA = s_delta;
    const int IM = d.IM;
    for (int t = threadIdx.x; t < IM * d.KM; t += SF_BS) {
        int i = t % IM + 1, k = t / IM + 1;
        const int n = ix3(d, i, j, k);
        float x = d.ROVX[n], r = d.ROVR[n];
        float RM = sqrtf(x * x + r * r);
        if (x < 0.0f) RM = -RM;
        d.ROVX[n] = x + x / RM * DELTA;
        d.ROVR[n] = r + r / RM * DELTA;
        float RO_WT = d.ROVT[n] - A2(d.UBLADE, j, k) * d.RO[n];
        d.ROVT[n] = d.ROVT[n] + RO_WT / RM * DELTA;
    }
}

void launch_setflo(const Dev &d, Launch L) {
    launchk(L, k_setflo_flow, dim3(d.JM), dim3(SF_BS), 0, d);
    mark(L, "k_setflo_flow");
    launchk(L, k_setflo_apply, dim3(d.JM), dim3(SF_BS), 0, d);
    mark(L, "k_setflo_apply");
}

// ---------------------------------------------------------------------
// IF_CUSP = 2 (5178-5233): forced separation at the trailing edge of a row.
// One thread per (row, K) runs the suction-side points (I = 1..6) and then
// the pressure-side points (I = IM-6..IM), as the reference orders them;
// the rows' ranges are disjoint (checked at commit).
// ---------------------------------------------------------------------
__global__ void k_cusp_sep(Dev d) {
    pdl_wait();
    const int nr = blockIdx.x + 1;
    if (A1(d.IF_CUSP, nr) != 2) return;
    const int IM = d.IM;
    const int JTEDGE = A1(d.JTE, nr);
    const int JSEP_I1 = JTEDGE - A1(d.NUP_I1, nr), JSEP_IM = JTEDGE - A1(d.NUP_IM, nr);
    const int JTHIK = JSEP_I1 > JSEP_IM ? JSEP_I1 : JSEP_IM;
    const float FDRAG = A1(d.SEP_DRAG, nr);
    const int NWKE = A1(d.N_WAKE, nr);
    for (int k = threadIdx.x + 1; k <= d.KM; k += blockDim.x) {
        auto force = [&](int i, int j) {
            const int n = ix3(d, i, j, k);
            d.ROVX[n] = FDRAG * d.ROVX[n];
            d.ROVR[n] = FDRAG * d.ROVR[n];
            float RO_VBLADE = d.RO[n] * A2(d.UBLADE, j, k);
            float RO_WT = d.ROVT[n] - RO_VBLADE;
            float RO_VT = FDRAG * RO_WT + RO_VBLADE;
            d.RORVT[n] = RO_VT * A2(d.R, j, k);
        };
        const float THIK_LIM = A1(d.SEP_THIK, nr) * A2(d.RT_THICK, JTHIK, k);
        const float SSSLOPE = (A3(d.RTHETA, 1, JSEP_I1 + 1, k) - A3(d.RTHETA, 1, JSEP_I1 - 1, k)) /
                              (A2(d.X, JSEP_I1 + 1, k) - A2(d.X, JSEP_I1 - 1, k));
        const float PSSLOPE = (A3(d.RTHETA, IM, JSEP_IM + 1, k) - A3(d.RTHETA, IM, JSEP_IM - 1, k)) /
                              (A2(d.X, JSEP_IM + 1, k) - A2(d.X, JSEP_IM - 1, k));
        for (int j = JSEP_I1; j <= JTEDGE + NWKE; ++j) {
            float RTEXTRAP = A3(d.RTHETA, 1, JSEP_I1, k) + SSSLOPE * (A2(d.X, j, k) - A2(d.X, JSEP_I1, k));
            for (int i = 1; i <= 6; ++i)
                if ((RTEXTRAP - A3(d.RTHETA, i, j, k)) > THIK_LIM) force(i, j);
        }
        for (int j = JSEP_IM; j <= JTEDGE + NWKE; ++j) {
            float RTEXTRAP = A3(d.RTHETA, IM, JSEP_IM, k) + PSSLOPE * (A2(d.X, j, k) - A2(d.X, JSEP_IM, k));
            for (int i = IM - 6; i <= IM; ++i)
                if ((A3(d.RTHETA, i, j, k) - RTEXTRAP) > THIK_LIM) force(i, j);
        }
    }
}

void launch_cusp(const Dev &d, Launch L) {
    launchk(L, k_cusp_sep, dim3(d.NROWS), dim3(64), 0, d);
    mark(L, "k_cusp_sep");
}

// ---------------------------------------------------------------------
// raw TFLUX of the moment-of-momentum (6200-6230) and radial-momentum
// (6300-6330) equations at one I, used for the periodic balances at I=1
// and I=IM (902, 6260)
// ---------------------------------------------------------------------
__device__ inline bool density_triggers(float ro, float ROAVG, float ROLIM) {
    return ro < 0.6f * ROAVG || ro > 1.5f * ROAVG || ro < ROLIM;
}

// PEFF = P - PREFF + F_PDOWN*(P(J+1) - P) (4321) of node (i, j, k), formed
// where it is read; the expression and its order are those of the
// reference's PEFF loop
__device__ __forceinline__ float peff_of(const Dev &d, const float *P, int o, int j) {
    const float p = P[o];
    const float pj1 = (d.F_PDOWN != 0.0f && j < d.JM) ? P[o + d.IM] : p;
    return p - d.PREFF + d.F_PDOWN * (pj1 - p);
}
__device__ __forceinline__ float peff_at(const Dev &d, int i, int j, int k) { return peff_of(d, d.P, ix3(d, i, j, k), j); }

__device__ inline float tflux_rvt_raw(const Dev &d, int i, int j, int k, float AVGR) {
    const float *VT = d.VT;
    float AVGVT = A3(VT, i, j, k) + A3(VT, i, j - 1, k) + A3(VT, i, j - 1, k + 1) + A3(VT, i, j, k + 1);
    float AVGP = peff_at(d, i, j, k) + peff_at(d, i, j - 1, k) + peff_at(d, i, j - 1, k + 1) + peff_at(d, i, j, k + 1);
    return (A3(d.FLOWT, i, j, k) * AVGVT + A2(d.ABT, j, k) * AVGP) * AVGR;
}

__device__ inline float tflux_rmom_raw(const Dev &d, int i, int j, int k, float *avgp4) {
    const float *VR = d.VR;
    float AVGVR = A3(VR, i, j, k) + A3(VR, i, j - 1, k) + A3(VR, i, j - 1, k + 1) + A3(VR, i, j, k + 1);
    float AVGP = peff_at(d, i, j, k) + peff_at(d, i, j - 1, k) + peff_at(d, i, j - 1, k + 1) + peff_at(d, i, j, k + 1);
    *avgp4 = AVGP;
    return 0.25f * (A3(d.FLOWT, i, j, k) * AVGVR + AVGP * A3(d.ABR, i, j, k));
}

// The three momentum equations' fluxes in one pass over the nodes
// (6100-6120, 6200-6230, 6300-6330 with the cusp and periodic balances).
// Each thread loads its node's neighbour cube of PEFF, VX, VT, VR and ROVT
// once -- the values at (i+di, j+dj, k+dk), di, dk in {0,1}, dj in {-1,0} --
// and forms every average from registers, each sum in the order of the
// reference's expression.  The balances at I=1 and I=IM, which also need the
// other end's column, keep the direct loads of the helpers above.

__global__ void __launch_bounds__(256, 3) k_flux_mom(Dev d) {
    pdl_wait();
    const int n = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int N = d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, (size_t)n, i, j, k);
    const int IM = d.IM, sJ = d.IM, sK = d.IM * d.JM;
    const bool hi = i < IM, hj = j >= 2, hk = k < d.KM;
    const float *__restrict__ PP = d.P;
    const float *__restrict__ VX = d.VX;
    const float *__restrict__ VT = d.VT;
    const float *__restrict__ VR = d.VR;
    const float *__restrict__ RV = d.ROVT;
    // c[di][dj + 1][dk]; positions outside the grid are never used
    float pe[2][2][2] = {}, vx[2][2][2] = {}, vt[2][2][2] = {}, vr[2][2][2] = {}, rv[2][2][2] = {};
#pragma unroll
    for (int di = 0; di < 2; ++di)
#pragma unroll
        for (int dj = -1; dj <= 0; ++dj)
#pragma unroll
            for (int dk = 0; dk < 2; ++dk) {
                if ((di && !hi) || (dj && !hj) || (dk && !hk)) continue;
                const int o = n + di + dj * sJ + dk * sK;
                pe[di][dj + 1][dk] = peff_of(d, PP, o, j + dj);
                vt[di][dj + 1][dk] = VT[o];
                if (!(di && dj && dk)) {
                    vx[di][dj + 1][dk] = VX[o];
                    vr[di][dj + 1][dk] = VR[o];
                }
                if (hi && hj && hk) rv[di][dj + 1][dk] = RV[o];
            }
#define C(a, di, dj, dk) a[di][(dj) + 1][dk]
    // every per-node operand is loaded before the first store, so that the
    // loads are in flight together (the stores below may not be reordered
    // ahead of loads through other Dev pointers)
    const bool fK = hi && hk, fJ = hi && hj, fI = hj && hk, fS = fJ && hk;
    const float xforce = fK ? d.XFORCE[n] : 0.0f, tforce = fK ? d.TFORCE[n] : 0.0f;
    const float aqx = fK ? d.AQX[n] : 0.0f, aqr = fK ? d.AQR[n] : 0.0f, flowx = fK ? d.FLOWX[n] : 0.0f;
    const float rjk = A2(d.R, j, k);
    const float rk1 = fK ? A2(d.R, j, k + 1) : 0.0f, rj1 = fJ ? A2(d.R, j - 1, k) : 0.0f;
    const float asx = fJ ? d.ASX[n] : 0.0f, asr = fJ ? d.ASR[n] : 0.0f, flowr = fJ ? d.FLOWR[n] : 0.0f;
    const float rforce = fS ? d.RFORCE[n] : 0.0f, volor = fS ? d.VOLOR[n] : 0.0f;
    const float FT = fI ? d.FLOWT[n] : 0.0f, abx = fI ? d.ABX[n] : 0.0f, abr = fI ? d.ABR[n] : 0.0f;
    const float abt = fI ? A2(d.ABT, j, k) : 0.0f, ravg = fI ? A2(d.RAVG_CELL, j, k) : 0.0f;
    const bool edge = (i == 1 || i == IM) && A1(d.IND, j) != 1;
    const float *RO = d.RO;
    const bool dens = j >= 3 && j <= d.JM - 3;
    const float ro0 = RO[n];
    const float rom2 = dens ? RO[n - 2 * sJ] : 0.0f, rom1 = dens ? RO[n - sJ] : 0.0f;
    const float rop1 = dens ? RO[n + sJ] : 0.0f, rop2 = dens ? RO[n + 2 * sJ] : 0.0f;
    d.PEFF[n] = C(pe, 0, 0, 0);    // PEFF of this step, read by the next step's energy fluxes
    const VarSet &VXm = d.var[V_ROVX], &VTm = d.var[V_RORVT], &VRm = d.var[V_ROVR];
    // faces K = const (XFLUX) and the axial / tangential sources
    if (fK) {
        VXm.SR[n] = xforce;
        float AVGP = C(pe, 0, 0, 0) + C(pe, 0, 0, 1) + C(pe, 1, 0, 1) + C(pe, 1, 0, 0);
        float AVGVX = C(vx, 0, 0, 0) + C(vx, 0, 0, 1) + C(vx, 1, 0, 1) + C(vx, 1, 0, 0);
        VXm.XF[n] = 0.25f * (AVGP * aqx + flowx * AVGVX);
        float AVGR = 0.125f * (rjk + rk1);
        float AVGVT = C(vt, 0, 0, 0) + C(vt, 0, 0, 1) + C(vt, 1, 0, 0) + C(vt, 1, 0, 1);
        VTm.SR[n] = tforce;
        VTm.XF[n] = flowx * AVGR * AVGVT;
        float AVGVR = C(vr, 0, 0, 0) + C(vr, 0, 0, 1) + C(vr, 1, 0, 0) + C(vr, 1, 0, 1);
        VRm.XF[n] = 0.25f * (flowx * AVGVR + aqr * AVGP);
    }
    // faces J = const (RFLUX) and the radial source
    if (fJ) {
        float AVGP = C(pe, 0, 0, 0) + C(pe, 0, -1, 0) + C(pe, 1, -1, 0) + C(pe, 1, 0, 0);
        float AVGVX = C(vx, 0, 0, 0) + C(vx, 0, -1, 0) + C(vx, 1, -1, 0) + C(vx, 1, 0, 0);
        VXm.RF[n] = 0.25f * (AVGP * asx + flowr * AVGVX);
        float AVGR = (rjk + rj1) * 0.125f;
        float AVGVT = C(vt, 0, 0, 0) + C(vt, 0, -1, 0) + C(vt, 1, -1, 0) + C(vt, 1, 0, 0);
        VTm.RF[n] = flowr * AVGVT * AVGR;
        float AVGVR = C(vr, 0, 0, 0) + C(vr, 0, -1, 0) + C(vr, 1, -1, 0) + C(vr, 1, 0, 0);
        VRm.RF[n] = 0.25f * (flowr * AVGVR + asr * AVGP);
        if (hk) {
            float AVGRVT = C(rv, 0, 0, 0) + C(rv, 0, 0, 1) + C(rv, 0, -1, 0) + C(rv, 0, -1, 1) + C(rv, 1, 0, 0) +
                           C(rv, 1, 0, 1) + C(rv, 1, -1, 0) + C(rv, 1, -1, 1);
            float AVGVT8 = 0.125f * (C(vt, 0, 0, 0) + C(vt, 0, -1, 0) + C(vt, 0, -1, 1) + C(vt, 0, 0, 1) + C(vt, 1, 0, 0) +
                                     C(vt, 1, -1, 0) + C(vt, 1, -1, 1) + C(vt, 1, 0, 1));
            float AVGP8 = C(pe, 0, 0, 0) + C(pe, 0, -1, 0) + C(pe, 0, -1, 1) + C(pe, 0, 0, 1) + C(pe, 1, 0, 0) +
                          C(pe, 1, -1, 0) + C(pe, 1, -1, 1) + C(pe, 1, 0, 1);
            VRm.SR[n] = rforce - (AVGRVT * AVGVT8 + AVGP8) * volor;
        }
    }
    // faces I = const (TFLUX)
    if (fI) {
        float AVGP = C(pe, 0, 0, 0) + C(pe, 0, -1, 0) + C(pe, 0, -1, 1) + C(pe, 0, 0, 1);
        if (edge) {
            float AVGPCUSP = peff_at(d, 1, j, k) + peff_at(d, 1, j - 1, k) + peff_at(d, 1, j, k + 1) +
                             peff_at(d, 1, j - 1, k + 1) + peff_at(d, IM, j, k) + peff_at(d, IM, j - 1, k) +
                             peff_at(d, IM, j, k + 1) + peff_at(d, IM, j - 1, k + 1);
            float AVGVXCUSP = A3(VX, 1, j, k) + A3(VX, 1, j - 1, k) + A3(VX, 1, j, k + 1) + A3(VX, 1, j - 1, k + 1) +
                              A3(VX, IM, j, k) + A3(VX, IM, j - 1, k) + A3(VX, IM, j, k + 1) + A3(VX, IM, j - 1, k + 1);
            VXm.TF[n] = 0.125f * (FT * AVGVXCUSP + AVGPCUSP * abx);
        } else {
            float AVGVX = C(vx, 0, 0, 0) + C(vx, 0, -1, 0) + C(vx, 0, -1, 1) + C(vx, 0, 0, 1);
            VXm.TF[n] = 0.25f * (FT * AVGVX + abx * AVGP);
        }
        const float AVGR = 0.25f * ravg;
        float AVGVT = C(vt, 0, 0, 0) + C(vt, 0, -1, 0) + C(vt, 0, -1, 1) + C(vt, 0, 0, 1);
        float tf = (FT * AVGVT + abt * AVGP) * AVGR;
        if (edge) {
            float t1 = (i == 1) ? tf : tflux_rvt_raw(d, 1, j, k, AVGR);
            float tm = (i == IM) ? tf : tflux_rvt_raw(d, IM, j, k, AVGR);
            tf = 0.5f * (t1 + tm);
        }
        VTm.TF[n] = tf;
        float AVGVR = C(vr, 0, 0, 0) + C(vr, 0, -1, 0) + C(vr, 0, -1, 1) + C(vr, 0, 0, 1);
        float tr = 0.25f * (FT * AVGVR + AVGP * abr);
        if (edge) {
            float ap1, apm;
            float t1raw = tflux_rmom_raw(d, 1, j, k, &ap1);
            float tmraw = tflux_rmom_raw(d, IM, j, k, &apm);
            float AVGP1 = 0.25f * (peff_at(d, 1, j, k) + peff_at(d, 1, j - 1, k) + peff_at(d, 1, j, k + 1) +
                                   peff_at(d, 1, j - 1, k + 1));
            float AVGPM = 0.25f * (peff_at(d, IM, j, k) + peff_at(d, IM, j - 1, k) + peff_at(d, IM, j, k + 1) +
                                   peff_at(d, IM, j - 1, k + 1));
            float T1 = t1raw - AVGP1 * A3(d.ABR, 1, j, k);
            float T2 = tmraw - AVGPM * A3(d.ABR, IM, j, k);
            tr = 0.5f * ((T1 + T2) + (AVGP1 + AVGPM) * abr);
        }
        VRm.TF[n] = tr;
    }
#undef C
    // the density limiter's column flags (7200): RO is final here (after
    // TSTEP(RO) and the inlet/exit conditions) and TSTEP of the momenta
    // does not change it
    if (d.ADJ_RO_LIM) d.ADJ_RO_LIM[n] = ro0;
    if (dens) {
        const float ROAVG = 0.25f * (rom2 + rom1 + rop1 + rop2);
        if (density_triggers(ro0, ROAVG, d.ROLIM)) d.DFLAG[(size_t)(k - 1) * d.IM + (i - 1)] = 1;
    }
}

void launch_flux_mom(const Dev &d, Launch L) {
    size_t N = (size_t)d.IM * d.JM * d.KM;
    launchk(L, k_flux_mom, dim3(grid_for(N, 256)), dim3(256), 0, d);
    mark(L, "k_flux_mom");
}

// ---------------------------------------------------------------------
// density limiter (7200).  The reference walks J in place, so RO(J-1) and
// RO(J-2) are already limited when RO(J) is tested.  A column's result
// differs from its input only if some J triggers a limit on the unmodified
// values (the first trigger is the same in both), so k_flux_mom flags those
// columns in parallel and k_density_fix replays the sequential walk on
// flagged columns only.  The thread owning (IMID,KMID) then sets the
// per-row Mach limits VLIMIT/ROLIMIT (7250) from its final densities.
// ---------------------------------------------------------------------
constexpr int DF_AHEAD = 64;     // J values a flagged column loads together in k_density_fix

__global__ void k_density_fix(Dev d) {
    pdl_wait();
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.IM * d.KM) return;
    int i = t % d.IM + 1, k = t / d.IM + 1;
    float *RO = d.RO;
    if (d.DFLAG[t]) {
        d.DFLAG[t] = 0;
        float ROLIM = d.ROLIM;
        const int JM = d.JM, sJ = d.IM;
        float *col = RO + (i - 1) + (size_t)sJ * JM * (k - 1);     // col[sJ * (j - 1)] = RO(i, j, k)
        float rm2 = col[0], rm1 = col[sJ], r0 = col[2 * sJ];
        float rp1 = col[3 * sJ];
        // the walk reads RO(J+2) before any write reaches it, so the
        // values ahead are loaded DF_AHEAD at a time: one memory latency
        // per batch instead of one per J
        for (int jb = 3; jb <= JM - 3; jb += DF_AHEAD) {
            float ahead[DF_AHEAD];
#pragma unroll
            for (int q = 0; q < DF_AHEAD; ++q) {
                const int jj = jb + 2 + q;
                ahead[q] = jj <= JM ? col[sJ * (jj - 1)] : 0.0f;
            }
#pragma unroll
            for (int q = 0; q < DF_AHEAD; ++q) {
                const int j = jb + q;
                if (j > JM - 3) break;
                float rp2 = ahead[q];
                float ROAVG = 0.25f * (rm2 + rm1 + rp1 + rp2);
                float ro = r0;
                if (ro < 0.6f * ROAVG) ro = 0.5f * (ro + 0.6f * ROAVG);
                if (ro > 1.5f * ROAVG) ro = 0.5f * (ro + 1.5f * ROAVG);
                if (ro < ROLIM) ro = 0.5f * (ro + ROLIM);
                if (ro != r0) {
                    col[sJ * (j - 1)] = ro;
                    if (d.ADJ_FLAG) atomicOr(d.ADJ_FLAG, 1);
                }
                rm2 = rm1;
                rm1 = ro;
                r0 = rp1;
                rp1 = rp2;
            }
        }
    }
    if (i == d.IMID && k == d.KMID) {
        float GM1 = d.GA - 1.0f;
        float TRATIO = 1.0f + d.MACHLIM * d.MACHLIM * 0.5f * GM1;
        float RFGM1 = 1.0f / GM1;
        float RORATIO = powf(TRATIO, RFGM1);
        for (int nr = 1; nr <= d.NROWS; ++nr) {
            int JREF = A1(d.JLE, nr);
            float TREF = A3(d.T_STATIC, d.IMID, JREF, d.KMID);
            float vx = A3(d.VX, d.IMID, JREF, d.KMID), vr = A3(d.VR, d.IMID, JREF, d.KMID), wt = A3(d.WT, d.IMID, JREF, d.KMID);
            float WREFSQ = vx * vx + vr * vr + wt * wt;
            float TOREL_REF = TREF + 0.5f * WREFSQ / d.CP;
            float TLIMIT = TOREL_REF / TRATIO;
            if (TLIMIT > d.TCOOL_MIN) TLIMIT = d.TCOOL_MIN;
            A1(d.VLIMIT, nr) = sqrtf(2.0f * d.CP * (TOREL_REF - TLIMIT));
            float ROSTAG_REL = A3(RO, d.IMID, JREF, d.KMID) * powf(TOREL_REF / TREF, RFGM1);
            A1(d.ROLIMIT, nr) = ROSTAG_REL / RORATIO;
        }
    }
}

// Mach-number / relative-mass-flux limiter (7100)
__global__ void k_mach_limiter(Dev d) {
    pdl_wait();
    size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t N = (size_t)d.IM * d.JM * d.KM;
    if (n >= N) return;
    int i, j, k;
    node_ijk(d, n, i, j, k);
    int nr = A1(d.NROW, j);
    float V_LIMIT = A1(d.VLIMIT, nr), RO_LIMIT = A1(d.ROLIMIT, nr);
    float ro = d.RO[n];
    const float vx = d.VX[n], vr = d.VR[n], wt = d.WT[n];   // loaded before any store
    if (d.ADJ_RO_MACH) d.ADJ_RO_MACH[n] = ro;
    if (ro < RO_LIMIT) {
        ro = RO_LIMIT;
        d.RO[n] = ro;
        if (d.ADJ_FLAG) atomicOr(d.ADJ_FLAG, 2);
    }
    float WRELSQ = vx * vx + vr * vr + wt * wt;
    float WREL = sqrtf(WRELSQ);
    float FACSAFE = V_LIMIT / WREL;
    if (FACSAFE < 1.0f) {
        if (d.ADJ_FLAG) atomicOr(d.ADJ_FLAG, 2);
        d.ROVX[n] = ro * vx * FACSAFE;
        d.ROVR[n] = ro * vr * FACSAFE;
        float ROVTREL = ro * wt * FACSAFE;
        d.ROWT[n] = ROVTREL;
        float rovt = ROVTREL + ro * A2(d.UBLADE, j, k);
        d.ROVT[n] = rovt;
        d.RORVT[n] = rovt * A2(d.R, j, k);
    }
}

void launch_limiters(const Dev &d, Launch L) {
    int lines = d.IM * d.KM;
    launchk(L, k_density_fix, dim3((lines + 127) / 128), dim3(128), 0, d);
    mark(L, "k_density_fix");
    size_t N = (size_t)d.IM * d.JM * d.KM;
    launchk(L, k_mach_limiter, dim3(grid_for(N, 256)), dim3(256), 0, d);
    mark(L, "k_mach_limiter");
}

// ---------------------------------------------------------------------
// NEW_MIXPLAN (14922-15251), IFGAS=0: one CTA per (row interface, K).
// The threads fill the per-I isentropic states and angles; the outward
// Prandtl-Meyer sweeps for a supersonic relative flow and the periodicity
// correction run in the reference's order on one thread; the threads then
// relax the J=JMIX+2 (or JMIX-1) plane.
// ---------------------------------------------------------------------
constexpr int MIX_MAXI = 160;
constexpr int MIX_BS = 64;

__global__ void __launch_bounds__(MIX_BS) k_mixplan(Dev d) {
    pdl_wait();
    __shared__ float ALPHAA[MIX_MAXI], GAMA[MIX_MAXI], WREF_JP2[MIX_MAXI], ROREF_JP2[MIX_MAXI], PISENT[MIX_MAXI];
    __shared__ float ROISENT[MIX_MAXI], WMACH_JP2[MIX_MAXI], TISENT[MIX_MAXI], WIS_JP2[MIX_MAXI];
    const int nr = blockIdx.x / d.KM + 1, k = blockIdx.x % d.KM + 1;
    const int IM = d.IM;
    const float RFMIX1 = 1.0f - d.RFMIX;
    const int KSUB = (k == d.KM) ? d.KM - 1 : k;
    int j = A1(d.JMIX, nr);
    int JP1, JP2, JP3;
    float F_ANGLE;
    if (A3(d.FLOWX, d.IMID, j, KSUB) < 0.0f) {
        JP1 = j + 1; JP2 = j + 2; JP3 = j + 3;
        F_ANGLE = d.FANGLE;
    } else {
        j = A1(d.JMIX, nr) + 1;
        JP1 = j - 1; JP2 = j - 2; JP3 = j - 3;
        F_ANGLE = 0.0f;
    }
    const float F_ANGLE1 = 1.0f - F_ANGLE;
    const float RJP1 = A2(d.R, JP1, k), UJP1 = A2(d.UBLADE, JP1, k);
    const float ROMIX = A3(d.RO, d.IMID, JP1, k);
    const float VXMIX = A3(d.ROVX, d.IMID, JP1, k) / ROMIX;
    const float VRMIX = A3(d.ROVR, d.IMID, JP1, k) / ROMIX;
    const float VTMIX = A3(d.RORVT, d.IMID, JP1, k) / ROMIX / RJP1;
    const float ROEMIX = A3(d.ROE, d.IMID, JP1, k);
    const float VMSQ = VXMIX * VXMIX + VRMIX * VRMIX;
    const float VABSQ = VMSQ + VTMIX * VTMIX;
    const float WTMIX = VTMIX - UJP1;
    const float WMIXSQ = VMSQ + WTMIX * WTMIX;
    const float WMIX = sqrtf(WMIXSQ);
    const float ALPHAMIX = asinf(WTMIX / WMIX);
    const float GAMAMIX = atan2f(VRMIX, VXMIX);
    const float TMIX = (ROEMIX / ROMIX - 0.5f * VABSQ) / d.CV;
    const float ROTHALPY = d.CP * TMIX + 0.5f * (WMIXSQ - UJP1 * UJP1);
    const float GAGAS = d.GA;
    const float PMIX = ROMIX * d.RGAS * TMIX;
    const float RJP2 = A2(d.R, JP2, k), UNOWJP2 = A2(d.UBLADE, JP2, k);
    const float RJP3 = A2(d.R, JP3, k), UNOWJP3 = A2(d.UBLADE, JP3, k);
    int nmach = 0;
    if (d.ADJ_MIX) {
        float *rec = d.ADJ_MIX + (size_t)blockIdx.x * mix_rec_size(IM);
        if (threadIdx.x == 0) {
            rec[0] = ROMIX;
            rec[1] = A3(d.ROVX, d.IMID, JP1, k);
            rec[2] = A3(d.ROVR, d.IMID, JP1, k);
            rec[3] = A3(d.RORVT, d.IMID, JP1, k);
            rec[4] = ROEMIX;
        }
        for (int i = threadIdx.x + 1; i <= IM; i += MIX_BS) {
            float *q = rec + 5 + 10 * (i - 1);
            q[0] = A3(d.RO, i, JP2, k); q[1] = A3(d.ROVX, i, JP2, k); q[2] = A3(d.ROVR, i, JP2, k);
            q[3] = A3(d.RORVT, i, JP2, k); q[4] = A3(d.ROE, i, JP2, k);
            q[5] = A3(d.RO, i, JP3, k); q[6] = A3(d.ROVX, i, JP3, k); q[7] = A3(d.ROVR, i, JP3, k);
            q[8] = A3(d.RORVT, i, JP3, k); q[9] = A3(d.ROE, i, JP3, k);
        }
    }
    for (int i = threadIdx.x + 1; i <= IM; i += MIX_BS) {
        float ROJP2 = A3(d.RO, i, JP2, k);
        float XVELJP2 = A3(d.ROVX, i, JP2, k) / ROJP2;
        float RVELJP2 = A3(d.ROVR, i, JP2, k) / ROJP2;
        float TVELJP2 = A3(d.RORVT, i, JP2, k) / RJP2 / ROJP2;
        float WTJP2 = TVELJP2 - UNOWJP2;
        float VMSQJP2 = XVELJP2 * XVELJP2 + RVELJP2 * RVELJP2;
        float VELSQJP2 = VMSQJP2 + TVELJP2 * TVELJP2;
        float WACT_SQ_JP2 = VMSQJP2 + WTJP2 * WTJP2;
        float WACT_JP2 = sqrtf(WACT_SQ_JP2);
        float T_ACT_JP2 = (A3(d.ROE, i, JP2, k) / ROJP2 - 0.5f * VELSQJP2) / d.CV;
        float ROJP3 = A3(d.RO, i, JP3, k);
        float ROVXJP3 = A3(d.ROVX, i, JP3, k), ROVRJP3 = A3(d.ROVR, i, JP3, k);
        float ROVTJP3 = A3(d.RORVT, i, JP3, k) / RJP3;
        float ROWTJP3 = ROVTJP3 - UNOWJP3 * ROJP3;
        float ROVMSQJP3 = ROVXJP3 * ROVXJP3 + ROVRJP3 * ROVRJP3;
        float ROWRELSQJP3 = ROVMSQJP3 + ROWTJP3 * ROWTJP3;
        float ROWRELJP3 = sqrtf(ROWRELSQJP3);
        float ALPHAJP3 = asinf(ROWTJP3 / ROWRELJP3);
        float GAMAJP3 = atan2f(ROVRJP3, ROVXJP3);
        float PSTAT = ROJP2 * d.RGAS * T_ACT_JP2;
        float TISENT_JP2 = TMIX * powf(PSTAT / PMIX, d.FGA);
        float WIS_SQ_JP2 = 2.0f * (ROTHALPY - d.CP * TISENT_JP2 + 0.5f * UNOWJP2 * UNOWJP2);
        ROISENT[i - 1] = PSTAT / d.RGAS / TISENT_JP2;
        PISENT[i - 1] = PSTAT;
        TISENT[i - 1] = TISENT_JP2;
        if (WIS_SQ_JP2 < 1.0f) WIS_SQ_JP2 = 1.0f;
        WIS_JP2[i - 1] = sqrtf(WIS_SQ_JP2);
        WREF_JP2[i - 1] = WACT_JP2;
        ROREF_JP2[i - 1] = ROJP2;
        float wm = WACT_JP2 / sqrtf(GAGAS * d.RGAS * T_ACT_JP2);
        WMACH_JP2[i - 1] = wm;
        if (wm > 1.0f) nmach = 1;
        ALPHAA[i - 1] = F_ANGLE1 * ALPHAMIX + F_ANGLE * ALPHAJP3;
        GAMA[i - 1] = F_ANGLE1 * GAMAMIX + F_ANGLE * GAMAJP3;
    }
    int NMACH = __syncthreads_or(nmach);
    if (NMACH != 0 && threadIdx.x == 0) {
        float FROTN = 1.0f;
        if (WTMIX < 0.0f) FROTN = -1.0f;
        for (int i = d.IMID + 1; i <= IM; ++i) {
            int a = i - 1, b = i - 2;   // 0-based I and I-1
            if (WMACH_JP2[a] > 1.001f && WMACH_JP2[b] > 1.001f) {
                float DELP = PISENT[a] - PISENT[b];
                float DELTAI = sqrtf(WMACH_JP2[a] * WMACH_JP2[a] - 1.0f) / (ROREF_JP2[a] * WREF_JP2[a] * WREF_JP2[a]);
                float DELTAIM1 = sqrtf(WMACH_JP2[b] * WMACH_JP2[b] - 1.0f) / (ROREF_JP2[b] * WREF_JP2[b] * WREF_JP2[b]);
                ALPHAA[a] = ALPHAA[b] + FROTN * DELP * 0.5f * (DELTAI + DELTAIM1);
            }
        }
        for (int i = d.IMID - 1; i >= 1; --i) {
            int a = i - 1, b = i;       // I and I+1
            if (WMACH_JP2[a] > 1.001f && WMACH_JP2[b] > 1.001f) {
                float DELP = PISENT[a] - PISENT[b];
                float DELTAI = sqrtf(WMACH_JP2[a] * WMACH_JP2[a] - 1.0f) / (ROREF_JP2[a] * WREF_JP2[a] * WREF_JP2[a]);
                float DELTAIP1 = sqrtf(WMACH_JP2[b] * WMACH_JP2[b] - 1.0f) / (ROREF_JP2[b] * WREF_JP2[b] * WREF_JP2[b]);
                ALPHAA[a] = ALPHAA[b] + FROTN * DELP * 0.5f * (DELTAI + DELTAIP1);
            }
        }
        float ROTN = ALPHAA[IM - 1] - ALPHAA[0];
        // periodicity correction (15177-15182); FP64 running sum in the
        // default precision split, REAL*4 with REDUCE_ORDER 1 and 2
        if (d.REDUCE_ORDER != 0) {
            float SUMFP = 0.0f;
            for (int i = 1; i <= IM; ++i) {
                ALPHAA[i - 1] = ALPHAA[i - 1] - ROTN * (SUMFP - 0.5f);
                SUMFP = SUMFP + A1(d.FP, i);
            }
        } else {
            double SUMFP = 0.0;
            for (int i = 1; i <= IM; ++i) {
                ALPHAA[i - 1] = (float)((double)ALPHAA[i - 1] - (double)ROTN * (SUMFP - 0.5));
                SUMFP += (double)A1(d.FP, i);
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x + 1; i <= IM; i += MIX_BS) {
        float RO_JP2 = ROISENT[i - 1];
        float WT_JP2 = WIS_JP2[i - 1] * sinf(ALPHAA[i - 1]);
        float VM_JP2 = WIS_JP2[i - 1] * cosf(ALPHAA[i - 1]);
        float VX_JP2 = VM_JP2 * cosf(GAMA[i - 1]);
        float VR_JP2 = VM_JP2 * sinf(GAMA[i - 1]);
        float VT_JP2 = WT_JP2 + UNOWJP2;
        float V_JP2_SQ = VM_JP2 * VM_JP2 + VT_JP2 * VT_JP2;
        float ROE_JP2 = ROISENT[i - 1] * (d.CV * TISENT[i - 1] + 0.5f * V_JP2_SQ);
        A3(d.RO, i, JP2, k) = RFMIX1 * A3(d.RO, i, JP2, k) + d.RFMIX * RO_JP2;
        A3(d.ROVX, i, JP2, k) = RFMIX1 * A3(d.ROVX, i, JP2, k) + d.RFMIX * RO_JP2 * VX_JP2;
        A3(d.ROVR, i, JP2, k) = RFMIX1 * A3(d.ROVR, i, JP2, k) + d.RFMIX * RO_JP2 * VR_JP2;
        A3(d.RORVT, i, JP2, k) = RFMIX1 * A3(d.RORVT, i, JP2, k) + d.RFMIX * RO_JP2 * VT_JP2 * RJP2;
        A3(d.ROE, i, JP2, k) = RFMIX1 * A3(d.ROE, i, JP2, k) + d.RFMIX * ROE_JP2;
    }
}

void launch_mixplan(const Dev &d, Launch L) {
    if (!(d.IFMIX > 0 && d.RFMIX > 1.0e-3f) || d.NRWSM1 <= 0) return;
    launchk(L, k_mixplan, dim3(d.NRWSM1 * d.KM), dim3(MIX_BS), 0, d);
    mark(L, "k_mixplan");
}

}  // namespace mgpu
