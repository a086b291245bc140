// minor.cu -- the minor species and soot of MSFLOW on the frozen flow
// (Msflow.f90, Gslv3m.f90, Sourcem.f90): the reaction rates RRMS, the right-
// hand sides of the seven species (CH4, O2, CO, H2O, CO2, N2, NO) and of soot,
// their clipped and relaxed updates, and the sums MSFLOW reports.  The line
// solves, the residuals, EXTRM and INTPM are the shared kernels.
//
// One thread per cell of the range I = 4..MPM2, J = NJY1..NJY2,
// K = LKZ1..LKZ2.  The reaction loop carries one value from cell to cell:
// RR2 keeps the previous cell's last value (its reaction 4+5 rate) where a
// cell's first reaction is off (Gslv3m.f90:45-60), and that cell subtracts it
// from its O2 inflow.  That value depends only on the previous cell's own
// state, so it is formed for every cell first (k_ms_r4), the previous
// reaction cell in loop order (I outer, K inner) is found by a prefix maximum,
// and the rates follow (k_ms_rates).
#include "state.cuh"

namespace gfm {
namespace {

constexpr int kMsBlock = 256;
__device__ __forceinline__ double wms_d(int l) {   // Var_mod.f90:223-229
    switch (l) {
        case 0: return 16.0426;
        case 1: return 31.9988;
        case 2: return 28.0104;
        case 3: return 18.0152;
        case 4: return 44.0098;
        case 5: return 28.0134;
        default: return 30.0061;
    }
}

struct MsRange {
    int i0, i1, j0, j1, k0, k1, ni, nj, nk;
    __host__ __device__ int count() const { return ni * nj * nk; }
    // thread t: I fastest (coalesced); q: the reference's loop order (K fastest)
    __device__ void at(int t, int& I, int& J, int& K, int& q) const {
        const int a = t % ni, b = (t / ni) % nj, d = t / (ni * nj);
        I = i0 + 2 * a; J = j0 + 2 * b; K = k0 + 2 * d;
        q = (a * nj + b) * nk + d;
    }
};
template <typename R>
MsRange ms_range(const GeoT<R>& g) {
    MsRange r;
    r.i0 = 4; r.i1 = g.MPM2; r.j0 = g.NJY1; r.j1 = g.NJY2; r.k0 = g.LKZ1; r.k1 = g.LKZ2;
    r.ni = r.i1 >= r.i0 ? (r.i1 - r.i0) / 2 + 1 : 0;
    r.nj = r.j1 >= r.j0 ? (r.j1 - r.j0) / 2 + 1 : 0;
    r.nk = r.k1 >= r.k0 ? (r.k1 - r.k0) / 2 + 1 : 0;
    return r;
}
int ms_grid(long long n) { return (int)((n + kMsBlock - 1) / kMsBlock < 4096 ? (n + kMsBlock - 1) / kMsBlock : 4096); }

template <typename R>
__device__ __forceinline__ int rcell(const GeoT<R>& g, int I, int J, int K) {   // RRMS(MZ,NZ,LZ) cell, I fastest
    return (I / 2 - 1) + (g.MP / 2) * ((J / 2 - 1) + (g.NP / 2) * (K / 2 - 1));
}

// reactions 4 and 5 of one cell (Gslv3m.f90:95-111): thermal and prompt NO
__device__ __forceinline__ double rate45(const double* G, double gfm6, double TMP, double VOL) {
    double RR2, RR3;
    if (G[1] > 1.0e-20 && G[2] > 1.0e-20 && G[5] > 1.0e-20) {
        const double R1 = pow(G[2], 0.721) * pow(G[1], 4.0111) * gfm6 / 0.725;
        RR2 = 7.94e22 * R1 * exp(-44369.0 / TMP) * VOL;
    } else {
        RR2 = 0;
    }
    if (G[1] > 1.0e-20 && G[5] > 1.0e-20) {
        const double R1 = G[5] * sqrt(G[1]);   // GFM6**ODR(5,1) * GFM2**ODR(5,2), orders 1 and 0.5
        RR3 = 9.33e14 * R1 * exp(-68899.0 / TMP) * pow(TMP, -0.5);
        RR3 = RR3 * VOL;
    } else {
        RR3 = 0;
    }
    return RR2 + RR3;
}

// the cell's concentrations (kmol/m3), temperature (K) and volume
template <typename R>
__device__ __forceinline__ void ms_cell(const Ctx<R>& c, const MinorDev<R>& m, long long o, int I, int J, int K, double* G,
                                        double& TMP, double& VOL) {
    const GeoT<R>& g = c.g;
    TMP = (double)c.T[o] * c.p.t0;
    const double DNST1 = (double)c.DNST[o] * c.p.dnst0;
    VOL = (double)g.DX[I] * (double)g.DR[J] * (double)g.DZ[K] * 1.0;   // *VOL0
    for (int l = 0; l < 7; ++l) G[l] = (double)m.gfm[l][o] / wms_d(l) * DNST1;
}

template <typename R>
__global__ void __launch_bounds__(kMsBlock) k_ms_r4(Ctx<R> c, MinorDev<R> m, MsScratch<R> s, MsRange r) {
    const int n = r.count();
    GFM_FOR(t, n) {
        int I, J, K, q;
        r.at(t, I, J, K, q);
        const long long o = pidx(c.g, I, J, K);
        if (c.g.ib[o] > 0) { s.setter[q] = -1; continue; }
        double G[7], TMP, VOL;
        ms_cell(c, m, o, I, J, K, G, TMP, VOL);
        s.r4[q] = rate45(G, (double)m.gfm[5][o], TMP, VOL);
        s.setter[q] = q;
    }
}

// SPIN (Gslv3m.f90:292-305): inflow of species l into the cell, kmol/s
template <typename R>
__device__ __forceinline__ double spin(const Ctx<R>& c, const MinorDev<R>& m, const R* const* as, long long o, int I, int J,
                                       int K, int l) {
    const GeoT<R>& g = c.g;
    const R* y = m.gfm[l];
    const double G11 = (double)as[0][o] * (double)y[pidx(g, I - 2, J, K)];
    const double G12 = (double)as[1][o] * (double)y[pidx(g, I + 2, J, K)];
    const double G21 = (double)as[2][o] * (double)y[pidx(g, I, J - 2, K)];
    const double G22 = (double)as[3][o] * (double)y[pidx(g, I, J + 2, K)];
    const double G31 = (double)as[4][o] * (double)y[pidx(g, I, J, K - 2)];
    const double G32 = (double)as[5][o] * (double)y[pidx(g, I, J, K + 2)];
    const double FXMS = G11 + G12 + G21 + G22 + G31 + G32;
    return FXMS * c.p.gmfr / wms_d(l);
}

struct AsPtrs { const void* p[6]; };

// the reaction rates of GSLV3M (Gslv3m.f90:24-115): RRMS 1, 2, 4
template <typename R>
__global__ void __launch_bounds__(kMsBlock) k_ms_rates(Ctx<R> c, MinorDev<R> m, MsScratch<R> s, MsRange r, AsPtrs ap) {
    const R* as[6];
    for (int q = 0; q < 6; ++q) as[q] = static_cast<const R*>(ap.p[q]);
    const int n = r.count();
    const int mz = c.g.MP / 2, ncl = mz * (c.g.NP / 2) * (c.g.LP / 2);
    GFM_FOR(t, n) {
        int I, J, K, q;
        r.at(t, I, J, K, q);
        const long long o = pidx(c.g, I, J, K);
        if (c.g.ib[o] > 0) continue;
        // RR2 as the previous reaction cell left it
        int prev = -1;
        if (q > 0) {
            prev = s.setter[q - 1];
            const int bp = s.blockmax[(q - 1) / 1024];
            if (bp > prev) prev = bp;
        }
        double RR2 = prev >= 0 ? s.r4[prev] : *s.carry;
        double G[7], TMP, VOL;
        ms_cell(c, m, o, I, J, K, G, TMP, VOL);
        R* rr = m.rrms + rcell(c.g, I, J, K);
        // reaction 1: CH4 + 1.5 O2 -> CO + 2 H2O
        const double FXMS1 = spin(c, m, as, o, I, J, K, 0);
        double FXMS2 = spin(c, m, as, o, I, J, K, 1);
        if (G[0] <= 1.0e-25 || G[1] <= 1.0e-25) {
            rr[0] = R(0);
        } else {
            const double RR1 = pow(G[0], 1.46) * pow(G[1], 0.5217);
            RR2 = 1.66e15 * RR1 * exp(-20643.0 / TMP) * VOL;
            if (RR2 > FXMS1) RR2 = FXMS1;
            if (FXMS2 / 1.5 < RR2) RR2 = FXMS2 / 1.5;
            rr[0] = R(RR2 * 0.3 + (double)rr[0] * 0.7);
        }
        // reaction 2: CO + 0.5 O2 -> CO2
        FXMS2 = FXMS2 - RR2 * 1.5;
        if (FXMS2 > 1.0e-20 && G[2] > 1.0e-20) {
            const double RR1 = pow(G[2], 1.6904) * pow(G[1], 1.57);
            RR2 = 7.94e14 * RR1 * exp(-11613.0 / TMP) * VOL;
            if (FXMS2 * 2 < RR2) RR2 = FXMS2 * 2;
            const double FXMS3 = spin(c, m, as, o, I, J, K, 2);
            RR2 = RR2 < FXMS3 ? RR2 : FXMS3;
        } else {
            RR2 = 0;
        }
        // reaction 3: CO2 -> CO + 0.5 O2
        double RR3;
        if (G[4] > 1.0e-20) {
            const double RR1 = G[4];   // GFM5**ODR(3,1), order 1
            RR3 = 2.24e14 * RR1 * exp(-62281.0 / TMP) * VOL;
            const double FXMS5 = spin(c, m, as, o, I, J, K, 4);
            RR3 = RR3 < FXMS5 ? RR3 : FXMS5;
        } else {
            RR3 = 0;
        }
        double RR1 = RR2 - RR3;
        if (RR1 < 0) RR1 = 0;
        rr[ncl] = R(RR1 * 0.3 + (double)rr[ncl] * 0.7);
        // reactions 4 and 5: N2 + O2 -> 2 NO
        rr[3 * (long long)ncl] = R(s.r4[q]);
    }
}
// RR2 leaving the last reaction cell: the value the next call starts from
__global__ void k_ms_carry(double* carry, const int* setter, const int* blockmax, const double* r4, int nq) {
    if (threadIdx.x != 0 || blockIdx.x != 0 || nq <= 0) return;
    int last = setter[nq - 1];
    const int bp = blockmax[(nq - 1) / 1024];
    if (bp > last) last = bp;
    if (last >= 0) *carry = r4[last];
}

// GSLV3G0's AP of the minor species' set, and AP/RFM of the species systems
// (SFP = 0 for the species: AP - SFP*VOL keeps AP)
template <typename R>
__global__ void __launch_bounds__(kMsBlock) k_ms_ap(Ctx<R> c, MsScratch<R> s, MsRange r) {
    const int n = r.count();
    GFM_FOR(t, n) {
        int I, J, K, q;
        r.at(t, I, J, K, q);
        const long long o = pidx(c.g, I, J, K);
        if (c.g.ib[o] >= 1) { s.ap1[o] = R(1); s.ap[o] = R(1); continue; }
        R a = R(0);
        for (int k = 0; k < 6; ++k) a = a + s.as[k][o];
        s.ap1[o] = a;
        s.ap[o] = a / R(s.rfm);
    }
}

// SOURCEM for the species (Sourcem.f90:12-39) and the relaxation of
// Gslv3m.f90:152-169: BS = G0*WMS/GMFR + RFMC*FZ*AP
template <typename R>
__global__ void __launch_bounds__(kMsBlock) k_ms_species(Ctx<R> c, MinorDev<R> m, MsScratch<R> s, MsRange r) {
    const int n = r.count();
    const int ncl = (c.g.MP / 2) * (c.g.NP / 2) * (c.g.LP / 2);
    const R rfmc = R(1.0 - s.rfm);
    GFM_FOR(t, n) {
        int I, J, K, q;
        r.at(t, I, J, K, q);
        const long long o = pidx(c.g, I, J, K);
        const int ib = c.g.ib[o];
        if (ib > 0) {
            for (int l = 0; l < 7; ++l) s.bs[l][o] = ib >= 1 ? m.gfm[l][o] : R(0);
            continue;
        }
        const R* rr = m.rrms + rcell(c.g, I, J, K);
        const R r1 = rr[0], r2 = rr[ncl], r4 = rr[3 * (long long)ncl];
        R g0[7];
        g0[0] = -r1;
        g0[1] = -r1 * R(1.5) - r2 * R(0.5) - r4;
        g0[2] = r1 - r2;
        g0[3] = r1 * R(2);
        g0[4] = r2;
        g0[5] = -r4;
        g0[6] = r4 * R(2);
        const R ap = s.ap[o];
        for (int l = 0; l < 7; ++l) {
            R bs = g0[l] * R(wms_d(l)) / R(c.p.gmfr);
            bs = bs + rfmc * s.fz[l][o] * ap;
            s.bs[l][o] = bs;
        }
    }
}

// the species' clip and relaxation after their solves (Gslv3m.f90:176-191),
// and the mass balance of the species (Gslv3m.f90:196-217)
template <typename R>
__global__ void __launch_bounds__(kMsBlock) k_ms_update(Ctx<R> c, MinorDev<R> m, MsScratch<R> s, MsRange r) {
    __shared__ double sh[32];
    const int n = r.count();
    const R rfm = R(s.rfm), rfmc = R(1.0 - s.rfm);
    double bal = 0.0;
    GFM_FOR(t, n) {
        int I, J, K, q;
        r.at(t, I, J, K, q);
        const long long o = pidx(c.g, I, J, K);
        if (c.g.ib[o] >= 1) continue;
        double sum = 0.0;
        for (int l = 0; l < 7; ++l) {
            R z = s.fz[l][o];
            if (z > R(1)) z = R(1);
            if (z < R(0)) z = R(0);
            if (l == 2 && z > R(0.1)) z = R(0.1);
            if (l == 6 && z > R(1.0e-2)) z = R(1.0e-2);
            R v = rfmc * m.gfm[l][o] + rfm * z;
            if (v < R(1.0e-20)) v = R(0);
            m.gfm[l][o] = v;
            sum = sum + (double)v;
        }
        bal += fabs(1.0 - sum) * (double)vol_c0(c.g, I, J, K);
    }
    const double b = block_sum(bal, sh);
    if (threadIdx.x == 0) c.partials[kSlMsBal * kRedBlocks + blockIdx.x] = b;
}

// SOURCEM for soot (Sourcem.f90:76-118, the current soot model) over the
// whole array, with the previous sources' relaxation; the new sources become
// bs_soot_prev and sfp_soot_prev
template <typename R>
__global__ void k_soot_source(Ctx<R> c, MinorDev<R> m, MsScratch<R> s, MsRange r, int itr_ms) {
    const GeoT<R>& g = c.g;
    const double E0_sf = s.t0_sf < 1.0e-20 ? 0.0 : exp(-s.esf_r / s.t0_sf);
    const double E0_so = s.t0_so < 1.0e-20 ? 0.0 : sqrt(s.t0_so) * exp(-s.eso_r / s.t0_so);
    const long long n = (long long)g.MP * g.NP * g.LP;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int I = (int)(t % g.MP) + 1, J = (int)((t / g.MP) % g.NP) + 1, K = (int)(t / ((long long)g.MP * g.NP)) + 1;
        const long long o = pidx(g, I, J, K);
        double bs = 0.0, sfp = 0.0;
        const bool in = !(I & 1) && !(J & 1) && !(K & 1) && I >= r.i0 && I <= r.i1 && J >= r.j0 && J <= r.j1 && K >= r.k0 &&
                        K <= r.k1;
        if (in && g.ib[o] <= 0 && s.react) {
            const double Tcell = (double)c.T[o] * c.p.t0;
            if (Tcell > s.t0_sf) {
                bs = s.aform * (double)m.gfm[0][o] * (exp(-s.esf_r / Tcell) - E0_sf) * s.snorm;
                if (itr_ms > 1) bs = s.rf_sf * bs + (1.0 - s.rf_sf) * (double)m.bsp[o];
            }
            if (Tcell > s.t0_so) {
                sfp = -s.aoxid * (double)m.gfm[1][o] * (sqrt(Tcell) * exp(-s.eso_r / Tcell) - E0_so) * s.snorm;
                if (itr_ms > 1) sfp = s.rf_so * sfp + (1.0 - s.rf_so) * (double)m.sfpp[o];
            }
        }
        m.bsp[o] = R(bs);
        m.sfpp[o] = R(sfp);
    }
}
// the soot system (Gslv3m.f90:237-256): AP = (sum AS - SFP*VOL)/RFM,
// BS = BS*VOL + RFMC*FZ*AP, in ap and bs[0] with fz[0] = smf
template <typename R>
__global__ void __launch_bounds__(kMsBlock) k_soot_system(Ctx<R> c, MinorDev<R> m, MsScratch<R> s, MsRange r) {
    const int n = r.count();
    const R rfm = R(s.rfm_soot), rfmc = R(1.0 - s.rfm_soot);
    GFM_FOR(t, n) {
        int I, J, K, q;
        r.at(t, I, J, K, q);
        const long long o = pidx(c.g, I, J, K);
        if (c.g.ib[o] >= 1) { s.ap[o] = R(1); s.bs[0][o] = s.fz[0][o]; continue; }
        const R vol = vol_c0(c.g, I, J, K);   // VOL_C at a centre
        R bs = m.bsp[o] * vol;
        R ap = s.ap1[o];
        ap = ap - (m.sfpp[o] * vol);
        ap = ap / rfm;
        bs = bs + rfmc * s.fz[0][o] * ap;
        s.ap[o] = ap;
        s.bs[0][o] = bs;
    }
}
// soot's clip at soot_cap and relaxation (Gslv3m.f90:263-284) with the soot
// mass and the largest mass fractions
template <typename R>
__global__ void __launch_bounds__(kMsBlock) k_soot_update(Ctx<R> c, MinorDev<R> m, MsScratch<R> s, MsRange r) {
    __shared__ double sh[32];
    const int n = r.count();
    const R rfm = R(s.rfm_soot), rfmc = R(1.0 - s.rfm_soot);
    double tot = 0.0, mx = 0.0, mxn = 0.0;
    GFM_FOR(t, n) {
        int I, J, K, q;
        r.at(t, I, J, K, q);
        const long long o = pidx(c.g, I, J, K);
        if (c.g.ib[o] >= 1) continue;
        const R z = s.fz[0][o];
        mxn = fmax(mxn, (double)z);
        R G0;
        if (z > R(s.soot_cap)) G0 = R(s.soot_cap);
        else if (z > R(1.0e-20)) G0 = z;
        else G0 = R(0);
        mx = fmax(mx, (double)G0);
        const R v = rfm * G0 + rfmc * m.smf[o];
        m.smf[o] = v;
        const double vol = (double)c.g.DX[I] * (double)c.g.DR[J] * (double)c.g.DZ[K];
        tot += (double)v * (double)c.DNST[o] * c.p.dnst0 * vol;
    }
    const double a = block_sum(tot, sh);
    const double b = block_max(mx, sh);
    const double d = block_max(mxn, sh);
    if (threadIdx.x == 0) {
        c.partials[kSlMsSoot * kRedBlocks + blockIdx.x] = a;
        c.partials[kSlMsSmfMax * kRedBlocks + blockIdx.x] = b;
        c.partials[kSlMsSmfMaxNc * kRedBlocks + blockIdx.x] = d;
    }
}

// FLX1DM's planes of MSFLOW's report (Flx1d.f90:114-160, Msflow.f90:53-57):
// block l < 7 sums species l+1 through x-faces 5 (negative flow) and MP-3
// (positive) and y-faces 5 and NP-3; block 7 the exits' area-mean soot
// volume fraction (Msflow.f90:65-82).  One block each, sums in a fixed order.
template <typename R>
__global__ void __launch_bounds__(kMsBlock) k_ms_stats(Ctx<R> c, MinorDev<R> m, MsScratch<R> s) {
    __shared__ double sh[32];
    const GeoT<R>& g = c.g;
    const int l = blockIdx.x;
    if (l < 7) {
        double sum = 0.0;
        const int nj = (g.NPM2 - 4) / 2 + 1, nk = (g.LKZ2 - g.LKZ1) / 2 + 1;
        const int ni = (g.MPM2 - 4) / 2 + 1;
        const int nx = nj * nk, ny = ni * nk;
        for (int t = threadIdx.x; t < 2 * nx + 2 * ny; t += blockDim.x) {
            int I, J, K, ix, want;
            if (t < 2 * nx) {
                const int u = t % nx;
                I = t < nx ? 5 : g.MP - 3; want = t < nx ? 2 : 1;
                J = 4 + 2 * (u / nk); K = g.LKZ1 + 2 * (u % nk); ix = 1;
            } else {
                const int u = (t - 2 * nx) % ny;
                J = t - 2 * nx < ny ? 5 : g.NP - 3; want = t - 2 * nx < ny ? 2 : 1;
                I = 4 + 2 * (u / nk); K = g.LKZ1 + 2 * (u % nk); ix = 2;
            }
            const long long o = pidx(g, I, J, K);
            if (g.ib[o] == 1) continue;
            const double g0 = (double)c.THETA[o] * (double)c.DNST[o] * (double)c.UG[ix - 1][o] *
                              (double)area_c(g, I, J, K, ix) * c.p.gmfr;
            if ((g0 >= 0.0 ? 1 : 2) == want) sum += fabs(g0) * (double)m.gfm[l][o];
        }
        const double tot = block_sum(sum, sh);
        if (threadIdx.x == 0) s.stats[l] = tot;
    } else {
        // the exit cells are EXTR's records of kind 3
        double num = 0.0, den = 0.0;
        for (int t = threadIdx.x; t < c.n_extr_io; t += blockDim.x) {
            const ExtrRec& e = c.extr_io[t];
            if (e.kind != 3) continue;
            const int I = e.I, J = e.J, K = e.K;
            const long long o = pidx(g, I, J, K);
            if (g.ib[o] != 3) continue;
            double G0 = (double)area_c(g, I, J, K, 3);
            if (G0 < 1.0e-20) G0 = (double)area_c(g, I, J, K, 2);
            if (G0 < 1.0e-20) G0 = (double)area_c(g, I, J, K, 1);
            den += G0;
            num += (double)m.smf[o] * (double)c.DNST[o] * c.p.dnst0 / 1.8e3 * G0;
        }
        const double a = block_sum(num, sh);
        const double b = block_sum(den, sh);
        if (threadIdx.x == 0) s.stats[7] = a / b;
    }
}

}  // namespace

template <typename R>
void launch_ms_rates(const Ctx<R>& c, const MinorDev<R>& m, const MsScratch<R>& s, R* const* as_spin, cudaStream_t st) {
    const MsRange r = ms_range(c.g);
    const int n = r.count();
    if (n <= 0) return;
    k_ms_r4<R><<<ms_grid(n), kMsBlock, 0, st>>>(c, m, s, r);
    launch_prefix_max(s.setter, n, s.blockmax, st);
    AsPtrs ap;
    for (int q = 0; q < 6; ++q) ap.p[q] = as_spin[q];
    k_ms_rates<R><<<ms_grid(n), kMsBlock, 0, st>>>(c, m, s, r, ap);
    k_ms_carry<<<1, 32, 0, st>>>(s.carry, s.setter, s.blockmax, s.r4, n);
}
template <typename R> void launch_ms_ap(const Ctx<R>& c, const MsScratch<R>& s, cudaStream_t st) {
    const MsRange r = ms_range(c.g);
    if (r.count() > 0) k_ms_ap<R><<<ms_grid(r.count()), kMsBlock, 0, st>>>(c, s, r);
}
template <typename R> void launch_ms_species(const Ctx<R>& c, const MinorDev<R>& m, const MsScratch<R>& s, cudaStream_t st) {
    const MsRange r = ms_range(c.g);
    if (r.count() > 0) k_ms_species<R><<<ms_grid(r.count()), kMsBlock, 0, st>>>(c, m, s, r);
}
template <typename R> void launch_ms_update(const Ctx<R>& c, const MinorDev<R>& m, const MsScratch<R>& s, cudaStream_t st) {
    const MsRange r = ms_range(c.g);
    const int nb = ms_grid(r.count()) < kRedBlocks ? ms_grid(r.count()) : kRedBlocks;
    if (r.count() > 0) k_ms_update<R><<<nb, kMsBlock, 0, st>>>(c, m, s, r);
}
template <typename R>
void launch_soot_system(const Ctx<R>& c, const MinorDev<R>& m, const MsScratch<R>& s, int itr_ms, cudaStream_t st) {
    const MsRange r = ms_range(c.g);
    const long long nall = (long long)c.g.MP * c.g.NP * c.g.LP;
    k_soot_source<R><<<ms_grid(nall), kMsBlock, 0, st>>>(c, m, s, r, itr_ms);
    if (r.count() > 0) k_soot_system<R><<<ms_grid(r.count()), kMsBlock, 0, st>>>(c, m, s, r);
}
template <typename R> void launch_soot_update(const Ctx<R>& c, const MinorDev<R>& m, const MsScratch<R>& s, cudaStream_t st) {
    const MsRange r = ms_range(c.g);
    const int nb = ms_grid(r.count()) < kRedBlocks ? ms_grid(r.count()) : kRedBlocks;
    if (r.count() > 0) k_soot_update<R><<<nb, kMsBlock, 0, st>>>(c, m, s, r);
}
template <typename R> void launch_ms_stats(const Ctx<R>& c, const MinorDev<R>& m, const MsScratch<R>& s, cudaStream_t st) {
    k_ms_stats<R><<<8, kMsBlock, 0, st>>>(c, m, s);
}

#define GFM_MS_INST(R)                                                                                          \
    template void launch_ms_rates<R>(const Ctx<R>&, const MinorDev<R>&, const MsScratch<R>&, R* const*,        \
                                     cudaStream_t);                                                             \
    template void launch_ms_ap<R>(const Ctx<R>&, const MsScratch<R>&, cudaStream_t);                            \
    template void launch_ms_species<R>(const Ctx<R>&, const MinorDev<R>&, const MsScratch<R>&, cudaStream_t);   \
    template void launch_ms_update<R>(const Ctx<R>&, const MinorDev<R>&, const MsScratch<R>&, cudaStream_t);    \
    template void launch_soot_system<R>(const Ctx<R>&, const MinorDev<R>&, const MsScratch<R>&, int,            \
                                        cudaStream_t);                                                          \
    template void launch_soot_update<R>(const Ctx<R>&, const MinorDev<R>&, const MsScratch<R>&, cudaStream_t);  \
    template void launch_ms_stats<R>(const Ctx<R>&, const MinorDev<R>&, const MsScratch<R>&, cudaStream_t);
GFM_MS_INST(double)
GFM_MS_INST(float)

}  // namespace gfm
