// bc.cu -- boundary extrapolation, staggered interpolation, exit mass
// balance, pressure re-reference, emission-only radiation, layout conversion
// and the deterministic finish of FP64 reductions.
#include "state.cuh"

namespace gfm {

#define A(arr, I, J, K) (arr)[pidx(g, (I), (J), (K))]

constexpr int kBlk = 256;
inline int gridn(long long n) {
    long long b = (n + kBlk - 1) / kBlk;
    if (b < 1) b = 1;
    if (b > kRedBlocks) b = kRedBlocks;
    return (int)b;
}

template <typename R> __device__ __forceinline__ R rmax2(R a, R b) { return a > b ? a : b; }
template <typename R> __device__ __forceinline__ R rmin2(R a, R b) { return a < b ? a : b; }


// dnst_calc at one position of the split arrays (calls CONC, Prop.f90:187-198)
template <typename R>
__device__ void dnst_at(const Ctx<R>& c, long long o) {
    R y[9];
    for (int l = 0; l < 9; ++l) y[l] = l == 7 ? R(0) : c.GF[l][o];
    R rho = dnst_calc<R>(y, 1, c.P[o], c.T[o], R(c.p.wt0));
    c.GF[kYF][o] = y[kYF]; c.GF[kYO2][o] = y[kYO2]; c.GF[kYCO2][o] = y[kYCO2];
    c.GF[kYN2][o] = y[kYN2]; c.GF[kYH2O][o] = y[kYH2O];
    c.DNST[o] = rho;
}

// ---------------------------------------------------------------------------
// EXTR(1) (Extr.f90:31-250) from host-built records
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_extr_io(Ctx<R> c) {
    __shared__ double sh[32];
    const GeoT<R>& g = c.g;
    double gfin0 = 0.0, qex = 0.0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < c.n_extr_io; t += gridDim.x * blockDim.x) {
        const ExtrRec& e = c.extr_io[t];
        const long long o = pidx(g, e.I, e.J, e.K), o1 = pidx(g, e.I1, e.J1, e.K1), o2 = pidx(g, e.I2, e.J2, e.K2);
        const R F1 = R(e.F1), F2 = R(e.F2);
        c.GF[kEps][o] = c.GF[kEps][o1];
        c.P[o] = c.P[o1] * F1 + c.P[o2] * F2;
        if (e.kind == 2) {
            // THER at the inlet keeps TMU and is overwritten in GAMA: only its eps clip survives
            c.GF[kEps][o] = rmax2(c.GF[kEps][o], R(1.0e-12));
            c.GAMA[o] = c.GAMA[o1];
            R area = area_c(g, e.I, e.J, e.K, e.IX);
            R g0 = c.THETA[o] * c.DNST[o] * c.UG[e.IX - 1][o] * area;
            gfin0 += fabs((double)g0);
            continue;
        }
        c.TMU[o] = c.TMU[o1];
        c.GAMA[o] = c.GAMA[o1];
        for (int L = 1; L <= 7; ++L) {
            if (L == kEps + 1) continue;
            R g0 = c.GF[L - 1][o1] * F1 + c.GF[L - 1][o2] * F2;
            if (L == kK + 1) c.GF[L - 1][o] = rmax2(g0, R(1.0e-6));
            else if (L == kH + 1) c.GF[L - 1][o] = g0;
            else c.GF[L - 1][o] = rmax2(g0, R(0));
        }
        {
            R y[9];
            for (int l = 0; l < 9; ++l) y[l] = l == 7 ? R(0) : c.GF[l][o];
            c.T[o] = enth_to_t<R>(*c.nist, y, 1, y[kH], c.T[o], R(c.p.t0), R(c.p.h_0));
        }
        dnst_at(c, o);
        R area = area_c(g, e.I, e.J, e.K, e.IX);
        double g0 = fabs((double)c.UG[e.IX - 1][o]) * c.p.ug0 * (double)area;
        g0 = g0 * (double)c.THETA[o] * (double)c.DNST[o] * c.p.dnst0;
        qex += (double)c.GF[kH][o] * c.p.h_0 * g0;
        if (e.kind == 3) {
            // SBC4 copy onto the exit face (Sbc.f90:506-522)
            const long long o3 = pidx(g, e.I3, e.J3, e.K3);
            c.P[o3] = c.P[o]; c.T[o3] = c.T[o];
            for (int l = 0; l < 9; ++l) if (l != 7) c.GF[l][o3] = c.GF[l][o];
            c.DNST[o3] = c.DNST[o]; c.THETA[o3] = c.THETA[o]; c.TMU[o3] = c.TMU[o]; c.GAMA[o3] = c.GAMA[o];
        }
    }
    double a = block_sum(gfin0, sh), b = block_sum(qex, sh);
    if (threadIdx.x == 0) { c.partials[8 * kRedBlocks + blockIdx.x] = a; c.partials[9 * kRedBlocks + blockIdx.x] = b; }
}

template <typename R>
__device__ void extr_wall_one(const Ctx<R>& c, const ExtrRec& e) {
    const GeoT<R>& g = c.g;
    const long long o = pidx(g, e.I, e.J, e.K), o1 = pidx(g, e.I1, e.J1, e.K1), o2 = pidx(g, e.I2, e.J2, e.K2);
    c.P[o] = c.P[o1] * R(e.F1) + c.P[o2] * R(e.F2);
    c.TMU[o] = c.TMU[o2];
    c.GAMA[o] = c.GAMA[o2];
    // walls adiabatic until a first full radiation call (Extr.f90:194-197)
    const bool adiabatic = c.scal[S_RAD_DONE] == 0.0;
    for (int L = 1; L <= 7; ++L)
        if (L - 1 != kH || adiabatic) c.GF[L - 1][o] = c.GF[L - 1][o1];
    if (adiabatic) c.T[o] = c.T[o1];
    dnst_at(c, o);
}

// Wall cells whose six axis neighbours are walls read the cell above them,
// (I,J,K+2) (EXT1 falls through, Extr.f90:626-660).  The Fortran loop visits
// K ascending, so every such cell reads the value its source had before this
// EXTR call: the sources are gathered first (k_extr_ft_gather), then written
// (k_extr_ft_apply), one thread per cell.
template <typename R>
__global__ void k_extr_ft_gather(Ctx<R> c) {
    const GeoT<R>& g = c.g;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < c.n_extr_ft; t += gridDim.x * blockDim.x) {
        const ExtrRec& e = c.extr_ft[t];
        const long long o1 = pidx(g, e.I1, e.J1, e.K1), o2 = pidx(g, e.I2, e.J2, e.K2);
        R* v = c.ft_buf + (long long)t * kFtVals;
        v[0] = c.P[o1] * R(e.F1) + c.P[o2] * R(e.F2);
        v[1] = c.TMU[o2];
        v[2] = c.GAMA[o2];
        for (int L = 1; L <= 7; ++L) v[2 + L] = c.GF[L - 1][o1];
        v[10] = c.T[o1];
    }
}
template <typename R>
__global__ void k_extr_ft_apply(Ctx<R> c) {
    const GeoT<R>& g = c.g;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < c.n_extr_ft; t += gridDim.x * blockDim.x) {
        const ExtrRec& e = c.extr_ft[t];
        const long long o = pidx(g, e.I, e.J, e.K);
        const R* v = c.ft_buf + (long long)t * kFtVals;
        c.P[o] = v[0];
        c.TMU[o] = v[1];
        c.GAMA[o] = v[2];
        // walls adiabatic until a first full radiation call (Extr.f90:194-197)
        const bool adiabatic = c.scal[S_RAD_DONE] == 0.0;
        for (int L = 1; L <= 7; ++L)
            if (L - 1 != kH || adiabatic) c.GF[L - 1][o] = v[2 + L];
        if (adiabatic) c.T[o] = v[10];
        dnst_at(c, o);
    }
}
template <typename R>
__global__ void k_extr_wall(Ctx<R> c) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < c.n_extr_wall; t += gridDim.x * blockDim.x)
        extr_wall_one(c, c.extr_wall[t]);
}

// ---------------------------------------------------------------------------
// EXTRV (Extr.f90:358-567): exit faces of direction IU.  Slots: 10 GFEX,
// 11 T*|G0|, 12 T*area, 13 area.
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R bound_v(R f, const Prm& p) {
    f = rmin2(f, R(p.u_mx));
    f = rmax2(f, R(p.u_mn));
    if (fabs(f) < R(1.0e-12)) f = R(0);
    return f;
}
template <typename R>
__global__ void k_extrv(Ctx<R> c, int mex, int first, int count) {
    __shared__ double sh[32];
    const GeoT<R>& g = c.g;
    double gfex = 0, tm = 0, ta = 0, ar = 0;
    const R factor = R(c.scal[S_FACTOR]);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
        const ExtrvRec& e = c.extrv[first + t];
        const int IU = e.IU;
        R* u = c.UG[IU - 1];
        const long long o = pidx(g, e.I, e.J, e.K);
        if (e.mode == 1) { u[o] = A(u, e.Is, e.Js, e.Ks); continue; }
        if (e.mode == 2) continue;
        const int M = e.m;
        int I1 = e.I, J1 = e.J, K1 = e.K, I0 = e.I, J0 = e.J, K0 = e.K;
        if (IU == 1) { I1 = e.I + 2 * M; I0 = e.I - M; }
        else if (IU == 2) { J1 = e.J + 2 * M; J0 = e.J - M; }
        else { K1 = e.K + 2 * M; K0 = e.K - M; }
        const long long o1 = pidx(g, I1, J1, K1);
        if (u[o1] * R(M) > R(0)) u[o1] = R(0);
        R area = area_c(g, e.I, e.J, e.K, IU);
        R g0 = c.THETA[o1] * c.DNST[o1] * u[o1] * area;
        if (mex == 0) {
            gfex += fabs((double)g0);
            tm += (double)c.T[o] * fabs((double)g0);
            ta += (double)c.T[o] * (double)area;
            ar += (double)area;
            continue;
        }
        ar += (double)area;
        u[o1] = u[o1] * factor;
        if (IU == 3) continue;   // GOTO 160 (Extr.f90:529)
        g0 = g0 * factor;
        R v = bound_v(g0 / (c.THETA[o] * c.DNST[o] * area), c.p);
        u[o] = v;
        A(u, I0, J0, K0) = v;
    }
    double a = block_sum(gfex, sh), b = block_sum(tm, sh), d = block_sum(ta, sh), e2 = block_sum(ar, sh);
    if (threadIdx.x == 0) {
        c.partials[10 * kRedBlocks + blockIdx.x] = a;
        c.partials[11 * kRedBlocks + blockIdx.x] = b;
        c.partials[12 * kRedBlocks + blockIdx.x] = d;
        c.partials[13 * kRedBlocks + blockIdx.x] = e2;
    }
}

// GFEX/Tmean_ex finish of EXTRV(0), GFIN of FLX1D and the exit FACTOR
// (Extr.f90:553-565, Flx1d.f90:75-77, Gslv3v.f90:213-231).  One thread.
__global__ void k_factor(double* scal, double gmfr, double t0, double f_mx, double f_mn) {
    if (threadIdx.x != 0) return;
    const int itr_gas = (int)scal[S_ITR_GAS];
    double gfex = scal[S_GFEX] * gmfr;
    scal[S_GFEX] = gfex;
    if (gfex < 1.0e-16) scal[S_TMEAN_EX] = scal[S_TAREA_MEAN] * t0 / scal[S_AREA_EX];
    else scal[S_TMEAN_EX] = scal[S_TMEAN_EX] * t0 * gmfr / gfex;
    scal[S_GFIN] = scal[S_GFIN0] * gmfr;
    if (itr_gas > 10) {
        if (gfex < 1.0e-20) { scal[S_FACTOR] = 1.0; scal[S_FADJ] = 0.0; }
        else {
            double f = scal[S_GFIN] / gfex;
            if (f > f_mx) { f = f_mx; scal[S_FADJ] = 0.0; }
            else if (f < f_mn) { f = f_mn; scal[S_FADJ] = 0.0; }
            scal[S_FACTOR] = f;
        }
    }
}

// ---------------------------------------------------------------------------
// INTPV (Intp.f90:84-139, 230-272): stage a/b/c of component IU
// ---------------------------------------------------------------------------
template <typename R>
__device__ R intp1(const GeoT<R>& g, int I, int J, int K, int ix) {
    if (ix == 3) return (g.DZ[K] <= R(0) || K > g.LP) ? R(0) : (g.Z[K] - g.Z[K - 1]) / g.DZ[K];
    if (ix == 2) return (g.DR[J] <= R(0) || J > g.NP) ? R(0) : (g.Rr[J] - g.Rr[J - 1]) / g.DR[J];
    return (g.DX[I] <= R(0) || I > g.MP) ? R(0) : (g.X[I] - g.X[I - 1]) / g.DX[I];
}

template <typename R>
__global__ void k_intpv(Ctx<R> c, int IU, int stage, int m0, int m1, int mstep, int n0, int n1, int nstep, int l0, int l1,
                        int lstep, int IX) {
    const GeoT<R>& g = c.g;
    const int nm = (m1 - m0) / mstep + 1, nn = (n1 - n0) / nstep + 1, nl = (l1 - l0) / lstep + 1;
    if (m1 < m0 || n1 < n0 || l1 < l0) return;
    const long long tot = (long long)nm * nn * nl;
    R* u = c.UG[IU - 1];
    GFM_FOR(t, tot) {
        // fastest-varying index is the one mapping to I
        int a = t % nm, b = (t / nm) % nn, d = t / (nm * nn);
        int M, N, L;
        if (IU == 1) { M = m0 + mstep * a; N = n0 + nstep * b; L = l0 + lstep * d; }
        else if (IU == 2) { L = l0 + lstep * (t % nl); int r = t / nl; M = m0 + mstep * (r % nm); N = n0 + nstep * (r / nm); }
        else { N = n0 + nstep * (t % nn); int r = t / nn; L = l0 + lstep * (r % nl); M = m0 + mstep * (r / nl); }
        int I, J, K;
        if (IU == 1) { I = M; J = N; K = L; } else if (IU == 2) { J = M; K = N; I = L; } else { K = M; I = N; J = L; }
        int b0 = IBC(g, I, J, K);
        if (b0 >= 1 && b0 != 4) continue;
        R f1 = intp1(g, I, J, K, IX), f2 = R(1) - f1;
        R v;
        if (IX == 1) {
            v = A(u, I + 1, J, K) * f1 + A(u, I - 1, J, K) * f2;
        } else if (IX == 2) {
            if (IBC(g, I, J + 1, K) == 2 && b0 == 0) { f1 = R(0); f2 = R(1); }
            else if (IBC(g, I, J - 1, K) == 2 && b0 == 0) { f1 = R(1); f2 = R(0); }
            v = A(u, I, J + 1, K) * f1 + A(u, I, J - 1, K) * f2;
        } else {
            if (IBC(g, I, J, K + 1) == 2 && b0 == 0) { f1 = R(0); f2 = R(1); }
            else if (IBC(g, I, J, K - 1) == 2 && b0 == 0) { f1 = R(1); f2 = R(0); }
            v = A(u, I, J, K + 1) * f1 + A(u, I, J, K - 1) * f2;
        }
        A(u, I, J, K) = bound_v(v, c.p);
        (void)stage;
    }
}

// ---------------------------------------------------------------------------
// INTP (Intp.f90:32-72, 145-206) with the carried-F1 code of each position
// (0 skip, 1 coordinate weight, 2 weight forced to 1, 3 weight forced to 0)
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_intp(Ctx<R> c, int stage) {
    const GeoT<R>& g = c.g;
    // stage 1: I even, K odd, J even; stage 2: I even, J odd, K all; stage 3: I odd, J all, K all
    int i0, i1, j0, j1, js, k0, k1, ks;
    if (stage == 1) { i0 = 2; i1 = g.MP; j0 = 2; j1 = g.NP; js = 2; k0 = 3; k1 = g.LPM1; ks = 2; }
    else if (stage == 2) { i0 = 2; i1 = g.MP; j0 = 3; j1 = g.NPM1; js = 2; k0 = 2; k1 = g.LP; ks = 1; }
    else { i0 = 3; i1 = g.MPM1; j0 = 2; j1 = g.NP; js = 1; k0 = 2; k1 = g.LP; ks = 1; }
    const int ni = (i1 - i0) / 2 + 1, nj = (j1 - j0) / js + 1, nk = (k1 - k0) / ks + 1;
    const long long tot = (long long)ni * nj * nk;
    GFM_FOR(t, tot) {
        int I = i0 + 2 * (t % ni);
        int r = t / ni;
        int J = j0 + js * (r % nj), K = k0 + ks * (r / nj);
        const long long o = pidx(g, I, J, K);
        int mode = c.intp_mode[o];
        if (mode == 0) continue;
        int I1, J1, K1, I2, J2, K2, ix;
        if (stage == 1) { I1 = I; J1 = J; K1 = K + 1; I2 = I; J2 = J; K2 = K - 1; ix = 3; }
        else if (stage == 2) { I1 = I; J1 = J + 1; K1 = K; I2 = I; J2 = J - 1; K2 = K; ix = 2; }
        else { I1 = I + 1; J1 = J; K1 = K; I2 = I - 1; J2 = J; K2 = K; ix = 1; }
        R f1 = mode == 1 ? intp1(g, I, J, K, ix) : (mode == 2 ? R(1) : R(0));
        R f2 = R(1) - f1;
        const long long a = pidx(g, I1, J1, K1), b = pidx(g, I2, J2, K2);
        c.P[o] = f1 * c.P[a] + f2 * c.P[b];
        c.T[o] = f1 * c.T[a] + f2 * c.T[b];
        R y[9];
        for (int l = 0; l < 9; ++l) y[l] = l == 7 ? R(0) : c.GF[l][o];
        for (int L = 1; L <= 7; ++L) y[L - 1] = f1 * c.GF[L - 1][a] + f2 * c.GF[L - 1][b];
        conc(y, 1);
        c.TMU[o] = f1 * c.TMU[a] + f2 * c.TMU[b];
        c.GAMA[o] = f1 * c.GAMA[a] + f2 * c.GAMA[b];
        c.THETA[o] = f1 * c.THETA[a] + f2 * c.THETA[b];
        R rho = dnst_calc<R>(y, 1, c.P[o], c.T[o], R(c.p.wt0));
        for (int l = 0; l < 9; ++l) if (l != 7) c.GF[l][o] = y[l];
        c.DNST[o] = rho;
    }
}

// ---------------------------------------------------------------------------
// Minor species (ms=1): INITSVM (Initsv.f90:329-378), EXTRM (Extr.f90:258-300)
// and INTPM (Intp.f90:348-420) on the seven GFM arrays, with the record
// tables and the carried-F1 codes of EXTR and INTP: the loops and the
// neighbour choices are the same.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_initsvm(Ctx<R> c, MinorDev<R> m, int restart) {
    const GeoT<R>& g = c.g;
    const long long n = (long long)g.MP * g.NP * g.LP;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int I = (int)(t % g.MP) + 1, J = (int)((t / g.MP) % g.NP) + 1, K = (int)(t / ((long long)g.MP * g.NP)) + 1;
        const long long o = pidx(g, I, J, K);
        const bool centre = !(I & 1) && !(J & 1) && !(K & 1);
        if (!restart) {   // smf = 0, GFM = 0, then the centres from the major species
            m.smf[o] = R(0);
            for (int l = 0; l < 7; ++l) m.gfm[l][o] = R(0);
            if (!centre) continue;
        } else if (!centre || g.ib[o] != 2) {
            continue;   // the restart state stays, but at the inlet cells
        }
        m.gfm[0][o] = c.GF[0][o];   // CH4  <- fuel
        m.gfm[1][o] = c.GF[1][o];   // O2
        m.gfm[3][o] = c.GF[8][o];   // H2O
        m.gfm[4][o] = c.GF[5][o];   // CO2
        m.gfm[5][o] = c.GF[6][o];   // N2
        if (restart) { m.gfm[2][o] = R(0); m.gfm[6][o] = R(0); }
    }
}
// EXTRM's exit loop: the exit cell from EXT0/EXTR1's cells and weights
// (the EXTR records of kind 3), copied onto the y-face toward J1
template <typename R>
__global__ void k_extrm_exit(Ctx<R> c, MinorDev<R> m) {
    const GeoT<R>& g = c.g;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < c.n_extr_io; t += gridDim.x * blockDim.x) {
        const ExtrRec& e = c.extr_io[t];
        if (e.kind != 3) continue;
        const long long o = pidx(g, e.I, e.J, e.K), o1 = pidx(g, e.I1, e.J1, e.K1), o2 = pidx(g, e.I2, e.J2, e.K2);
        const long long oy = pidx(g, e.I, (e.J + e.J1) / 2, e.K);
        const R F1 = R(e.F1), F2 = R(e.F2);
        for (int l = 0; l < 7; ++l) {
            const R g0 = m.gfm[l][o1] * F1 + m.gfm[l][o2] * F2;
            m.gfm[l][o] = rmax2(g0, R(0));
            m.gfm[l][oy] = m.gfm[l][o];
        }
        m.smf[o] = m.smf[o1];
    }
}
// EXTRM's wall loop: the neighbour's value into the wall cell and onto the
// face between them.  The fall-through cells read the cell above them before
// this loop writes it (gather, then apply), as for EXTR.
template <typename R>
__device__ __forceinline__ void extrm_wall_put(const GeoT<R>& g, const MinorDev<R>& m, const ExtrRec& e, const R* v) {
    const long long o = pidx(g, e.I, e.J, e.K);
    long long of;
    if (e.IX == 1) of = pidx(g, (e.I + e.I1) / 2, e.J, e.K);
    else if (e.IX == 2) of = pidx(g, e.I, (e.J + e.J1) / 2, e.K);
    else of = pidx(g, e.I, e.J, (e.K + e.K1) / 2);
    for (int l = 0; l < 7; ++l) { m.gfm[l][o] = v[l]; m.gfm[l][of] = v[l]; }
}
template <typename R>
__global__ void k_extrm_ft_gather(Ctx<R> c, MinorDev<R> m) {
    const GeoT<R>& g = c.g;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < c.n_extr_ft; t += gridDim.x * blockDim.x) {
        const ExtrRec& e = c.extr_ft[t];
        const long long o1 = pidx(g, e.I1, e.J1, e.K1);
        for (int l = 0; l < 7; ++l) c.ft_buf[(long long)t * kFtVals + l] = m.gfm[l][o1];
    }
}
template <typename R>
__global__ void k_extrm_ft_apply(Ctx<R> c, MinorDev<R> m) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < c.n_extr_ft; t += gridDim.x * blockDim.x)
        extrm_wall_put(c.g, m, c.extr_ft[t], c.ft_buf + (long long)t * kFtVals);
}
template <typename R>
__global__ void k_extrm_wall(Ctx<R> c, MinorDev<R> m) {
    const GeoT<R>& g = c.g;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < c.n_extr_wall; t += gridDim.x * blockDim.x) {
        const ExtrRec& e = c.extr_wall[t];
        const long long o1 = pidx(g, e.I1, e.J1, e.K1);
        R v[7];
        for (int l = 0; l < 7; ++l) v[l] = m.gfm[l][o1];
        extrm_wall_put(g, m, e, v);
    }
}
// INTPM: INTP's positions, stages and carried-F1 codes on the seven species
template <typename R>
__global__ void k_intpm(Ctx<R> c, MinorDev<R> m, int stage) {
    const GeoT<R>& g = c.g;
    int i0, i1, j0, j1, js, k0, k1, ks;
    if (stage == 1) { i0 = 2; i1 = g.MP; j0 = 2; j1 = g.NP; js = 2; k0 = 3; k1 = g.LPM1; ks = 2; }
    else if (stage == 2) { i0 = 2; i1 = g.MP; j0 = 3; j1 = g.NPM1; js = 2; k0 = 2; k1 = g.LP; ks = 1; }
    else { i0 = 3; i1 = g.MPM1; j0 = 2; j1 = g.NP; js = 1; k0 = 2; k1 = g.LP; ks = 1; }
    const int ni = (i1 - i0) / 2 + 1, nj = (j1 - j0) / js + 1, nk = (k1 - k0) / ks + 1;
    const long long tot = (long long)ni * nj * nk;
    GFM_FOR(t, tot) {
        const int I = i0 + 2 * (t % ni);
        const int r = t / ni;
        const int J = j0 + js * (r % nj), K = k0 + ks * (r / nj);
        const long long o = pidx(g, I, J, K);
        const int mode = c.intp_mode[o];
        if (mode == 0) continue;
        int I1, J1, K1, I2, J2, K2, ix;
        if (stage == 1) { I1 = I; J1 = J; K1 = K + 1; I2 = I; J2 = J; K2 = K - 1; ix = 3; }
        else if (stage == 2) { I1 = I; J1 = J + 1; K1 = K; I2 = I; J2 = J - 1; K2 = K; ix = 2; }
        else { I1 = I + 1; J1 = J; K1 = K; I2 = I - 1; J2 = J; K2 = K; ix = 1; }
        const R f1 = mode == 1 ? intp1(g, I, J, K, ix) : (mode == 2 ? R(1) : R(0));
        const R f2 = R(1) - f1;
        const long long a = pidx(g, I1, J1, K1), b = pidx(g, I2, J2, K2);
        for (int l = 0; l < 7; ++l) m.gfm[l][o] = f1 * m.gfm[l][a] + f2 * m.gfm[l][b];
    }
}

// P at the reference inlet and the re-reference shift G0 (Gflow.f90:182-242)
template <typename R>
__global__ void k_pref(Ctx<R> c, int I1, int J1, int K1, int I2, int J2, int K2, double F1, double F2) {
    const GeoT<R>& g = c.g;
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    A(c.P, c.i_ref, c.j_ref, c.k_ref) = A(c.P, I1, J1, K1) * R(F1) + A(c.P, I2, J2, K2) * R(F2);
    c.scal[S_G0] = (double)(A(c.P, I1, J1, K1) - R(c.p_ref));
}

// ---------------------------------------------------------------------------
// Emission-only radiation (rad_qe_only, Rad_emis.f90:411-466; RAD0 with gray
// bands, Rad0.f90:112-157; DEBX Rad_fun.f90:122-140).  QE on every centre
// (zero where the cell does not emit), then T=(T*T0)/T0 as the reference's
// whole-array round trip does.
// ---------------------------------------------------------------------------
// 1/n and its powers for the terms of RIF(3,0,X), n = 1..1000, formed once on
// the host with the products the device formed per term before (the same
// bits: q = 1/n, then q*q, q2*q, q3*q).  Every thread of
// a warp reads the same n at once, a broadcast from constant memory, so a
// term costs no division on the narrow FP64 pipe.
constexpr int kRifTerms = 1000;
__constant__ double c_rif_q[4 * kRifTerms];

int prepare_rif_table() {
    static double tab[4 * kRifTerms];
    for (int n = 1; n <= kRifTerms; ++n) {
        const double q = 1.0 / (double)n;
        const double q2 = q * q, q3 = q2 * q, q4 = q3 * q;
        double* t = tab + 4 * (n - 1);
        t[0] = q; t[1] = q2; t[2] = q3; t[3] = q4;
    }
    return cudaMemcpyToSymbol(c_rif_q, tab, sizeof tab) == cudaSuccess ? GFM_OK : GFM_E_CUDA;
}

// RIF(3,0,X) of rif3 (physics.h) with exp(-n*x) formed as the n-th power of
// exp(-x) and the powers of 1/n from the table: one exponential per call and
// no division per term in place of one exponential and four divisions per
// term (the same sum to the last bits).
__device__ __forceinline__ double rif3_tab(double x) {
    const double pi = 3.141592653589793;
    if (x > 1.0e16) return 0.0;
    if (x == 0.0) return 1.0;
    const double ex = exp(-x);
    const double x2 = x * x, x3 = x2 * x;
    double e = ex;
    double r = 0.0;
    for (int n = 1; n <= kRifTerms; ++n) {
        const double* q = c_rif_q + 4 * (n - 1);
        double g0 = 0.0;
        g0 = g0 + x3 * q[0];
        g0 = g0 + 3.0 * x2 * q[1];
        g0 = g0 + 6.0 * x * q[2];
        g0 = g0 + 6.0 * q[3];
        g0 = g0 * e;
        r = r + g0;
        if (fabs(g0) <= 1.0e-16) break;
        e = e * ex;
    }
    r = r * 1.5e1 / (pi * pi * pi * pi);
    return r > 1.0 ? 1.0 : r;
}

template <typename R>
__global__ void k_rad_emission(Ctx<R> c, const double* __restrict__ gas_aklg, const double* __restrict__ gas_akls) {
    const GeoT<R>& g = c.g;
    const int hx = g.HX, hy = g.HY, hz = g.HZ;
    const long long tot = (long long)hx * hy * hz;
    const double sgn = c.p.sig * c.p.ri * c.p.ri;
    GFM_FOR(t, tot) {
        int ia = t % hx;
        int r = t / hx;
        int ja = r % hy, ka = r / hy;
        int I = 2 * ia, J = 2 * ja, K = 2 * ka;
        if (I < 2 || J < 2 || K < 2) continue;
        const long long o = pidx(g, I, J, K);
        double qe = 0.0;
        double T_rad = (double)c.T[o] * c.p.t0;
        if (g.ib[o] <= 0 && T_rad >= 300.0) {
            double dx = g.DX[I], dr = g.DR[J], dz = g.DZ[K];
            double vol = dx * dr * (double)g.RS[J] * dz;   // VOL_C0
            if (g.HALF && g.ib[o] <= -1) vol = vol * (double)g.BVF[-g.ib[o] - 1];
            double sa = ((dx * dr) + (dr * dz) + (dx * dz)) * 2.0;
            double opl = sa > 1.0e-16 ? 6.0 * vol / sa : 0.0;
            if (sa > 1.0e-16 && opl > 1.0e-10) {
                double deb[16], eb0 = 0.0;
                for (int l = 1; l <= c.nwl - 1; ++l) {
                    double x1 = (c.p.hck / c.p.ri / c.wl[l - 1]) / T_rad;
                    double eb1 = rif3_tab(x1);
                    deb[l - 1] = eb1 - eb0;
                    if (deb[l - 1] <= 1.0e-3) deb[l - 1] = 0.0; else eb0 = eb1;
                }
                deb[c.nwl - 1] = 1.0 - eb0;
                double t2 = T_rad * T_rad;
                double s = 0.0;
                if (gas_aklg) {   // AKL0 = AKLG + AKLS of the band model, per cell (I fastest)
                    const int mz = g.MP / 2, ncl = mz * (g.NP / 2) * (g.LP / 2);
                    const int cc = (ia - 1) + mz * ((ja - 1) + (g.NP / 2) * (ka - 1));
                    for (int l = 0; l < c.nwl; ++l)
                        s = s + deb[l] * emf(gas_aklg[cc + (long long)l * ncl] + gas_akls[cc + (long long)l * ncl], opl);
                } else {
                    for (int l = 0; l < c.nwl; ++l) s = s + deb[l] * emf(c.akl0[l], opl);
                }
                qe = sa * sgn * (t2 * t2) * s;
            }
        }
        c.QE[o] = R(qe);
    }
}
template <typename R>
__global__ void k_t_roundtrip(R* T, long long n, double t0) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        T[t] = R(((double)T[t] * t0) / t0);
}

// ---------------------------------------------------------------------------
// layout conversion
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_to_split(GeoT<R> g, const double* __restrict__ src, R* __restrict__ dst) {
    const long long n = (long long)g.MP * g.NP * g.LP;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int I = (int)(t % g.MP) + 1;
        long long r = t / g.MP;
        int J = (int)(r % g.NP) + 1, K = (int)(r / g.NP) + 1;
        dst[pidx(g, I, J, K)] = R(src[t]);
    }
}
// conversion of an uploaded field with its count of non-finite values, one
// read of the source (which may be mapped host memory)
template <typename R>
__global__ void k_to_split_count(GeoT<R> g, const double* __restrict__ src, R* __restrict__ dst, unsigned int* cnt) {
    const long long n = (long long)g.MP * g.NP * g.LP;
    unsigned int local = 0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int I = (int)(t % g.MP) + 1;
        long long r = t / g.MP;
        int J = (int)(r % g.NP) + 1, K = (int)(r / g.NP) + 1;
        const double v = src[t];
        local += isfinite(v) ? 0u : 1u;
        dst[pidx(g, I, J, K)] = R(v);
    }
    if (local) atomicAdd(cnt, local);
}
template <typename R>
__global__ void k_from_split(GeoT<R> g, const R* __restrict__ src, double* __restrict__ dst) {
    const long long n = (long long)g.MP * g.NP * g.LP;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int I = (int)(t % g.MP) + 1;
        long long r = t / g.MP;
        int J = (int)(r % g.NP) + 1, K = (int)(r / g.NP) + 1;
        dst[t] = (double)src[pidx(g, I, J, K)];
    }
}
template <typename R>
__global__ void k_cells_to_split(GeoT<R> g, const double* __restrict__ src, R* __restrict__ dst, int mz, int nz, int lz) {
    const long long n = (long long)mz * nz * lz;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int id = (int)(t % mz) + 1;
        long long r = t / mz;
        int jd = (int)(r % nz) + 1, kd = (int)(r / nz) + 1;
        dst[pidx(g, 2 * id, 2 * jd, 2 * kd)] = R(src[t]);
    }
}
template <typename R>
__global__ void k_cells_from_split(GeoT<R> g, const R* __restrict__ src, double* __restrict__ dst, int mz, int nz, int lz) {
    const long long n = (long long)mz * nz * lz;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int id = (int)(t % mz) + 1;
        long long r = t / mz;
        int jd = (int)(r % nz) + 1, kd = (int)(r / nz) + 1;
        dst[t] = (double)src[pidx(g, 2 * id, 2 * jd, 2 * kd)];
    }
}

// ---------------------------------------------------------------------------
// deterministic finish of block partials (FinishSpec in state.cuh)
// ---------------------------------------------------------------------------
// one block per item; each block adds its 1024 partials in a fixed order
__global__ void k_finish(const double* __restrict__ partials, double* scal, FinishSpec f, double ncells) {
    __shared__ double sh[32];
    for (int q = blockIdx.x; q < f.n; q += gridDim.x) {
        const double* p = partials + (long long)f.slot[q] * kRedBlocks;
        double v = f.op[q] == 1 ? -1.0e308 : 0.0;
        for (int b = threadIdx.x; b < kRedBlocks; b += blockDim.x) v = f.op[q] == 1 ? (p[b] > v ? p[b] : v) : v + p[b];
        double tot = f.op[q] == 1 ? block_max(v, sh) : block_sum(v, sh);
        if (threadIdx.x == 0) {
            double out = tot;
            if (f.op[q] == 2) { out = tot / ncells; out = out > 1.0e-16 ? out : 1.0e-16; }
            else if (f.op[q] == 3) out = tot / ncells;
            scal[f.dst[q]] = out;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <typename R> void launch_extr(const Ctx<R>& c, cudaStream_t s) {
    k_extr_io<R><<<gridn(c.n_extr_io), kBlk, 0, s>>>(c);
    if (c.n_extr_ft > 0) {
        k_extr_ft_gather<R><<<gridn(c.n_extr_ft), kBlk, 0, s>>>(c);
        k_extr_ft_apply<R><<<gridn(c.n_extr_ft), kBlk, 0, s>>>(c);
    }
    if (c.n_extr_wall > 0) k_extr_wall<R><<<gridn(c.n_extr_wall), kBlk, 0, s>>>(c);
}
template <typename R> void launch_extrv(const Ctx<R>& c, int mex, cudaStream_t s) {
    int first = 0;
    for (int d = 0; d < 3; ++d) {
        // one block per direction pass: the partial sums of the three passes go
        // to blocks 0..2 of slots 10-13
        Ctx<R> cc = c;
        cc.partials = c.partials + d;   // shift so block 0 of pass d lands in column d
        k_extrv<R><<<1, kBlk, 0, s>>>(cc, mex, first, c.n_extrv[d]);
        first += c.n_extrv[d];
    }
}
template <typename R> void launch_intpv(const Ctx<R>& c, cudaStream_t s) {
    const GeoT<R>& g = c.g;
    for (int IU = 1; IU <= 3; ++IU) {
        int M3, N3, L3;
        if (IU == 1) { M3 = g.MP; N3 = g.NP; L3 = g.LP; } else if (IU == 2) { M3 = g.NP; N3 = g.LP; L3 = g.MP; } else { M3 = g.LP; N3 = g.MP; L3 = g.NP; }
        int ixa = IU == 1 ? 2 : (IU == 2 ? 3 : 1), ixb = IU == 1 ? 3 : (IU == 2 ? 1 : 2);
        long long na = (long long)((M3 - 4) / 2 + 1) * ((N3 - 4) / 2 + 1) * (L3 / 2);
        if (N3 > 3) k_intpv<R><<<gridn(na), kBlk, 0, s>>>(c, IU, 0, 3, M3 - 1, 2, 3, N3 - 1, 2, 2, L3, 2, ixa);
        long long nb = (long long)((M3 - 4) / 2 + 1) * (N3 - 1) * ((L3 - 4) / 2 + 1);
        if (L3 > 3) k_intpv<R><<<gridn(nb), kBlk, 0, s>>>(c, IU, 1, 3, M3 - 1, 2, 2, N3, 1, 3, L3 - 1, 2, ixb);
        long long nc = (long long)((M3 - 4) / 2 + 1) * (N3 - 1) * (L3 - 1);
        k_intpv<R><<<gridn(nc), kBlk, 0, s>>>(c, IU, 2, 4, M3, 2, 2, N3, 1, 2, L3, 1, IU);
    }
}
template <typename R> void launch_initsvm(const Ctx<R>& c, const MinorDev<R>& m, int restart, cudaStream_t s) {
    k_initsvm<R><<<gridn((long long)c.g.MP * c.g.NP * c.g.LP), kBlk, 0, s>>>(c, m, restart);
}
template <typename R> void launch_extrm(const Ctx<R>& c, const MinorDev<R>& m, cudaStream_t s) {
    if (c.n_extr_io > 0) k_extrm_exit<R><<<gridn(c.n_extr_io), kBlk, 0, s>>>(c, m);
    if (c.n_extr_ft > 0) {
        k_extrm_ft_gather<R><<<gridn(c.n_extr_ft), kBlk, 0, s>>>(c, m);
        k_extrm_ft_apply<R><<<gridn(c.n_extr_ft), kBlk, 0, s>>>(c, m);
    }
    if (c.n_extr_wall > 0) k_extrm_wall<R><<<gridn(c.n_extr_wall), kBlk, 0, s>>>(c, m);
}
template <typename R> void launch_intpm(const Ctx<R>& c, const MinorDev<R>& m, cudaStream_t s) {
    long long n = (long long)c.g.MP * c.g.NP * c.g.LP / 4;
    for (int st = 1; st <= 3; ++st) k_intpm<R><<<gridn(n), kBlk, 0, s>>>(c, m, st);
}
template <typename R> void launch_intp(const Ctx<R>& c, cudaStream_t s) {
    long long n = (long long)c.g.MP * c.g.NP * c.g.LP / 4;
    for (int st = 1; st <= 3; ++st) k_intp<R><<<gridn(n), kBlk, 0, s>>>(c, st);
}
template <typename R> void launch_rad_emission(const Ctx<R>& c, cudaStream_t s, const double* gas_aklg,
                                               const double* gas_akls) {
    long long n = (long long)c.g.HX * c.g.HY * c.g.HZ;
    k_rad_emission<R><<<gridn(n), kBlk, 0, s>>>(c, gas_aklg, gas_akls);
    k_t_roundtrip<R><<<gridn(8 * c.g.CB), kBlk, 0, s>>>(c.T, 8 * c.g.CB, c.p.t0);
}
template <typename R> void launch_factor(const Ctx<R>& c, cudaStream_t s) {
    k_factor<<<1, 32, 0, s>>>(c.scal, c.p.gmfr, c.p.t0, c.p.f_mx, c.p.f_mn);
}
void launch_finish(const double* partials, double* scal, const FinishSpec& f, double ncells, cudaStream_t s) {
    k_finish<<<f.n > 0 ? f.n : 1, 256, 0, s>>>(partials, scal, f, ncells);
}
template <typename R> void launch_pref_idx(const Ctx<R>& c, int I1, int J1, int K1, int I2, int J2, int K2, double F1, double F2,
                                           cudaStream_t s) {
    k_pref<R><<<1, 32, 0, s>>>(c, I1, J1, K1, I2, J2, K2, F1, F2);
}
template <typename R> void launch_to_split(const GeoT<R>& g, const double* src, R* dst, cudaStream_t s) {
    k_to_split<R><<<gridn((long long)g.MP * g.NP * g.LP), kBlk, 0, s>>>(g, src, dst);
}
template <typename R> void launch_to_split_count(const GeoT<R>& g, const double* src, R* dst, unsigned int* cnt, cudaStream_t s) {
    k_to_split_count<R><<<gridn((long long)g.MP * g.NP * g.LP), kBlk, 0, s>>>(g, src, dst, cnt);
}
template <typename R> void launch_from_split(const GeoT<R>& g, const R* src, double* dst, cudaStream_t s) {
    k_from_split<R><<<gridn((long long)g.MP * g.NP * g.LP), kBlk, 0, s>>>(g, src, dst);
}
template <typename R> void launch_cells_to_split(const GeoT<R>& g, const double* src, R* dst, cudaStream_t s) {
    k_cells_to_split<R><<<gridn((long long)(g.MP / 2) * (g.NP / 2) * (g.LP / 2)), kBlk, 0, s>>>(g, src, dst, g.MP / 2, g.NP / 2, g.LP / 2);
}
template <typename R> void launch_cells_from_split(const GeoT<R>& g, const R* src, double* dst, cudaStream_t s) {
    k_cells_from_split<R><<<gridn((long long)(g.MP / 2) * (g.NP / 2) * (g.LP / 2)), kBlk, 0, s>>>(g, src, dst, g.MP / 2, g.NP / 2, g.LP / 2);
}

#define INST(R)                                                                                                     \
    template void launch_extr<R>(const Ctx<R>&, cudaStream_t);                                                     \
    template void launch_extrv<R>(const Ctx<R>&, int, cudaStream_t);                                               \
    template void launch_intpv<R>(const Ctx<R>&, cudaStream_t);                                                    \
    template void launch_intp<R>(const Ctx<R>&, cudaStream_t);                                                     \
    template void launch_initsvm<R>(const Ctx<R>&, const MinorDev<R>&, int, cudaStream_t);                         \
    template void launch_extrm<R>(const Ctx<R>&, const MinorDev<R>&, cudaStream_t);                                \
    template void launch_intpm<R>(const Ctx<R>&, const MinorDev<R>&, cudaStream_t);                                \
    template void launch_rad_emission<R>(const Ctx<R>&, cudaStream_t, const double*, const double*);                                             \
    template void launch_factor<R>(const Ctx<R>&, cudaStream_t);                                                   \
    template void launch_pref_idx<R>(const Ctx<R>&, int, int, int, int, int, int, double, double, cudaStream_t);  \
    template void launch_to_split<R>(const GeoT<R>&, const double*, R*, cudaStream_t);                             \
    template void launch_to_split_count<R>(const GeoT<R>&, const double*, R*, unsigned int*, cudaStream_t);        \
    template void launch_from_split<R>(const GeoT<R>&, const R*, double*, cudaStream_t);                           \
    template void launch_cells_to_split<R>(const GeoT<R>&, const double*, R*, cudaStream_t);                       \
    template void launch_cells_from_split<R>(const GeoT<R>&, const R*, double*, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace gfm
