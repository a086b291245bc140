// gas.cu -- the gas and soot band model of RAD0's open cells (Rad0.f90:116-132
// with RAD_GAS, AH2O, ACO2, A1, CHIWHI, BANDA, Rad_gas.f90:16-395, and SOOTA,
// SOC, Rad_soot.f90:26-69): per cell, the wave-number intervals the H2O and
// CO2 bands cover at the cell's temperature, pressure, composition and mean
// beam length OPL, merged and integrated over the spectral bands into AKLG,
// and the soot coefficient AKLS from the soot volume fraction.
//
// One thread per cell.  The reference keeps its band-model variables in
// module GBL_VAR and runs the cells in loop order (I outer, K inner), and one
// of them carries over: SOOTA leaves AKLS as the previous cell set it when a
// cell's soot volume fraction is below 1e-14 (Rad_soot.f90:29; AKLS is zeroed
// once per RAD0 call, Rad0.f90:27).  Here that is a prefix maximum over the
// cells' loop-order positions of the last cell that set AKLS, and AKLS is
// formed from that cell's soot volume fraction.  AACO2 carries over too when
// W_R <= 0 (Rad_gas.f90:233), which needs a non-positive pressure with
// YCO2 > 1e-4; that, and BANDA's stop_run on a negative argument
// (Rad_gas.f90:368-371), set an error bit instead.
//
// CHIWHI at the reference temperature T0_R depends on the cell only through
// the final division by SQRT(TT0) (Rad_gas.f90:341-344): CHI and YN/XY there
// are formed once on the host for each of the twelve call sites, with the
// same operations, and the device divides by the cell's SQRT(TT0).
#include "state.cuh"

#include <cmath>
#include <type_traits>

namespace gfm {
namespace {

constexpr double kT0R = 1.0e2, kP0R = 1.01325e5;   // Var_mod.f90:135-136
constexpr double kHckR = 1.439e-2;                   // Var_mod.f90:134
constexpr double kWco2 = 44.0098, kWh2o = 18.0152;   // Var_mod.f90:145-146
constexpr double kDnstSoot = 1.8e3;                  // Var_mod.f90:137
// molecular weights of the minor species (Var_mod.f90:223-229)
__host__ __device__ inline double wms(int m) {
    switch (m) {
        case 0: return 16.0426;
        case 1: return 31.9988;
        case 2: return 28.0104;
        case 3: return 18.0152;
        case 4: return 44.0098;
        case 5: return 28.0134;
        default: return 30.0061;
    }
}
constexpr double kTgMnGas = 300.0;                   // TG_MN (Rad0.f90:42)
constexpr int kScanBlock = 1024;

// The twelve (V, NG, ND_R) combinations AH2O and ACO2 pass to CHIWHI, in
// the order they are met: H2O bands 1, 2, the three parts of band 3, 4, 5;
// CO2 band 1, bands 2 and 3, 4, 5, 6 (Rad_gas.f90:161-207, 235-269)
enum GasSite { H1, H2, H3A, H3B, H3C, H4, H5, C1, C23, C4, C5, C6, kSites };
// gas of a site: 0 H2O (NG 1,1,1), 1 CO2 (NG 1,2,1); ND_R(K) of a site
__host__ __device__ inline int site_gas(int s) { return s >= C1 ? 1 : 0; }
__host__ __device__ inline int site_nd(int s, int k) {
    switch (s) {
        case H2: return k == 1 ? 1 : 0;
        case H3A: return k == 1 ? 2 : 0;
        case H3B: return k == 0 ? 1 : 0;
        case H3C: return k == 2 ? 1 : 0;
        case H4: return k == 0 ? 0 : 1;
        case H5: return k == 1 ? 0 : 1;
        case C1: return k == 1 ? 1 : 0;
        case C23: return k == 0 ? -1 : k == 1 ? 0 : 1;
        case C4: return k == 2 ? 1 : 0;
        case C5: return k == 1 ? 0 : 1;
        case C6: return k == 0 ? 2 : k == 1 ? 0 : 1;
        default: return 0;
    }
}
__host__ __device__ inline double site_v(int gas, int k) {
    return gas == 0 ? (k == 0 ? 3.652e+5 : k == 1 ? 1.595e+5 : 3.756e+5) : (k == 0 ? 1.351e+5 : k == 1 ? 6.67e+4 : 2.396e+5);
}
__host__ __device__ inline int site_ng(int gas, int k) { return gas == 1 && k == 1 ? 2 : 1; }

struct GasConst {
    double chi0[kSites], ynxy0[kSites];   // CHI and YN/XY of CHIWHI at T0_R
    double soot_g0[kRadMaxBands];         // 18*PI*X2NK/((XN_K+2)^2+X2NK^2) of SOC(WL(N))
    double wl[kRadMaxBands];
    int nwl;
};

__host__ __device__ inline double per(int M, int N) {   // PER, Rad_fun.f90:14-31 (M >= N here)
    double p = 1.0;
    if (M == 0 || N == 0) return p;
    for (int I = M - N + 1; I <= M; ++I) p = p * I;
    return p;
}
// the same in integers: CHIWHI's factors stay below 103*102*101, exact in int
__host__ __device__ inline int per_i(int M, int N) {
    int p = 1;
    if (M == 0 || N == 0) return p;
    for (int I = M - N + 1; I <= M; ++I) p = p * I;
    return p;
}

// CHIWHI's sums (Rad_gas.f90:314-340) for a site with some ND_R non-zero:
// CHI and YN/XY at temperature TT
__host__ __device__ inline void chiwhi_sums(int s, double TT, double& CHI, double& YNXY) {
    const int gas = site_gas(s);
    double UD = 0.0, XD = 0.0, XY = 0.0, YN = 0.0;
    for (int K = 0; K < 3; ++K) {
        const int ng = site_ng(gas, K), nd = site_nd(s, K);
        const double U = kHckR * site_v(gas, K) / TT;
        int NV = nd < 0 ? -nd : 0;
        const int NDK = nd < 0 ? -nd : nd;
        double Y1 = 0.0;
        for (;;) {
            const double XGAS = exp(-U * NV) / per(ng - 1, ng - 1);
            const double X1 = XGAS * per(NV + ng + NDK - 1, ng + NDK - 1);
            const double X2 = XGAS * per(NV + ng - 1, ng - 1);
            if (X1 < 1.0e-10) break;
            XY = XY + X1;
            XD = XD + X2;
            Y1 = Y1 + sqrt(X1);
            NV = NV + 1;
            if (NV >= 100) break;
        }
        YN = YN + Y1 * Y1;
        UD = UD - U * nd;
    }
    CHI = (1.0 - exp(UD)) * XY / XD;
    YNXY = YN / XY;
}

// The band model in the arithmetic of the path: double on the FP64 path,
// float on the mixed one (T below).  Every constant is converted to T first.

// BANDA (Rad_gas.f90:360-395)
template <typename T>
__device__ inline T banda(T ALP, T BTA, T A0, T W_R, T PE, int& err) {
    if (A0 <= T(0)) return T(0);
    if (ALP < T(0) || BTA < T(0) || A0 < T(0) || W_R * PE < T(0)) { err |= 2; return T(0); }
    if (W_R * PE == T(0)) return T(0);
    const T ETA = BTA * PE;
    const T TAU = ALP * W_R / A0;
    T A_S;
    if (ETA >= T(1)) A_S = TAU <= T(1) ? TAU : T(1) + log(TAU);
    else if (TAU <= ETA) A_S = TAU;
    else if (TAU <= T(1) / ETA) A_S = T(2) * sqrt(ETA * TAU) - ETA;
    else A_S = log(ETA * TAU) + T(2) - ETA;
    return A0 * A_S;
}

// A cell's state for the band model, with U = HCK*V/T_RAD of the three band
// centres of each gas and exp(-U), exp(-U/2): CHIWHI's terms
// exp(-U*NV)/PER(NG-1,NG-1)*PER(...) are formed as products of these powers,
// and the square roots of its integer factors PER(M,N) come from a table,
// which leaves one exponential per centre and cell in place of one per term
// (the same sums to the last bits: the powers carry NV rounding steps)
template <typename T>
struct Cell {
    T T_RAD, TT0, P_RAD, YCO2, YH2O, OPL;
    T U[2][3], eU[2][3], eUh[2][3];
};
constexpr int kPerRows = 104;   // NV + NG + NDK - 1 <= 99 + 2 + 2 - 1 (NV stops at 100)

template <typename T>
__device__ inline void chiwhi_fast(const Cell<T>& c, const T* __restrict__ sqper, int s, T& CHI, T& YNXY) {
    const int gas = site_gas(s);
    T UD = T(0), XD = T(0), XY = T(0), YN = T(0);
    for (int K = 0; K < 3; ++K) {
        const int ng = site_ng(gas, K), nd = site_nd(s, K);
        int NV = nd < 0 ? -nd : 0;
        const int NDK = nd < 0 ? -nd : nd;
        T e = T(1), eh = T(1);                    // exp(-U*NV), exp(-U*NV/2)
        for (int q = 0; q < NV; ++q) { e *= c.eU[gas][K]; eh *= c.eUh[gas][K]; }
        T Y1 = T(0);
        for (;;) {
            // PER(NG-1,NG-1) = 1 for NG = 1, 2
            const T X1 = e * T(per_i(NV + ng + NDK - 1, ng + NDK - 1));
            const T X2 = e * T(per_i(NV + ng - 1, ng - 1));
            if (X1 < T(1.0e-10)) break;
            XY = XY + X1;
            XD = XD + X2;
            Y1 = Y1 + eh * __ldg(sqper + (NV + ng + NDK - 1) * 4 + (ng + NDK - 1));
            NV = NV + 1;
            if (NV >= 100) break;
            e *= c.eU[gas][K];
            eh *= c.eUh[gas][K];
        }
        YN = YN + Y1 * Y1;
        UD = UD - c.U[gas][K] * T(nd);
    }
    CHI = (T(1) - exp(UD)) * XY / XD;
    YNXY = YN / XY;
}

// CHIWHI at T0_R and at T_RAD for one site
template <typename T>
__device__ inline void chiwhi_pair(const GasConst& k, const T* sqper, int s, const Cell<T>& c, T& CHI0, T& WHI0, T& CHI,
                                   T& WHI) {
    const T r = sqrt(c.TT0);
    if (s == H1) {   // pure rotational band: ND_R all zero
        CHI0 = T(1); WHI0 = T(1) / r; CHI = T(1); WHI = T(1) / r;
        return;
    }
    CHI0 = T(k.chi0[s]);
    WHI0 = T(k.ynxy0[s]) / r;
    T ynxy;
    chiwhi_fast(c, sqper, s, CHI, ynxy);
    WHI = ynxy / r;
}

// A1 (Rad_gas.f90:284-296)
template <typename T>
__device__ inline T a1(const GasConst& k, const T* sqper, int s, T B1, T B2, T B3, const Cell<T>& c, T W_R, T PE, int& err) {
    T CHI0, WHI0, CHI, WHI;
    chiwhi_pair(k, sqper, s, c, CHI0, WHI0, CHI, WHI);
    const T C3 = B3 * sqrt(c.T_RAD / T(kT0R));
    const T C1 = B1 * CHI / CHI0;
    const T C2 = T(2) * sqrt(C1 * C3 * B2 * WHI / WHI0);
    return banda(C1, C2, C3, W_R, PE, err);
}

// AH2O (Rad_gas.f90:149-212): band absorptances of H2O (1/m)
template <typename T>
__device__ void ah2o(const GasConst& k, const T* sqper, const Cell<T>& c, T* AA, int& err) {
    for (int n = 0; n < 5; ++n) AA[n] = T(0);
    if (c.YH2O <= T(0) || c.T_RAD <= T(3.0e+2)) return;
    const T PE = c.P_RAD + c.P_RAD * c.YH2O * (T(0.86e+1) / c.TT0 - T(0.5));
    const T W_R = c.P_RAD * c.YH2O * c.OPL / c.T_RAD / T(8.208e-2) * T(kWh2o);
    AA[0] = a1(k, sqper, H1, T(0.52e+4) * exp(T(-0.176e+2) / c.TT0), T(0.14311), T(0.284e+2), c, W_R, PE, err);
    AA[1] = a1(k, sqper, H2, T(0.412e+2), T(0.9427e-1), T(0.564e+2), c, W_R, PE, err);
    T CHI0, WHI0, CHI, WHI;
    chiwhi_pair(k, sqper, H3A, c, CHI0, WHI0, CHI, WHI);
    const T T1 = T(0.19) * CHI / CHI0, T4 = T(0.13219) * WHI / WHI0;
    chiwhi_pair(k, sqper, H3B, c, CHI0, WHI0, CHI, WHI);
    const T T2 = T(0.23e+1) * CHI / CHI0, T5 = T(0.13219) * WHI / WHI0;
    chiwhi_pair(k, sqper, H3C, c, CHI0, WHI0, CHI, WHI);
    const T T3 = T(0.224e+2) * CHI / CHI0, T6 = T(0.13219) * WHI / WHI0;
    const T C1 = T1 + T2 + T3;
    const T C3 = T(0.6e+2) * c.TT0;
    const T BTA = T(2) * sqrt(C3) * (sqrt(T1 * T4) + sqrt(T2 * T5) + sqrt(T3 * T6));
    AA[2] = banda(C1, BTA, C3, W_R, PE, err);
    AA[3] = a1(k, sqper, H4, T(3.0), T(0.8169e-1), T(0.431e2), c, W_R, PE, err);
    AA[4] = a1(k, sqper, H5, T(0.25e+1), T(0.11628), T(0.32e+2), c, W_R, PE, err);
    for (int n = 0; n < 5; ++n) AA[n] = AA[n] * T(1.0e+2);
}

// ACO2 (Rad_gas.f90:224-274): band absorptances of CO2 (1/m)
template <typename T>
__device__ void aco2(const GasConst& k, const T* sqper, const Cell<T>& c, T* AA, int& err) {
    const T W_R = c.P_RAD * c.YCO2 * c.OPL / c.T_RAD / T(8.208e-2) * T(kWco2);
    if (W_R <= T(0)) { err |= 4; for (int n = 0; n < 6; ++n) AA[n] = T(0); return; }
    const T q = c.P_RAD + c.P_RAD * c.YCO2 * T(0.3);
    T PE = pow(q, T(0.7));
    AA[0] = a1(k, sqper, C1, T(0.19e+2), T(0.6157e-1), T(0.127e2), c, W_R, PE, err);
    PE = pow(q, T(0.8));
    AA[1] = a1(k, sqper, C23, T(0.36), T(0.4017e-1), T(0.134e+2), c, W_R, PE, err);
    AA[2] = a1(k, sqper, C23, T(0.24), T(0.11888), T(0.101e+2), c, W_R, PE, err);
    AA[3] = a1(k, sqper, C4, T(0.11e+3), T(0.24723), T(0.112e+2), c, W_R, PE, err);
    PE = pow(q, T(0.65));
    AA[4] = a1(k, sqper, C5, T(4.0), T(0.13341), T(23.5), c, W_R, PE, err);
    AA[5] = a1(k, sqper, C6, T(0.66e-1), T(0.39305), T(0.345e+2), c, W_R, PE, err);
    for (int n = 0; n < 6; ++n) AA[n] = AA[n] * T(1.0e+2);
}

// RAD_GAS without SOOTA (Rad_gas.f90:23-134): AKLG of every band
template <typename T>
__device__ void rad_gas(const GasConst& k, const T* sqper, const Cell<T>& c, T* AKLG, int& err) {
    const T EPS1 = T(1.0e-4);
    T WH[5][3], WC[6][3], WNG[11][2];
    for (int n = 0; n < 5; ++n) WH[n][0] = WH[n][1] = WH[n][2] = T(0);
    for (int n = 0; n < 6; ++n) WC[n][0] = WC[n][1] = WC[n][2] = T(0);
    for (int n = 0; n < k.nwl; ++n) AKLG[n] = T(0);
    if (c.YH2O > EPS1) {
        WH[1][1] = T(1.60e+5); WH[2][1] = T(3.76e+5); WH[3][1] = T(5.35e+5); WH[4][1] = T(7.25e+5);
        T AA[5];
        ah2o(k, sqper, c, AA, err);
        WH[0][1] = AA[0] / T(2);
        WH[0][2] = AA[0];
        for (int N = 1; N < 5; ++N) {
            const T G0 = AA[N] / T(2);
            WH[N][0] = WH[N][1] - G0;
            WH[N][2] = WH[N][1] + G0;
            if (WH[N - 1][2] > WH[N][0]) WH[N - 1][2] = WH[N][0];
        }
    }
    if (c.YCO2 > EPS1) {
        WC[0][1] = T(6.67e+4); WC[1][1] = T(9.60e+4); WC[2][1] = T(1.06e+5);
        WC[3][2] = T(2.41e+5); WC[4][1] = T(3.66e+5); WC[5][1] = T(5.20e+5);
        T AA[6];
        aco2(k, sqper, c, AA, err);
        for (int N = 0; N < 6; ++N) {
            const T G0 = AA[N] / T(2);
            if (N == 0 && G0 > WC[0][1]) {
                WC[0][0] = T(0);
                WC[0][2] = AA[0];
            } else if (N == 3) {
                WC[N][1] = WC[N][2] - G0;
                WC[N][0] = WC[N][1] - G0;
            } else {
                WC[N][0] = WC[N][1] - G0;
                WC[N][2] = WC[N][1] + G0;
            }
            if (N == 0) continue;
            if (WC[N - 1][2] > WC[N][0]) WC[N - 1][2] = WC[N][0];
        }
    }
    for (int n = 0; n < 5; ++n) { WNG[n][0] = WH[n][0]; WNG[n][1] = WH[n][2]; }
    for (int n = 0; n < 6; ++n) { WNG[n + 5][0] = WC[n][0]; WNG[n + 5][1] = WC[n][2]; }
    for (int N = 0; N < 10; ++N) {
        for (int N2 = N + 1; N2 < 11; ++N2) {
            if (WNG[N][0] < WNG[N2][0]) continue;
            T t = WNG[N][0]; WNG[N][0] = WNG[N2][0]; WNG[N2][0] = t;
            t = WNG[N][1]; WNG[N][1] = WNG[N2][1]; WNG[N2][1] = t;
        }
        if (N == 0) continue;
        if (WNG[N - 1][1] > WNG[N][0]) WNG[N - 1][1] = WNG[N][0];
    }
    T WL2 = T(10) / T(k.wl[0]);
    int N0 = 10;
    for (int N = 0; N < k.nwl; ++N) {
        const T WL1 = N == k.nwl - 1 ? T(0) : T(1) / T(k.wl[N]);
        if (WL2 <= WL1 || WNG[10][1] <= WL1) { WL2 = WL1; continue; }
        T E0 = T(0);
        for (int N1 = N0; N1 >= 0; --N1) {
            if (WNG[N1][1] <= WL1) { N0 = N1; break; }
            if (WNG[N1][1] >= WL1 && WNG[N1][1] <= WL2) {
                if (WNG[N1][0] < WL1) {
                    E0 = E0 + WNG[N1][1] - WL1;
                    WNG[N1][1] = WL1;
                    N0 = N1;
                    break;
                }
                E0 = E0 + WNG[N1][1] - WNG[N1][0];
            }
        }
        if (E0 <= T(0) || WL2 <= WL1) {
            AKLG[N] = T(0);
        } else {
            E0 = E0 / (WL2 - WL1);
            T G0 = T(1) - E0;
            if (G0 <= T(1.0e-20)) G0 = T(1.0e-20);
            AKLG[N] = -log(G0) / c.OPL;
        }
        WL2 = WL1;
    }
}

template <typename R>
struct GasArgs {
    GeoT<double> g;
    const R *T, *P, *DNST, *smf;
    const R* gfm[7];
    int MZ, NZ, LZ;
    double t0, pg0, dnst0;
    GasConst k;
    double *aklg, *akls, *fvs;   // aklg/akls: cell + l*n (cell = I fastest); fvs by loop order
    const R* sqper;              // sqrt(PER(M,N)), M < kPerRows, N <= 3, at M*4 + N, in the path's arithmetic
    int* setter;                 // by loop order q = ((I/2-1)*NZ + J/2-1)*LZ + K/2-1: q or -1
    int* blockmax;
    int* err;
};

// RAD0's per-cell part for the open cells (Rad0.f90:116-132): AKLG, and
// the cells that reach SOOTA with a soot volume fraction >= 1e-14
template <typename R>
__global__ void __launch_bounds__(128) k_gas_band(GasArgs<R> a) {
    const int n = a.MZ * a.NZ * a.LZ;
    int err = 0;
    GFM_FOR(c, n) {
        const int id = c % a.MZ, jd = (c / a.MZ) % a.NZ, kd = c / (a.MZ * a.NZ);
        const int I = 2 * (id + 1), J = 2 * (jd + 1), K = 2 * (kd + 1);
        const int q = (id * a.NZ + jd) * a.LZ + kd;
        R aklg[kRadMaxBands];
        for (int l = 0; l < a.k.nwl; ++l) aklg[l] = R(0);
        int set = -1;
        double fvs = 0.0;
        const long long o = pidx(a.g, I, J, K);
        const double T_RAD = (double)a.T[o] * a.t0;
        if (a.g.ib[o] <= 0 && T_RAD >= kTgMnGas) {
            Cell<R> cl;
            cl.T_RAD = R(T_RAD);
            cl.TT0 = sqrt(R(T_RAD) / R(kT0R));
            cl.P_RAD = R((1.0 + (double)a.P[o]) * a.pg0 / kP0R);
            double sum = 0.0;
            for (int m = 0; m < 7; ++m) sum = sum + (double)a.gfm[m][o] / wms(m);
            const double wmix = 1.0 / sum;
            cl.YCO2 = R((double)a.gfm[4][o] * wmix / kWco2);
            cl.YH2O = R((double)a.gfm[3][o] * wmix / kWh2o);
            fvs = (double)a.smf[o] * (double)a.DNST[o] * a.dnst0 / kDnstSoot;
            const double dx = a.g.DX[I], dr = a.g.DR[J], dz = a.g.DZ[K];
            double vol = dx * dr * a.g.RS[J] * dz;
            if (a.g.HALF && a.g.ib[o] <= -1) vol = vol * a.g.BVF[-a.g.ib[o] - 1];
            const double sa = ((dx * dr) + (dr * dz) + (dx * dz)) * 2.0;
            if (sa > kSmall16) {
                const double opl = 6.0 * vol / sa;
                cl.OPL = R(opl);
                if (opl > 1.0e-10) {
                    for (int gs = 0; gs < 2; ++gs)
                        for (int K3 = 0; K3 < 3; ++K3) {
                            cl.U[gs][K3] = R(kHckR * site_v(gs, K3)) / cl.T_RAD;
                            cl.eU[gs][K3] = exp(-cl.U[gs][K3]);
                            cl.eUh[gs][K3] = exp(R(-0.5) * cl.U[gs][K3]);
                        }
                    rad_gas(a.k, a.sqper, cl, aklg, err);
                    if (fvs >= 1.0e-14) set = q;
                }
            }
        }
        for (int l = 0; l < a.k.nwl; ++l) a.aklg[c + (long long)l * n] = (double)aklg[l];
        a.setter[q] = set;
        a.fvs[q] = fvs;
    }
    if (err) atomicOr(a.err, err);
}

// prefix maximum of setter[] in loop order: per block, then over blocks
__global__ void __launch_bounds__(kScanBlock) k_gas_scan_block(int* setter, int n, int* blockmax) {
    __shared__ int sh[kScanBlock];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    int v = i < n ? setter[i] : -1;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = 1; s < kScanBlock; s <<= 1) {
        const int t = (int)threadIdx.x >= s ? sh[threadIdx.x - s] : -1;
        __syncthreads();
        if (t > v) v = t;
        sh[threadIdx.x] = v;
        __syncthreads();
    }
    if (i < n) setter[i] = v;
    if (threadIdx.x == kScanBlock - 1) blockmax[blockIdx.x] = v;
}
__global__ void __launch_bounds__(kScanBlock) k_gas_scan_top(int* blockmax, int nb) {
    __shared__ int sh[kScanBlock];
    int carry = -1;
    for (int b0 = 0; b0 < nb; b0 += kScanBlock) {
        const int i = b0 + threadIdx.x;
        int v = i < nb ? blockmax[i] : -1;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int s = 1; s < kScanBlock; s <<= 1) {
            const int t = (int)threadIdx.x >= s ? sh[threadIdx.x - s] : -1;
            __syncthreads();
            if (t > v) v = t;
            sh[threadIdx.x] = v;
            __syncthreads();
        }
        // exclusive prefix: the blocks before block i
        const int ex = threadIdx.x == 0 ? -1 : sh[threadIdx.x - 1];
        const int outv = ex > carry ? ex : carry;
        const int tot = sh[kScanBlock - 1];
        __syncthreads();
        if (i < nb) blockmax[i] = outv;
        if (tot > carry) carry = tot;
        __syncthreads();
    }
}

// AKLS of every cell that reached RAD_GAS: SOOTA (Rad_soot.f90:29-35) on the
// soot volume fraction of the last cell up to this one that set it
template <typename R>
__global__ void k_gas_soot(GasArgs<R> a) {
    const int n = a.MZ * a.NZ * a.LZ;
    GFM_FOR(c, n) {
        const int id = c % a.MZ, jd = (c / a.MZ) % a.NZ, kd = c / (a.MZ * a.NZ);
        const int q = (id * a.NZ + jd) * a.LZ + kd;
        int src = a.setter[q];
        const int bp = a.blockmax[q / kScanBlock];
        if (bp > src) src = bp;
        const double f = src >= 0 ? a.fvs[src] : 0.0;
        for (int l = 0; l < a.k.nwl; ++l)
            a.akls[c + (long long)l * n] = src >= 0 ? a.k.soot_g0[l] * f / a.k.wl[l] : 0.0;
    }
}

// SOC (Rad_soot.f90:49-69) on the host: the soot optical constants' factor
// of SOOTA for band edge WL0
double soot_g0(double WL0) {
    const double SOCF[3] = {7.2e+26, 4.07e+27, 4.47e+28};
    const double SOCH[3] = {1.2e+15, 5.90e+15, 5.60e+15};
    const double SOCW[3] = {0.0, 1.25e+15, 7.25e+15};
    const double C_0 = 2.9984e+8, E2ME0 = 3.185e+3, PI = 3.141592653589793;
    double XN_K = 1.0, X2NK = 0.0;
    const double W = 2.0 * PI * C_0 / WL0;
    for (int J = 0; J < 3; ++J) {
        const double A = SOCW[J] * SOCW[J] - W * W;
        const double B = A * A + W * W * SOCH[J] * SOCH[J];
        if (B < 1.0e-20) break;
        const double G0 = SOCF[J] * E2ME0;
        XN_K = XN_K + G0 * A / B;
        X2NK = X2NK + G0 * SOCH[J] * W / B;
    }
    return 18.0 * PI * X2NK / ((XN_K + 2.0) * (XN_K + 2.0) + X2NK * X2NK);
}

}  // namespace

int gas_scan_blocks(int ncell) { return (ncell + kScanBlock - 1) / kScanBlock; }

int gas_sqper_size() { return kPerRows * 4; }
void gas_sqper_fill(double* t) {
    for (int m = 0; m < kPerRows; ++m)
        for (int n = 0; n < 4; ++n) t[m * 4 + n] = n <= m ? std::sqrt(per(m, n)) : 0.0;
}

void launch_prefix_max(int* a, int n, int* blockmax, cudaStream_t st) {
    const int nb = gas_scan_blocks(n);
    k_gas_scan_block<<<nb, kScanBlock, 0, st>>>(a, n, blockmax);
    k_gas_scan_top<<<1, kScanBlock, 0, st>>>(blockmax, nb);
}

template <typename R>
int launch_gas_band(const GasBuffers& b, const GeoT<double>& g, const R* T, const R* P, const R* DNST,
                    const R* const* gfm, const R* smf, double t0, double pg0, double dnst0, int nwl, const double* wl,
                    cudaStream_t st) {
    if (nwl < 1 || nwl > kRadMaxBands) return GFM_E_ARG;
    GasArgs<R> a{};
    a.g = g;
    a.T = T; a.P = P; a.DNST = DNST; a.smf = smf;
    for (int m = 0; m < 7; ++m) a.gfm[m] = gfm[m];
    a.MZ = g.MP / 2; a.NZ = g.NP / 2; a.LZ = g.LP / 2;
    a.t0 = t0; a.pg0 = pg0; a.dnst0 = dnst0;
    a.k.nwl = nwl;
    for (int l = 0; l < nwl; ++l) { a.k.wl[l] = wl[l]; a.k.soot_g0[l] = soot_g0(wl[l]); }
    for (int s = 0; s < kSites; ++s) {
        if (s == H1) { a.k.chi0[s] = 1.0; a.k.ynxy0[s] = 1.0; continue; }
        chiwhi_sums(s, kT0R, a.k.chi0[s], a.k.ynxy0[s]);
    }
    a.aklg = b.aklg; a.akls = b.akls; a.fvs = b.fvs; a.setter = b.setter; a.blockmax = b.blockmax; a.err = b.err;
    if constexpr (std::is_same<R, double>::value) a.sqper = b.sqper;
    else a.sqper = b.sqperf;
    const int n = a.MZ * a.NZ * a.LZ;
    const int gb = (n + 127) / 128 < 4096 ? (n + 127) / 128 : 4096;
    k_gas_band<R><<<gb, 128, 0, st>>>(a);
    launch_prefix_max(b.setter, n, b.blockmax, st);
    k_gas_soot<R><<<(n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096, 256, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? GFM_OK : GFM_E_CUDA;
}
template int launch_gas_band<double>(const GasBuffers&, const GeoT<double>&, const double*, const double*, const double*,
                                     const double* const*, const double*, double, double, double, int, const double*,
                                     cudaStream_t);
template int launch_gas_band<float>(const GasBuffers&, const GeoT<double>&, const float*, const float*, const float*,
                                    const float* const*, const float*, double, double, double, int, const double*,
                                    cudaStream_t);

}  // namespace gfm
