// gfm_oracle.cpp -- TEST INFRASTRUCTURE ONLY: single-threaded FP64 C++
// restatement of the reference's steady SIMPLER iteration (GFLOW and callees,
// combustion/Code/*.f90), used as the parity checker and CPU baseline.
//
// Every routine keeps the Fortran loop order, array layout (doubled staggered
// grid, column-major, 1-based indices) and expression order.  Build with
// -ffp-contract=off so x86 and Arm hosts give the same bits.
#include "gfm_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

typedef std::vector<double> vec;

const double ZERO = 0.0, ONE = 1.0, TWO = 2.0, HALF = 0.5;
const double small20 = 1.0e-20, small16 = 1.0e-16, BIG = 1.0e+20;
const double WF = 16.0426, WO2 = 31.9988, WCO2 = 44.0098, WH2O = 18.0152, WN2 = 28.0134;
const int IYF = 1, IYO2 = 2, IH = 3, IK = 4, IEPS = 5, IYCO2 = 6, IYN2 = 7, IYH2O = 9;
const int LSTAR = 1, LEND = 7;
const double SMX0 = 1.0e-14;
const double CP0 = 1.0057e+3;
const double CPF1 = 2.156e+3 / 1.0057e+3, CPO21 = 0.9136e+3 / 1.0057e+3, CPCO21 = 2.0e+3 / 1.0057e+3,
             CPH2O1 = 2.0e+3 / 1.0057e+3, CPN21 = 0.526e+3 / 1.0057e+3;   // Var_mod.f90:156-160

// NIST Shomate sets (Setup.f90:103-141), [species][lo/hi], species CH4,O2,CO2,N2,H2O
const double A_N[5][2] = {{-0.703029, 85.81217}, {29.659, 29.659}, {24.99735, 58.16639}, {26.092, 26.092}, {30.092, 41.96426}};
const double B_N[5][2] = {{108.4773, 11.26467}, {6.137261, 6.137261}, {55.18696, 2.720074}, {8.218801, 8.218801}, {6.832514, 8.622053}};
const double C_N[5][2] = {{-42.52157, -2.114146}, {-1.186521, -1.186521}, {-33.69137, -0.492289}, {-1.976141, -1.976141}, {6.793435, -1.49978}};
const double D_N[5][2] = {{5.862788, 0.13819}, {0.09578, 0.09578}, {7.948387, 0.038844}, {0.159274, 0.159274}, {-2.53448, 0.098119}};
const double E_N[5][2] = {{0.678565, -26.42221}, {-0.219663, -0.219663}, {-0.136638, -6.447293}, {0.044434, 0.044434}, {0.082139, -11.15764}};
const double F_N[5][2] = {{-76.84376, -153.5327}, {-9.861391, -9.861391}, {-403.6075, -425.9186}, {-7.98923, -7.98923}, {-250.881, -272.1797}};
const double H_N[5][2] = {{-74.8731, -74.8731}, {0.0, 0.0}, {-393.5224, -393.5224}, {0.0, 0.0}, {-241.8264, -241.8264}};
const double CUTT[5] = {1300.0, 6000.0, 1200.0, 6000.0, 1700.0};
const int GFCI[5] = {IYF, IYO2, IYCO2, IYN2, IYH2O};   // gf_chem_index
const double T0C = 5.0e+2;
const double H0C = 1.0057e+3 * (5.0e+2 - 298.15);

inline double fmax2(double a, double b) { return a > b ? a : b; }   // Fortran MAX(a,b): NaN in a -> b
inline double fmin2(double a, double b) { return a < b ? a : b; }

// ---------------------------------------------------------------------------
// Prop.f90 routines on a 9-component GF vector accessed with stride s
// ---------------------------------------------------------------------------
struct Y9 {
    double* p; long s;
    double& operator()(int l) const { return p[(long)(l - 1) * s]; }
};

void conc(Y9 y) {   // CONC, Prop.f90:28-59
    double g0 = y(IYF) + y(IYO2) + y(IYCO2) + y(IYN2);
    if (g0 > ONE) {
        g0 = g0 + y(IYH2O);
        y(IYF) = y(IYF) / g0;
        y(IYO2) = y(IYO2) / g0;
        y(IYCO2) = y(IYCO2) / g0;
        y(IYN2) = y(IYN2) / g0;
        y(IYH2O) = y(IYH2O) / g0;
    } else {
        y(IYH2O) = ONE - g0;
    }
}

double wmix(Y9 y) {
    return ONE / (y(IYF) / WF + y(IYCO2) / WCO2 + y(IYH2O) / WH2O + y(IYO2) / WO2 + y(IYN2) / WN2);
}

struct Mix { double a, b, c, d, e, f, h; int lohi[5]; };

void mix_coeffs(Y9 y, double real_T, Mix& m) {   // Prop.f90:396-418 (incl. f_mix=d_mix+... quirk)
    m.a = m.b = m.c = m.d = m.e = m.f = m.h = 0;
    for (int n = 0; n < 5; ++n) {
        int st = real_T < CUTT[n] ? 0 : 1;
        double g = y(GFCI[n]);
        m.a = m.a + g * A_N[n][st];
        m.b = m.b + g * B_N[n][st];
        m.c = m.c + g * C_N[n][st];
        m.d = m.d + g * D_N[n][st];
        m.e = m.e + g * E_N[n][st];
        m.f = m.d + g * F_N[n][st];
        m.h = m.e + g * H_N[n][st];
        m.lohi[n] = st + 1;
    }
}

double enth_to_T(Y9 y, double t_now) {   // enth_to_T, Prop.f90:369-505
    double w_mix = wmix(y);
    double h_s = y(IH) * H0C;
    double h_molar = h_s * w_mix / 1.0e6;
    double real_T = t_now * T0C;
    Mix m;
    mix_coeffs(y, real_T, m);
    double T_old = real_T / 1000.0, T_new = T_old;
    for (int n = 1; n <= 10; ++n) {
        double gp = m.a + T_old * (m.b + T_old * (m.c + T_old * m.d)) + m.e / (T_old * T_old);
        if (gp == ZERO) break;
        double g0 = T_old * (m.a + T_old * ((m.b / 2.0) + T_old * ((m.c / 3.0) + T_old * (m.d / 4.0)))) -
                    (m.e / T_old) + m.f - m.h;
        double changeT = (g0 - h_molar) / gp;
        T_new = T_old - changeT;
        if (std::fabs(changeT) < 1.0e-11) break;
        T_old = T_new;
        for (int nn = 1; nn <= 5; ++nn) {
            if (nn == 2 || nn == 4) continue;
            int q = nn - 1;
            double g = y(GFCI[q]);
            if (T_new * 1000.0 < CUTT[q] && m.lohi[q] != 1) {
                m.a = m.a - g * A_N[q][1]; m.b = m.b - g * B_N[q][1]; m.c = m.c - g * C_N[q][1];
                m.d = m.d - g * D_N[q][1]; m.e = m.e - g * E_N[q][1];
                m.f = m.d - g * F_N[q][1]; m.h = m.e - g * H_N[q][1];
                m.lohi[q] = 1;
                m.a = m.a + g * A_N[q][0]; m.b = m.b + g * B_N[q][0]; m.c = m.c + g * C_N[q][0];
                m.d = m.d + g * D_N[q][0]; m.e = m.e + g * E_N[q][0];
                m.f = m.d + g * F_N[q][0]; m.h = m.e + g * H_N[q][0];
            }
            if (T_new * 1000.0 >= CUTT[q] && m.lohi[q] != 2) {
                m.a = m.a - g * A_N[q][0]; m.b = m.b - g * B_N[q][0]; m.c = m.c - g * C_N[q][0];
                m.d = m.d - g * D_N[q][0]; m.e = m.e - g * E_N[q][0];
                m.f = m.d - g * F_N[q][0]; m.h = m.e - g * H_N[q][0];
                m.lohi[q] = 2;
                m.a = m.a + g * A_N[q][1]; m.b = m.b + g * B_N[q][1]; m.c = m.c + g * C_N[q][1];
                m.d = m.d + g * D_N[q][1]; m.e = m.e + g * E_N[q][1];
                m.f = m.d + g * F_N[q][1]; m.h = m.e + g * H_N[q][1];
            }
        }
    }
    return T_new * 1000.0 / T0C;
}

double T_to_enth(Y9 y, double t_now) {   // T_to_enth, Prop.f90:525-565
    double w_mix = wmix(y);
    double real_T = t_now * T0C;
    Mix m;
    mix_coeffs(y, real_T, m);
    double tn = real_T / 1000.0;
    double ef = tn * (m.a + tn * ((m.b / 2.0) + tn * ((m.c / 3.0) + tn * (m.d / 4.0)))) - (m.e / tn) + m.f - m.h;
    return ef * 1.0e6 / (w_mix * H0C);
}

double DA(double D, double F) {   // Prop.f90:97-117
    const double sixth = 1.0 / 6.0;
    if (D <= 1.0e-25) return 0.0;
    double FA = std::fabs(F);
    double PE = FA / D;
    if (PE <= 1.0e-2) return D / (1.0 + PE * (0.5 + PE * (sixth + PE / 24.0)));
    if (PE <= 2.0e+1) return FA / (std::exp(PE) - 1.0);
    return 0.0;
}

double TGAMF(double B) {   // Gflow.f90:417-426
    if (B < 11.5) return 1.0;
    double G0 = B / (std::log(9 * B) * 2.5);
    return fmax2(G0, 1.0);
}

double EMF(double XKL, double XL0) {   // Rad_fun.f90:97-115
    const double X1 = 1.0e-3;
    const double G1 = (ONE - std::exp(-X1)) / X1;
    double X0 = XKL * XL0;
    return X0 <= X1 ? X0 * G1 : ONE - std::exp(-X0);
}

double RIF3(double X) {   // RIF(3,0,X), Rad_fun.f90:45-91
    const double PI = 3.141592653589793;
    if (X > 1.0e16) return 0.0;
    if (X == 0.0) return 1.0;
    const double Y[4] = {1.0, 3.0, 6.0, 6.0};   // PER(3,I), I=0..3
    double rif = 0.0;
    for (int N = 1; N <= 1000; ++N) {
        double G0 = 0.0;
        for (int I = 0; I <= 3; ++I) {
            double xp = 1.0;
            for (int q = 0; q < 3 - I; ++q) xp = xp * X;
            double an = 1.0;
            for (int q = 0; q < I + 1; ++q) an = an * (double)N;
            G0 = G0 + Y[I] * xp / an;
        }
        G0 = G0 * std::exp(-((double)N) * X);
        rif = rif + G0;
        if (std::fabs(G0) <= 1.0e-16) break;
    }
    rif = rif * 1.5e+1 / (PI * PI * PI * PI);
    return rif > 1.0 ? 1.0 : rif;
}

// ---------------------------------------------------------------------------
// Gas and soot band model of RAD0's open cells (Rad_gas.f90, Rad_soot.f90):
// the module variables the routines share (T_RAD, TT0, P_RAD, YCO2, YH2O,
// FVS, OPL, W_R, PE, AAH2O, AACO2, AKLG, AKLS) live in one object that is
// reused from cell to cell as the reference's globals are.  Two of them carry
// over between cells: AKLS when a cell's FVS < 1e-14 (SOOTA returns without
// setting it, Rad_soot.f90:29) and AACO2 when W_R <= 0 (Rad_gas.f90:233).
// ---------------------------------------------------------------------------
const double HCK_R = 1.439e-2, T0_R = 1.0e2, P0_R = 1.01325e5;     // Var_mod.f90:134-136
const double PI_R = 3.141592653589793;
const double DNST_SOOT = 1.8e3;                                     // Var_mod.f90:137
const double WMS[7] = {16.0426, 31.9988, 28.0104, 18.0152, 44.0098, 28.0134, 30.0061};   // Var_mod.f90:223-229

double PER(int M, int N) {   // Rad_fun.f90:14-31 (M >= N always holds here)
    double p = 1.0;
    if (M == 0 || N == 0) return p;
    for (int I = M - N + 1; I <= M; ++I) p = p * I;
    return p;
}

struct RadGas {
    int NWL = 0;
    const double* WL = nullptr;        // band edges (m), 0-based
    double T_RAD = 0, TT0 = 0, P_RAD = 0, YCO2 = 0, YH2O = 0, FVS = 0, OPL = 0, W_R = 0, PE = 0;
    double AAH2O[6] = {0}, AACO2[7] = {0};           // 1-based
    double WNH2O[6][4], WNCO2[7][4], WNG[12][3];     // 1-based
    vec AKLG, AKLS, AKL0, E0;                        // 1-based, NWL
    int error = 0;                                   // BANDA's stop_run condition (Rad_gas.f90:368-371)

    void init(int nwl, const double* wl) {   // RAD0's ALLOCATE + zero (Rad0.f90:22-28)
        NWL = nwl; WL = wl;
        AKLG.assign(NWL + 1, 0.0); AKLS.assign(NWL + 1, 0.0); AKL0.assign(NWL + 1, 0.0); E0.assign(NWL + 1, 0.0);
    }
    double wl(int n) const { return WL[n - 1]; }

    // CHIWHI (Rad_gas.f90:308-348): WHI divides by SQRT(TT0), the value of
    // the current cell, also when TT is T0_R
    void CHIWHI(double TT, const double V[4], const int NG[4], const int ND_R[4], double& CHI, double& WHI) {
        if (ND_R[1] != 0 || ND_R[2] != 0 || ND_R[3] != 0) {
            double U[4], UD = ZERO, XD = ZERO, XY = ZERO, YN = ZERO;
            int NV[4];
            for (int K = 1; K <= 3; ++K) {
                U[K] = HCK_R * V[K] / TT;
                NV[K] = 0;
                if (ND_R[K] < 0) NV[K] = std::abs(ND_R[K]);
                const int NDK = std::abs(ND_R[K]);
                double Y1 = ZERO;
                for (;;) {
                    const double XGAS = std::exp(-U[K] * NV[K]) / PER(NG[K] - 1, NG[K] - 1);
                    const double X1 = XGAS * PER(NV[K] + NG[K] + NDK - 1, NG[K] + NDK - 1);
                    const double X2 = XGAS * PER(NV[K] + NG[K] - 1, NG[K] - 1);
                    if (X1 < 1.0e-10) break;
                    XY = XY + X1;
                    XD = XD + X2;
                    Y1 = Y1 + std::sqrt(X1);
                    NV[K] = NV[K] + 1;
                    if (NV[K] >= 100) break;
                }
                YN = YN + Y1 * Y1;
                UD = UD - U[K] * ND_R[K];
            }
            CHI = (ONE - std::exp(UD)) * XY / XD;
            WHI = YN / XY / std::sqrt(TT0);
        } else {
            CHI = ONE;
            WHI = ONE / std::sqrt(TT0);
        }
    }
    double BANDA(double ALP, double BTA, double A0) {   // Rad_gas.f90:360-395
        if (A0 <= 0) return 0;
        if (ALP < ZERO || BTA < ZERO || A0 < ZERO || W_R * PE < 0) { error = 1; return 0; }
        if (W_R * PE == 0) return 0;
        const double ETA = BTA * PE;
        const double TAU = ALP * W_R / A0;
        double A_S;
        if (ETA >= ONE) {
            A_S = TAU <= 1.0 ? TAU : 1.0 + std::log(TAU);
        } else if (TAU <= ETA) {
            A_S = TAU;
        } else if (TAU <= 1 / ETA) {
            A_S = 2.0 * std::sqrt(ETA * TAU) - ETA;
        } else {
            A_S = std::log(ETA * TAU) + 2.0 - ETA;
        }
        return A0 * A_S;
    }
    double A1(const double V[4], const int NG[4], const double B[4], const int ND_R[4]) {   // Rad_gas.f90:284-296
        double CHI0, WHI0, CHI, WHI;
        CHIWHI(T0_R, V, NG, ND_R, CHI0, WHI0);
        CHIWHI(T_RAD, V, NG, ND_R, CHI, WHI);
        const double C3 = B[3] * std::sqrt(T_RAD / T0_R);
        const double C1 = B[1] * CHI / CHI0;
        const double C2 = 2.0 * std::sqrt(C1 * C3 * B[2] * WHI / WHI0);
        return BANDA(C1, C2, C3);
    }
    void AH2O() {   // Rad_gas.f90:149-212
        const int NG[4] = {0, 1, 1, 1};
        const double V[4] = {0, 3.652e+5, 1.595e+5, 3.756e+5};
        double AA[6] = {0}, B[4] = {0};
        int ND_R[4] = {0, 0, 0, 0};
        for (int n = 1; n <= 5; ++n) AAH2O[n] = 0;
        if (YH2O <= ZERO || T_RAD <= 3.0e+2) return;
        PE = P_RAD + P_RAD * YH2O * (0.86e+1 / TT0 - 0.5);
        W_R = P_RAD * YH2O * OPL / T_RAD / 8.208e-2 * WH2O;
        B[1] = 0.52e+4 * std::exp(-0.176e+2 / TT0); B[2] = 0.14311; B[3] = 0.284e+2;
        ND_R[1] = ND_R[2] = ND_R[3] = 0;
        AA[1] = A1(V, NG, B, ND_R);
        B[1] = 0.412e+2; B[2] = 0.9427e-1; B[3] = 0.564e+2;
        ND_R[2] = 1;
        AA[2] = A1(V, NG, B, ND_R);
        B[1] = 0.19; B[2] = 0.13219; B[3] = 0.6e+2;
        ND_R[2] = 2;
        double CHI0, WHI0, CHI, WHI;
        CHIWHI(T0_R, V, NG, ND_R, CHI0, WHI0);
        CHIWHI(T_RAD, V, NG, ND_R, CHI, WHI);
        const double T1 = B[1] * CHI / CHI0, T4 = B[2] * WHI / WHI0;
        B[1] = 0.23e+1; ND_R[1] = 1; ND_R[2] = 0;
        CHIWHI(T0_R, V, NG, ND_R, CHI0, WHI0);
        CHIWHI(T_RAD, V, NG, ND_R, CHI, WHI);
        const double T2 = B[1] * CHI / CHI0, T5 = B[2] * WHI / WHI0;
        B[1] = 0.224e+2; ND_R[1] = 0; ND_R[3] = 1;
        CHIWHI(T0_R, V, NG, ND_R, CHI0, WHI0);
        CHIWHI(T_RAD, V, NG, ND_R, CHI, WHI);
        const double T3 = B[1] * CHI / CHI0, T6 = B[2] * WHI / WHI0;
        const double C1 = T1 + T2 + T3;
        const double C3 = B[3] * TT0;
        const double BTA = 2.0 * std::sqrt(C3) * (std::sqrt(T1 * T4) + std::sqrt(T2 * T5) + std::sqrt(T3 * T6));
        AA[3] = BANDA(C1, BTA, C3);
        B[1] = 3.0; B[2] = 0.8169e-1; B[3] = 0.431e2;
        ND_R[2] = 1;
        AA[4] = A1(V, NG, B, ND_R);
        B[1] = 0.25e+1; B[2] = 0.11628; B[3] = 0.32e+2;
        ND_R[1] = 1; ND_R[2] = 0;
        AA[5] = A1(V, NG, B, ND_R);
        for (int n = 1; n <= 5; ++n) AAH2O[n] = AA[n] * 1.0e+2;
    }
    void ACO2() {   // Rad_gas.f90:224-274
        const int NG[4] = {0, 1, 2, 1};
        const double V[4] = {0, 1.351e+5, 6.67e+4, 2.396e+5};
        double AA[7] = {0}, B[4] = {0};
        int ND_R[4] = {0, 0, 0, 0};
        W_R = P_RAD * YCO2 * OPL / T_RAD / 8.208e-2 * WCO2;
        if (W_R <= ZERO) return;
        PE = std::pow(P_RAD + P_RAD * YCO2 * 0.3, 0.7);
        B[1] = 0.19e+2; B[2] = 0.6157e-1; B[3] = 0.127e2;
        ND_R[1] = 0; ND_R[2] = 1; ND_R[3] = 0;
        AA[1] = A1(V, NG, B, ND_R);
        PE = std::pow(P_RAD + P_RAD * YCO2 * 0.3, 0.8);
        B[1] = 0.36; B[2] = 0.4017e-1; B[3] = 0.134e+2;
        ND_R[1] = -1; ND_R[2] = 0; ND_R[3] = 1;
        AA[2] = A1(V, NG, B, ND_R);
        B[1] = 0.24; B[2] = 0.11888; B[3] = 0.101e+2;
        AA[3] = A1(V, NG, B, ND_R);
        B[1] = 0.11e+3; B[2] = 0.24723; B[3] = 0.112e+2;
        ND_R[1] = 0;
        AA[4] = A1(V, NG, B, ND_R);
        PE = std::pow(P_RAD + P_RAD * YCO2 * 0.3, 0.65);
        B[1] = 4.0; B[2] = 0.13341; B[3] = 23.5;
        ND_R[1] = 1;
        AA[5] = A1(V, NG, B, ND_R);
        B[1] = 0.66e-1; B[2] = 0.39305; B[3] = 0.345e+2;
        ND_R[1] = 2;
        AA[6] = A1(V, NG, B, ND_R);
        for (int n = 1; n <= 6; ++n) AACO2[n] = AA[n] * 1.0e+2;
    }
    static void SOC(double WL0, double& XN_K, double& X2NK) {   // Rad_soot.f90:49-69
        const double SOCF[3] = {7.2e+26, 4.07e+27, 4.47e+28};
        const double SOCH[3] = {1.2e+15, 5.90e+15, 5.60e+15};
        const double SOCW[3] = {0.0, 1.25e+15, 7.25e+15};
        const double C_0 = 2.9984e+8, E2ME0 = 3.185e+3;
        XN_K = ONE;
        X2NK = ZERO;
        const double W = TWO * PI_R * C_0 / WL0;
        for (int J = 0; J < 3; ++J) {
            const double A = SOCW[J] * SOCW[J] - W * W;
            const double B = A * A + W * W * SOCH[J] * SOCH[J];
            if (B < 1.0e-20) return;
            const double G0 = SOCF[J] * E2ME0;
            XN_K = XN_K + G0 * A / B;
            X2NK = X2NK + G0 * SOCH[J] * W / B;
        }
    }
    void SOOTA() {   // Rad_soot.f90:26-37
        if (FVS < 1.0e-14) return;
        for (int N = 1; N <= NWL; ++N) {
            const double WL0 = wl(N);
            double XN_K, X2NK;
            SOC(WL0, XN_K, X2NK);
            const double G0 = 18.0 * PI_R * X2NK / ((XN_K + TWO) * (XN_K + TWO) + X2NK * X2NK);
            AKLS[N] = G0 * FVS / WL0;
        }
    }
    void RAD_GAS() {   // Rad_gas.f90:16-137
        const double EPS1 = 1.0e-4;
        for (int n = 0; n < 6; ++n) for (int m = 0; m < 4; ++m) WNH2O[n][m] = 0;
        for (int n = 0; n < 7; ++n) for (int m = 0; m < 4; ++m) WNCO2[n][m] = 0;
        for (int n = 0; n < 12; ++n) for (int m = 0; m < 3; ++m) WNG[n][m] = 0;
        for (int n = 1; n <= NWL; ++n) AKLG[n] = ZERO;
        if (YH2O > EPS1) {
            WNH2O[1][1] = 0;
            WNH2O[2][2] = 1.60e+5; WNH2O[3][2] = 3.76e+5; WNH2O[4][2] = 5.35e+5; WNH2O[5][2] = 7.25e+5;
            AH2O();
            WNH2O[1][2] = AAH2O[1] / 2;
            WNH2O[1][3] = AAH2O[1];
            for (int N = 2; N <= 5; ++N) {
                const double G0 = AAH2O[N] / 2;
                WNH2O[N][1] = WNH2O[N][2] - G0;
                WNH2O[N][3] = WNH2O[N][2] + G0;
                if (WNH2O[N - 1][3] > WNH2O[N][1]) WNH2O[N - 1][3] = WNH2O[N][1];
            }
        }
        if (YCO2 > EPS1) {
            WNCO2[1][2] = 6.67e+4; WNCO2[2][2] = 9.60e+4; WNCO2[3][2] = 1.06e+5;
            WNCO2[4][3] = 2.41e+5; WNCO2[5][2] = 3.66e+5; WNCO2[6][2] = 5.20e+5;
            ACO2();
            for (int N = 1; N <= 6; ++N) {
                const double G0 = AACO2[N] / 2;
                if (N == 1 && G0 > WNCO2[1][2]) {
                    WNCO2[1][1] = 0;
                    WNCO2[1][3] = AACO2[1];
                } else if (N == 4) {
                    WNCO2[N][2] = WNCO2[N][3] - G0;
                    WNCO2[N][1] = WNCO2[N][2] - G0;
                } else {
                    WNCO2[N][1] = WNCO2[N][2] - G0;
                    WNCO2[N][3] = WNCO2[N][2] + G0;
                }
                if (N <= 1) continue;
                if (WNCO2[N - 1][3] > WNCO2[N][1]) WNCO2[N - 1][3] = WNCO2[N][1];
            }
        }
        SOOTA();
        for (int n = 1; n <= 5; ++n) { WNG[n][1] = WNH2O[n][1]; WNG[n][2] = WNH2O[n][3]; }
        for (int n = 1; n <= 6; ++n) { WNG[n + 5][1] = WNCO2[n][1]; WNG[n + 5][2] = WNCO2[n][3]; }
        for (int N = 1; N <= 10; ++N) {
            for (int N2 = N + 1; N2 <= 11; ++N2) {
                if (WNG[N][1] < WNG[N2][1]) continue;
                std::swap(WNG[N][1], WNG[N2][1]);
                std::swap(WNG[N][2], WNG[N2][2]);
            }
            if (N <= 1) continue;
            if (WNG[N - 1][2] > WNG[N][1]) WNG[N - 1][2] = WNG[N][1];
        }
        double WL2 = 10 / wl(1);
        for (int n = 1; n <= NWL; ++n) E0[n] = ZERO;
        int N0 = 11;
        for (int N = 1; N <= NWL; ++N) {
            const double WL1 = N == NWL ? 0 : 1 / wl(N);
            if (WL2 <= WL1 || WNG[11][2] <= WL1) { WL2 = WL1; continue; }
            for (int N1 = N0; N1 >= 1; --N1) {
                if (WNG[N1][2] <= WL1) { N0 = N1; break; }
                if (WNG[N1][2] >= WL1 && WNG[N1][2] <= WL2) {
                    if (WNG[N1][1] < WL1) {
                        E0[N] = E0[N] + WNG[N1][2] - WL1;
                        WNG[N1][2] = WL1;
                        N0 = N1;
                        break;
                    }
                    E0[N] = E0[N] + WNG[N1][2] - WNG[N1][1];
                }
            }
            if (E0[N] <= 0 || WL2 <= WL1) {
                AKLG[N] = ZERO;
            } else {
                E0[N] = E0[N] / (WL2 - WL1);
                double G0 = 1 - E0[N];
                if (G0 <= 1.0e-20) G0 = 1.0e-20;
                AKLG[N] = -std::log(G0) / OPL;
            }
            WL2 = WL1;
        }
        for (int n = 1; n <= NWL; ++n) AKL0[n] = AKLG[n] + AKLS[n];
    }
};

double ZY1(const double* X, const double* Y, double X1, int N) {   // Source.f90:814-831
    if (X1 < X[0]) return Y[0] * X1 / X[0];
    for (int I = 2; I <= N; ++I)
        if (X1 < X[I - 1]) {
            double RATIO = (X1 - X[I - 2]) / (X[I - 1] - X[I - 2]);
            return Y[I - 2] + (Y[I - 1] - Y[I - 2]) * RATIO;
        }
    return Y[N - 1];
}

// ---------------------------------------------------------------------------
// The oracle state: module GBL_VAR
// ---------------------------------------------------------------------------
struct Oracle {
    int MP, NP, LP, MPM1, MPM2, NPM1, NPM2, LPM1, LPM2, MZ, NZ, LZ;
    long N;
    int NJY1, NJY2, LKZ1, LKZ2, NJY1V[4], NJY2V[4], LKZ1V[4], LKZ2V[4];
    int NCELLS, I_REF, J_REF, K_REF;
    double P_REF;
    vec X, DX, R, DR, RS, Z, DZ;   // 1-based (index 0 unused)
    std::vector<int16_t> IBC;
    double BV_F[3], BA_F[4][3];    // COMMON /GRD1/ (Grid3.f90:12), 1-based: BV_F(IBC), BA_F(IX,IBC)
    vec P, T, DNST, THETA, TMU, GAMA, CRATE, HRATE, GTE, FZ, BS, SFP, AP, bs_hprev, UG, GF, AS, QA, QE;
    gfm_params pr;
    double RFC[21], RFLC[21];
    // wall patches, kinetics, bands
    std::vector<int> b_typ, b_i, b_j, b_k, b_orient, b_direct;
    vec b_T, q_conv;
    // wall radiation exchange (Qwall.f90), set up by gfo_wall_setup
    bool wall_on = false;
    int i1st_rad_done = 0;
    gfm_wall_spec ws{};
    std::vector<int> bc_i, bc_j, bc_k, b_exh;
    vec emis, patch_area, b_face_area, vf, radiosity, q_amb, qc, qeb, qrs;
    double avg_wall_T = 1600.0, radi_min = 0, rad_from_bnds = 0;
    double wall_area_total = 0, melt_area_total = 0, inlet_area_total = 0, exit_area_total = 0, boundary_area_total = 0;
    double q_melt = 0, q_wall_loss = 0, q_incident_total = 0, q_incident_wall = 0, q_incident_inlet = 0;
    double q_incident_exit = 0, q_incident_melt = 0, q_rad_inlet = 0, q_rad_outlet = 0, qm_flame = 0, qm_bnds = 0, qm_conv = 0;
    double last_rel_rad_chg_mean = 0;
    int iterw = 0, wall_outer = 0, have_frac_exh_T = 0;
    int NR0;
    vec RTIM, DELRT, HRT, DELR, TIMED, HRD;
    int NWL;
    vec WL, AKL0;
    // minor species and soot (ms=1, Setup.f90:904-929): GFM(MP,NP,LP,7), smf,
    // the soot sources of the last MSFLOW iteration, RRMS(MZ,NZ,LZ,5)
    vec GFMS, SMF, BS_SOOT_PREV, SFP_SOOT_PREV, RRMS, AP1;
    int itr_ms = 0, imscon = 0, IGS0 = 0, minor_on = 0, minor_from_host = 0;
    double resid_ms[9] = {0}, resid_ms_pre[9] = {0};
    // state scalars
    int itr_gas, do_rad_qe_only_cnt, i1st_rad_qe_done, NELG;
    double FACTOR, FADJ, GFIN0, GFIN, GFEX, SGM, q_h_in;
    double res_mass, res_mass_max, p_resid_pre, p_resid, pcorr_resid, u_resid_pre[3], u_resid[3];
    double gf_resid_pre[10], gf_resid[10], h_resid_pre;
    double q_react, q_exhaust, qconv_total, q_rad_vol_tot, Tmean_ex, Tave;

    long ix(int i, int j, int k) const {
#ifdef GFO_CHECK
        if (i < 1 || i > MP || j < 1 || j > NP || k < 1 || k > LP) {
            std::fprintf(stderr, "gfm_oracle: index (%d,%d,%d) outside (%d,%d,%d)\n", i, j, k, MP, NP, LP);
            std::abort();
        }
#endif
        return (long)(i - 1) + (long)MP * ((long)(j - 1) + (long)NP * (long)(k - 1));
    }
    int ibcell(int i, int j, int k) const { return IBC[ix(i, j, k)]; }
    double& a3(vec& v, int i, int j, int k) { return v[ix(i, j, k)]; }
    double& ug(int i, int j, int k, int l) { return UG[ix(i, j, k) + (long)(l - 1) * N]; }
    double& gf(int i, int j, int k, int l) { return GF[ix(i, j, k) + (long)(l - 1) * N]; }
    double& as(int i, int j, int k, int l, int m) { return AS[ix(i, j, k) + (long)((l - 1) * 2 + (m - 1)) * N]; }
    Y9 y9(int i, int j, int k) { return Y9{&GF[ix(i, j, k)], N}; }
    long cix(int id2, int jd2, int kd2) const { return (long)(id2 - 1) + (long)MZ * ((long)(jd2 - 1) + (long)NZ * (long)(kd2 - 1)); }
    double& gfm(int i, int j, int k, int l) { return GFMS[ix(i, j, k) + (long)(l - 1) * N]; }
    double& rrms(int id2, int jd2, int kd2, int l) { return RRMS[cix(id2, jd2, kd2) + (long)(l - 1) * MZ * NZ * LZ]; }
    // RAD0's inputs of RAD_GAS for one open cell, T_RAD in kelvin
    // (Rad0.f90:118-123 with wmix_ms_calc, Prop.f90:207-218)
    void rad_gas_inputs(RadGas& g, int I, int J, int K, double T_RAD) {
        g.T_RAD = T_RAD;
        g.TT0 = std::sqrt(T_RAD / T0_R);
        g.P_RAD = (ONE + a3(P, I, J, K)) * pr.pg0 / P0_R;
        double sum = ZERO;
        for (int n = 1; n <= 7; ++n) sum = sum + gfm(I, J, K, n) / WMS[n - 1];
        const double wmix_ms = ONE / sum;
        g.YCO2 = gfm(I, J, K, 5) * wmix_ms / WCO2;
        g.YH2O = gfm(I, J, K, 4) * wmix_ms / WH2O;
        g.FVS = a3(SMF, I, J, K) * a3(DNST, I, J, K) * pr.dnst0 / DNST_SOOT;
    }

    // ---- Grid3.f90 metric functions -----------------------------------------
    double DXAV(int I, int J, int K) {
        if (ibcell(I - 2, J, K) >= 1) return X[I + 1] - X[I - 2];
        if (ibcell(I + 2, J, K) >= 1) return X[I + 2] - X[I - 1];
        return DX[I];
    }
    double DRAV(int I, int J, int K) {
        if (ibcell(I, J - 2, K) >= 1) { double DRC = R[J + 1] - R[J - 2]; return (RS[J + 1] + RS[J - 2]) * 0.5 / RS[J] * DRC; }
        if (ibcell(I, J + 2, K) >= 1) { double DRC = R[J + 2] - R[J - 1]; return (RS[J + 2] + RS[J - 1]) * 0.5 / RS[J] * DRC; }
        return DR[J];
    }
    double DZAV(int I, int J, int K) {
        if (ibcell(I, J, K - 2) >= 1) return Z[K + 1] - Z[K - 2];
        if (ibcell(I, J, K + 2) >= 1) return Z[K + 2] - Z[K - 1];
        return DZ[K];
    }
    // VOL_C0 (Grid3.f90:395-405)
    double VOL_C0(int I, int J, int K) {
        double VOL = DX[I] * DR[J] * RS[J] * DZ[K];
        if (ibcell(I, J, K) <= -1) {
            int IBCX = -ibcell(I, J, K);
            VOL = VOL * BV_F[IBCX];
        }
        return VOL;
    }
    double VOL_C(int I, int J, int K) {
        double VOL;
        if ((I / 2) * 2 != I) {
            double VM = VOL_C0(I - 1, J, K); if (ibcell(I - 2, J, K) <= 0) VM = VM * 0.5;
            double VP = VOL_C0(I + 1, J, K); if (ibcell(I + 2, J, K) <= 0) VP = VP * 0.5;
            VOL = VP + VM;
        } else if ((J / 2) * 2 != J) {
            double VM = VOL_C0(I, J - 1, K); if (ibcell(I, J - 2, K) <= 0) VM = VM * 0.5;
            double VP = VOL_C0(I, J + 1, K); if (ibcell(I, J + 2, K) <= 0) VP = VP * 0.5;
            VOL = VP + VM;
        } else if ((K / 2) * 2 != K) {
            double VM = VOL_C0(I, J, K - 1); if (ibcell(I, J, K - 2) <= 0) VM = VM * 0.5;
            double VP = VOL_C0(I, J, K + 1); if (ibcell(I, J, K + 2) <= 0) VP = VP * 0.5;
            VOL = VP + VM;
        } else {
            VOL = VOL_C0(I, J, K);
        }
        return VOL;
    }
    // AREA_C (Grid3.f90:411-471)
    double AREA_C(int I, int J, int K, int IXD) {
        if (ibcell(I, J, K) == 1) return ZERO;
        double AREA;
        if (IXD == 1) AREA = DR[J] * RS[J] * DZ[K];
        else if (IXD == 2) AREA = DX[I] * DZ[K];
        else AREA = DX[I] * DR[J] * RS[J];
        if (ibcell(I, J, K) == 0) return AREA;
        if (ibcell(I, J, K) <= -1) return AREA * BA_F[IXD][-ibcell(I, J, K)];
        int IBCX;
        if (IXD == 1) {
            if (I <= MPM2 && ibcell(I + 2, J, K) <= -1) IBCX = -ibcell(I + 2, J, K);
            else if (I >= 4 && ibcell(I - 2, J, K) <= -1) IBCX = -ibcell(I - 2, J, K);
            else return AREA;
        } else if (IXD == 2) {
            if (J <= NPM2 && ibcell(I, J + 2, K) <= -1) IBCX = -ibcell(I, J + 2, K);
            else if (J >= 4 && ibcell(I, J - 2, K) <= -1) IBCX = -ibcell(I, J - 2, K);
            else return AREA;
        } else {
            if (K <= LPM2 && ibcell(I, J, K + 2) <= -1) IBCX = -ibcell(I, J, K + 2);
            else if (K >= 4 && ibcell(I, J, K - 2) <= -1) IBCX = -ibcell(I, J, K - 2);
            else return AREA;
        }
        return AREA * BA_F[IXD][IBCX];
    }

    // ---- Prop.f90 per-position wrappers --------------------------------------
    void CONC(int i, int j, int k) { conc(y9(i, j, k)); }
    void dnst_calc(int i, int j, int k) {
        conc(y9(i, j, k));
        double wt = wmix(y9(i, j, k));
        double temp = (ONE + a3(P, i, j, k)) / a3(T, i, j, k) * wt / pr.wt0;
        a3(DNST, i, j, k) = fmax2(temp, small20);
    }
    void THER(int i, int j, int k) {
        gf(i, j, k, IEPS) = fmax2(gf(i, j, k, IEPS), 1.0e-12);
        double G0 = pr.cmu * pr.reyg * pr.epsr / (TWO * pr.taur) * (gf(i, j, k, IK) * gf(i, j, k, IK)) /
                    gf(i, j, k, IEPS) * a3(DNST, i, j, k);
        a3(TMU, i, j, k) = G0;
        a3(GAMA, i, j, k) = TWO / pr.reyg * (a3(TMU, i, j, k) + std::pow(a3(T, i, j, k) / pr.trdg, pr.amu));
    }
    void enth_to_T_at(int i, int j, int k) { a3(T, i, j, k) = enth_to_T(y9(i, j, k), a3(T, i, j, k)); }
    void T_to_enth_at(int i, int j, int k) { gf(i, j, k, IH) = T_to_enth(y9(i, j, k), a3(T, i, j, k)); }
    void BOUND(double& F, int IL, int IPP) {   // Prop.f90:243-296
        if (IPP == 1) {
            if (IL == 0) { F = fmin2(F, pr.p_mx); F = fmax2(F, pr.p_mn); }
            else if (IL == 4) { F = fmin2(F, pr.t_mx); F = fmax2(F, pr.t_mn); }
            else if (IL == 5) { F = fmax2(F, 1.0e-6); }
            else { F = fmin2(F, pr.u_mx); F = fmax2(F, pr.u_mn); if (std::fabs(F) < 1.0e-12) F = ZERO; }
        } else if (IPP == 2) {
            if (IL == IK) F = fmax2(F, 1.0e-6);
            else if (IL == IEPS) F = fmax2(F, 1.0e-12);
            else if (IL == IH) return;
            else if (IL == 20) F = fmax2(F, 1.0e-1);
            else if (IL == 8) F = fmax2(F, 1.0e-14);
            else { F = fmin2(F, ONE); F = fmax2(F, ZERO); }
        }
    }

    // ---- Gslv3x.f90 -----------------------------------------------------------
    void ECELL(int I, int J, int K, int IU, double FFL[4][3]) {
        if (IU == 1) {
            int I1 = I - 1, I2 = I - 2;
            for (int M = 1; M <= 2; ++M) {
                if (ibcell(I2, J, K) >= 1) FFL[1][M] = DX[I1]; else FFL[1][M] = std::fabs(X[I] - X[I1]);
                FFL[2][M] = FFL[1][M] * DZ[K];
                FFL[3][M] = FFL[1][M] * RS[J] * DR[J];
                I1 = I + 1; I2 = I + 2;
            }
        } else if (IU == 2) {
            int J1 = J - 1, J2 = J - 2;
            for (int M = 1; M <= 2; ++M) {
                if (ibcell(I, J2, K) >= 1) FFL[2][M] = RS[J1] * DR[J1]; else FFL[2][M] = RS[J1] * std::fabs(R[J] - R[J1]);
                FFL[1][M] = FFL[2][M] * DZ[K];
                FFL[3][M] = FFL[2][M] * DX[I];
                J1 = J + 1; J2 = J + 2;
            }
        } else {
            int K1 = K - 1, K2 = K - 2;
            for (int M = 1; M <= 2; ++M) {
                if (ibcell(I, J, K2) >= 1) FFL[3][M] = DZ[K1]; else FFL[3][M] = std::fabs(Z[K] - Z[K1]);
                FFL[1][M] = FFL[3][M] * RS[J] * DR[J];
                FFL[2][M] = FFL[3][M] * DX[I];
                K1 = K + 1; K2 = K + 2;
            }
        }
    }
    double FDDL(int I, int J, int K, int IU) {
        double DDL;
        int b = ibcell(I, J, K);
        if (IU == 1) {
            if (b <= 0) DDL = DX[I];
            else if (ibcell(I + 1, J, K) == 0) DDL = X[I + 1] - X[I];
            else if (ibcell(I - 1, J, K) == 0) DDL = X[I] - X[I - 1];
            else DDL = BIG;
        } else if (IU == 2) {
            if (b <= 0) DDL = DR[J] * RS[J];
            else if (ibcell(I, J + 1, K) == 0) DDL = (R[J + 1] - R[J]) * RS[J];
            else if (ibcell(I, J - 1, K) == 0) DDL = (R[J] - R[J - 1]) * RS[J];
            else DDL = BIG;
        } else {
            if (b <= 0) DDL = DZ[K];
            else if (ibcell(I, J, K + 1) == 0) DDL = Z[K + 1] - Z[K];
            else if (ibcell(I, J, K - 1) == 0) DDL = Z[K] - Z[K - 1];
            else DDL = BIG;
        }
        return DDL;
    }
    double VOL1(int I, int J, int K, int IXD, double FFL[4][3]) {
        double AREA = AREA_C(I, J, K, IXD);
        double VOL = (FFL[IXD][1] + FFL[IXD][2]) * AREA;
        if (IXD == 1) {
            if (ibcell(I - 1, J, K) <= -1) VOL = VOL - DX[I - 1] * AREA / TWO;
            if (ibcell(I + 1, J, K) <= -1) VOL = VOL - DX[I + 1] * AREA / TWO;
        } else if (IXD == 2) {
            if (ibcell(I, J - 1, K) <= -1) VOL = VOL - RS[J - 1] * DR[J - 1] * AREA / TWO;
            if (ibcell(I, J + 1, K) <= -1) VOL = VOL - RS[J + 1] * DR[J + 1] * AREA / TWO;
        } else {
            if (ibcell(I, J, K - 1) <= -1) VOL = VOL - DZ[K - 1] * AREA / TWO;
            if (ibcell(I, J, K + 1) <= -1) VOL = VOL - DZ[K + 1] * AREA / TWO;
        }
        return VOL;
    }
    double FLW(int I, int J, int K, int IXD, int M) {
        double AREA = AREA_C(I, J, K, IXD);
        double F = a3(THETA, I, J, K) * a3(DNST, I, J, K) * ug(I, J, K, IXD) * AREA;
        return M == 1 ? fmax2(ZERO, F) : fmax2(ZERO, -F);
    }
    double FLWD(int I, int J, int K, int IXD, int M) {
        double AREA = AREA_C(I, J, K, IXD);
        double DDL = IXD == 1 ? DX[I] : (IXD == 2 ? DR[J] : DZ[K]);
        double F = a3(THETA, I, J, K) * a3(DNST, I, J, K) * ug(I, J, K, IXD) * AREA;
        double DIFF = a3(THETA, I, J, K) * a3(GAMA, I, J, K) / SGM * AREA / DDL;
        return M == 1 ? DA(DIFF, F) + fmax2(ZERO, F) : DA(DIFF, F) + fmax2(ZERO, -F);
    }
    static void VINDX(int IU, int M, int I, int J, int K, int& I1, int& J1, int& K1, int& I2, int& J2, int& K2) {
        int NX[4] = {0, 0, 0, 0};
        NX[IU] = M;
        I1 = I + NX[1]; I2 = I1 + NX[1];
        J1 = J + NX[2]; J2 = J1 + NX[2];
        K1 = K + NX[3]; K2 = K1 + NX[3];
    }
    void GSLV3X1(int I, int J, int K, int IU, double& G0) {
        G0 = ZERO;
        for (int M = -1; M <= 1; M += 2) {
            int M1 = (M + 3) / 2, I1, J1, K1, I2, J2, K2;
            VINDX(IU, M, I, J, K, I1, J1, K1, I2, J2, K2);
            int IBC1 = ibcell(I2, J2, K2);
            if (IBC1 == 3) as(I, J, K, IU, M1) = ZERO;
            else if (IBC1 == 2) as(I, J, K, IU, M1) = FLW(I2, J2, K2, IU, M1);
            else as(I, J, K, IU, M1) = FLWD(I1, J1, K1, IU, M1);
            a3(AP, I, J, K) = a3(AP, I, J, K) + as(I, J, K, IU, M1);
            G0 = G0 + as(I, J, K, IU, M1) * a3(FZ, I2, J2, K2);
        }
    }
    void GSLVX1(int IU1) {
        int NX[4] = {0, 0, 0, 0};
        NX[IU1] = 1;
        int MI1 = 4 + NX[1], MI3 = MPM2 - NX[1], NJ1 = NJY1V[IU1], NJ3 = NJY2V[IU1], LK1 = LKZ1V[IU1], LK3 = LKZ2V[IU1];
        SOURCE(MI1, MI3, NJ1, NJ3, LK1, LK3);
        double FFL[4][3];
        for (int I = MI1; I <= MI3; I += 2)
            for (int J = NJ1; J <= NJ3; J += 2)
                for (int K = LK1; K <= LK3; K += 2) {
                    if (ibcell(I, J, K) >= 1) continue;
                    a3(AP, I, J, K) = ZERO;
                    double G0 = ZERO;
                    GSLV3X1(I, J, K, IU1, G0);
                    ECELL(I, J, K, IU1, FFL);
                    for (int IU = 1; IU <= 3; ++IU) {
                        if (IU == IU1) continue;
                        for (int M = -1; M <= 1; M += 2) {
                            int M1 = (M + 3) / 2, I1, J1, K1, I2, J2, K2;
                            VINDX(IU, M, I, J, K, I1, J1, K1, I2, J2, K2);
                            if (ibcell(I1, J1, K1) == 3) { as(I, J, K, IU, M1) = ZERO; continue; }
                            double F = ZERO, DIFF = ZERO;
                            int II1 = 0, JJ1 = 0, KK1 = 0;
                            for (int Nn = -1; Nn <= 1; Nn += 2) {
                                int N1 = (Nn + 3) / 2;
                                II1 = I1 + NX[1] * Nn; JJ1 = J1 + NX[2] * Nn; KK1 = K1 + NX[3] * Nn;
                                int IBC1 = ibcell(II1, JJ1, KK1);
                                if (IBC1 == 3) continue;
                                double AREA = FFL[IU][N1];
                                F = F + a3(THETA, II1, JJ1, KK1) * a3(DNST, II1, JJ1, KK1) * a3(FZ, II1, JJ1, KK1) * AREA;
                                if (IBC1 == 2) continue;
                                double DDL = FDDL(II1, JJ1, KK1, IU);
                                DIFF = DIFF + a3(THETA, II1, JJ1, KK1) * a3(GAMA, II1, JJ1, KK1) / SGM * AREA / DDL;
                            }
                            double FLD = M1 == 1 ? DA(DIFF, F) + fmax2(ZERO, F) : DA(DIFF, F) + fmax2(ZERO, -F);
                            if (ibcell(II1, JJ1, KK1) == 2 && ibcell(I2, J2, K2) == 1) {
                                double BS0 = FLD * (ug(II1, J2, K2, IU1) - ug(I, J, K, IU1));
                                a3(BS, I, J, K) = a3(BS, I, J, K) + BS0;
                                as(I, J, K, IU, M1) = ZERO;
                                continue;
                            }
                            as(I, J, K, IU, M1) = FLD;
                            a3(AP, I, J, K) = a3(AP, I, J, K) + FLD;
                            G0 = G0 + FLD * a3(FZ, I2, J2, K2);
                        }
                    }
                    const double EVPM = ZERO, CONM = ZERO;
                    double VOL = VOL1(I, J, K, IU1, FFL);
                    a3(BS, I, J, K) = a3(BS, I, J, K) * VOL;
                    a3(AP, I, J, K) = a3(AP, I, J, K) + (EVPM - CONM - a3(SFP, I, J, K)) * VOL;
                    if (std::fabs(a3(AP, I, J, K)) > small20) ug(I, J, K, IU1) = (G0 + a3(BS, I, J, K)) / a3(AP, I, J, K);
                }
    }

    // ---- Source.f90 ------------------------------------------------------------
    void SRC1(int I, int J, int K, int IU1) {
        if (ibcell(I, J, K) >= 1) { a3(BS, I, J, K) = ZERO; a3(SFP, I, J, K) = ZERO; return; }
        double VIS[4][3], DXN[4], DX1[4], DX0[4];
        DXN[1] = DX[I]; DXN[2] = DR[J] * RS[J]; DXN[3] = DZ[K];
        for (int M = -1; M <= 1; M += 2) {
            int I1, J1, K1, I2, J2, K2;
            VINDX(IU1, M, I, J, K, I1, J1, K1, I2, J2, K2);
            if (IU1 == 1) { DX0[1] = DX[I]; DX1[1] = DX[I1]; }
            else if (IU1 == 2) { DX0[2] = DR[J] * RS[J]; DX1[2] = DR[J1] * RS[J1]; }
            else { DX0[3] = DZ[K]; DX1[3] = DZ[K1]; }
            double THGM;
            if (ibcell(I2, J2, K2) == 2) {
                THGM = a3(THETA, I2, J2, K2) * a3(GAMA, I2, J2, K2);
                if (IU1 == 1) DXN[1] = DXN[1] + std::fabs(X[I2] - X[I1]);
                if (IU1 == 2) DXN[2] = DXN[2] + std::fabs(R[J2] - R[J1]) * RS[J];
                if (IU1 == 3) DXN[3] = DXN[3] + std::fabs(Z[K2] - Z[K1]);
            } else {
                THGM = a3(THETA, I1, J1, K1) * a3(GAMA, I1, J1, K1);
            }
            if (M == -1) VIS[IU1][1] = THGM * (a3(FZ, I, J, K) - a3(FZ, I2, J2, K2)) / DX1[IU1];
            else VIS[IU1][2] = THGM * (a3(FZ, I2, J2, K2) - a3(FZ, I, J, K)) / DX1[IU1];
        }
        double VMS = (VIS[IU1][2] - VIS[IU1][1]) / DXN[IU1];
        for (int IU = 1; IU <= 3; ++IU) {
            if (IU == IU1) continue;
            int I1 = I, J1 = J, K1 = K;
            for (int M = -1; M <= 1; M += 2) {
                if (IU == 1) I1 = I + M; else if (IU == 2) J1 = J + M; else K1 = K + M;
                double DU0;
                if (IU1 == 1) DU0 = a3(FZ, I + 1, J1, K1) - a3(FZ, I - 1, J1, K1);
                else if (IU1 == 2) DU0 = a3(FZ, I1, J + 1, K1) - a3(FZ, I1, J - 1, K1);
                else DU0 = a3(FZ, I1, J1, K + 1) - a3(FZ, I1, J1, K - 1);
                int M1 = (M + 3) / 2;
                VIS[IU][M1] = a3(THETA, I1, J1, K1) * a3(GAMA, I1, J1, K1) * DU0 / DX0[IU1];
                if (IU == 2) VIS[IU][M1] = VIS[IU][M1] * RS[J1];
            }
            VMS = VMS + (VIS[IU][2] - VIS[IU][1]) / DXN[IU];
        }
        const double GDZ = ZERO, GDZU = ZERO, DUAV = ZERO;   // single phase: KEY=1, no droplets
        a3(BS, I, J, K) = VMS + GDZU + DUAV;
        a3(BS, I, J, K) = a3(BS, I, J, K) + a3(THETA, I, J, K) * a3(DNST, I, J, K) * pr.gra[IU1 - 1];
        a3(SFP, I, J, K) = -GDZ;
    }

    // Qwall.f90:1370-1475 with T in K: T*T0 in the gas solve (tscale = T0),
    // T itself inside RAD_EMIS, which has already multiplied T by T0
    void calc_q_conv_wall(double tscale = -1.0) {
        if (tscale < 0) tscale = pr.t0;
        const double pi = 3.141592653589793;
        const double kappa_cmu = 0.4 * std::pow(9.0e-2, 0.25), E_cmu = 9.0 * std::pow(9.0e-2, 0.25);
        const double c_htw = 0.4 * ((pi / 4) / std::sin(pi / 4)) * std::sqrt(26.0) * (0.7 - ONE) / std::pow(0.7, 0.25);
        qconv_total = ZERO;
        for (size_t n = 0; n < b_typ.size(); ++n) {
            if (b_typ[n] == 2 || b_typ[n] == 3) { q_conv[n] = ZERO; continue; }
            int inc = b_i[n], jnc = b_j[n], knc = b_k[n];
            double ds;
            if (b_orient[n] == 1) {
                if (b_direct[n] == 0) { inc = inc + 1; ds = X[b_i[n] + 1] - X[b_i[n]]; }
                else { inc = inc - 1; ds = X[b_i[n]] - X[b_i[n] - 1]; }
            } else if (b_orient[n] == 2) {
                if (b_direct[n] == 0) { jnc = jnc + 1; ds = R[b_j[n] + 1] - R[b_j[n]]; }
                else { jnc = jnc - 1; ds = R[b_j[n]] - R[b_j[n] - 1]; }
            } else {
                if (b_direct[n] == 0) { knc = knc + 1; ds = Z[b_k[n] + 1] - Z[b_k[n]]; }
                else { knc = knc - 1; ds = Z[b_k[n]] - Z[b_k[n] - 1]; }
            }
            double cpmix = CP0 * (CPF1 * gf(inc, jnc, knc, IYF) + CPCO21 * gf(inc, jnc, knc, IYCO2) +
                                  CPH2O1 * gf(inc, jnc, knc, IYH2O) + CPO21 * gf(inc, jnc, knc, IYO2) +
                                  CPN21 * gf(inc, jnc, knc, IYN2));
            double Tgas = a3(T, inc, jnc, knc) * tscale;
            double gmu_T = ((2.0e-15 * Tgas + -1.1e-11) * Tgas + 4.5e-8) * Tgas + 7.0e-6;
            double h_t;
            if (pr.tk0 * gf(inc, jnc, knc, IK) < 0.1) {
                h_t = ZERO;
            } else {
                double sqrt_tke = std::sqrt(pr.tk0 * gf(inc, jnc, knc, IK));
                double dtmp = (std::log(E_cmu * ds * pr.dnst0 * a3(DNST, inc, jnc, knc) * sqrt_tke / gmu_T) + (c_htw / sqrt_tke));
                if (dtmp < 0.01) h_t = ZERO;
                else h_t = fmin2(50.0, cpmix * kappa_cmu * pr.dnst0 * a3(DNST, inc, jnc, knc) * sqrt_tke / dtmp);
            }
            double delta_T = Tgas - b_T[n];
            q_conv[n] = fmax2(pr.h_g, h_t) * delta_T;
            double patch_area = b_orient[n] == 1 ? DR[b_j[n]] * DZ[b_k[n]]
                                : (b_orient[n] == 2 ? DX[b_i[n]] * DZ[b_k[n]] : DX[b_i[n]] * DR[b_j[n]]);
            qconv_total = qconv_total + (q_conv[n] * patch_area);
        }
    }

    // ---- wall radiation exchange (Qwall.f90) ---------------------------------
    // X**4 with an integer exponent: (X*X)*(X*X)
    static double pow4(double x) { const double x2 = x * x; return x2 * x2; }
    // prepare_for_wall_radiation_calculation steps 1-5 (Qwall.f90:72-513):
    // MAPB = IBCELL with each exit tunnel closed, then the boundary patches.
    // Each patch: type, i, j, k, orientation, direction.
    void wall_patch_list(std::vector<int>& out) const {
        std::vector<int> mapb(IBC.begin(), IBC.end());
        auto mb = [&](int i, int j, int k) -> int& { return mapb[ix(i, j, k)]; };
        auto mbs = [&](int i, int j, int k) -> int {   // outside the grid: closed
            if (i < 1 || i > MP || j < 1 || j > NP || k < 1 || k > LP) return 1;
            return mapb[ix(i, j, k)];
        };
        auto set = [&](int i0, int i1, int j0, int j1, int k0, int k1, int v) {
            for (int ii = i0; ii <= i1; ++ii)
                for (int jj = j0; jj <= j1; ++jj)
                    for (int kk = k0; kk <= k1; ++kk) mb(ii, jj, kk) = v;
        };
        // the end of a run of exit positions; a run reaching the grid's edge ends there
        auto endrun = [&](int start, int lim, auto at) {
            int e = start;
            for (int q = start + 2; q <= lim; q += 2) { if (at(q) != 3) return q - 2; e = q; }
            return e;
        };
        // back wall, I = 2
        for (int J = 2; J <= NP; J += 2)
            for (int K = 2; K <= LP; K += 2) {
                const int I = 2;
                if (mb(I, J, K) != 3) continue;
                int ks = K, ke = endrun(K, LP, [&](int q) { return mb(I, J, q); });
                int js = J, je = endrun(J, NP, [&](int q) { return mb(I, q, K); });
                int inew = -1;
                for (int ii = 4; ii <= MP; ii += 2)
                    if (mbs(ii, js - 2, ks - 2) == 0 || mbs(ii, je + 2, ke + 2) == 0 || mbs(ii, js - 2, ke + 2) == 0 ||
                        mbs(ii, je + 2, ks - 2) == 0) { inew = ii - 2; break; }
                if (inew < 0) continue;
                set(inew, inew + 1, js, je, ks, ke, 3);
                set(2, inew - 1, js, je, ks, ke, 1);
            }
        // front wall, I = MP
        for (int J = 2; J <= NP; J += 2)
            for (int K = 2; K <= LP; K += 2) {
                const int I = MP;
                if (mb(I, J, K) != 3) continue;
                int ks = K, ke = endrun(K, LP, [&](int q) { return mb(I, J, q); });
                int js = J, je = endrun(J, NP, [&](int q) { return mb(I, q, K); });
                int inew = -1;
                for (int ii = MP - 2; ii >= 2; ii -= 2)
                    if (mbs(ii, js - 2, ks - 2) == 0 || mbs(ii, je + 2, ke + 2) == 0 || mbs(ii, js - 2, ke + 2) == 0 ||
                        mbs(ii, je + 2, ks - 2) == 0) { inew = ii + 2; break; }
                if (inew < 0) continue;
                set(inew - 1, inew, js, je, ks, ke, 3);
                set(inew + 1, MP, js, je, ks, ke, 1);
            }
        // side walls, J = 2 and J = NP
        for (int side = 0; side < 2; ++side)
            for (int I = 2; I <= MP; I += 2)
                for (int K = 2; K <= LP; K += 2) {
                    const int J = side == 0 ? 2 : NP;
                    if (mb(I, J, K) != 3) continue;
                    int ks = K, ke = endrun(K, LP, [&](int q) { return mb(I, J, q); });
                    int is = I, ie = endrun(I, MP, [&](int q) { return mb(q, J, K); });
                    int jnew = -1;
                    if (side == 0) {
                        for (int jj = 4; jj <= NP; jj += 2)
                            if (mbs(is - 2, jj, ks - 2) == 0 || mbs(ie + 2, jj, ke + 2) == 0 || mbs(is - 2, jj, ke + 2) == 0 ||
                                mbs(ie + 2, jj, ks - 2) == 0) { jnew = jj - 2; break; }
                        if (jnew < 0) continue;
                        set(is, ie, jnew, jnew + 1, ks, ke, 3);
                        set(is, ie, 2, jnew - 1, ks, ke, 1);
                    } else {
                        for (int jj = NP - 2; jj >= 2; jj -= 2)
                            if (mbs(is - 2, jj, ks - 2) == 0 || mbs(ie + 2, jj, ke + 2) == 0 || mbs(is - 2, jj, ke + 2) == 0 ||
                                mbs(ie + 2, jj, ks - 2) == 0) { jnew = jj + 2; break; }
                        if (jnew < 0) continue;
                        set(is, ie, jnew - 1, jnew, ks, ke, 3);
                        set(is, ie, jnew + 1, NP, ks, ke, 1);
                    }
                }
        // top, K = LP
        for (int I = 2; I <= MP; I += 2)
            for (int J = 2; J <= NP; J += 2) {
                const int K = LP;
                if (mb(I, J, K) != 3) continue;
                int is = I, ie = endrun(I, MP, [&](int q) { return mb(q, J, K); });
                int js = J, je = endrun(J, NP, [&](int q) { return mb(I, q, K); });
                int knew = -1;
                for (int kk = LP - 2; kk >= 2; kk -= 2)
                    if (mbs(is - 2, js - 2, kk) == 0 || mbs(ie + 2, je + 2, kk) == 0 || mbs(is - 2, je + 2, kk) == 0 ||
                        mbs(ie + 2, js - 2, kk) == 0) { knew = kk + 2; break; }
                if (knew < 0) continue;
                set(is, ie, js, je, knew - 1, knew, 3);
                set(is, ie, js, je, knew + 1, LP, 1);
            }
        out.clear();
        auto add = [&](int t, int i, int j, int k, int o, int d) {
            const int v[6] = {t, i, j, k, o, d};
            out.insert(out.end(), v, v + 6);
        };
        for (int k = 2; k <= LP; k += 2)
            for (int j = 2; j <= NP; j += 2)
                for (int i = 3; i <= MP - 1; i += 2) {
                    if (mb(i, j, k) < 1) continue;
                    if (mb(i - 1, j, k) > 0 && mb(i + 1, j, k) > 0) continue;
                    add(mb(i, j, k), i, j, k, 1, mb(i + 1, j, k) == 0 ? 0 : 1);
                }
        for (int k = 2; k <= LP; k += 2)
            for (int j = 3; j <= NP - 1; j += 2)
                for (int i = 2; i <= MP; i += 2) {
                    if (mb(i, j, k) < 1) continue;
                    if (mb(i, j - 1, k) > 0 && mb(i, j + 1, k) > 0) continue;
                    add(mb(i, j, k), i, j, k, 2, mb(i, j + 1, k) == 0 ? 0 : 1);
                }
        for (int k = 3; k <= LP - 1; k += 2)
            for (int j = 2; j <= NP; j += 2)
                for (int i = 2; i <= MP; i += 2) {
                    if (mb(i, j, k) < 1) continue;
                    if (mb(i, j, k - 1) > 0 && mb(i, j, k + 1) > 0) continue;
                    add(mb(i, j, k), i, j, k, 3, mb(i, j, k + 1) == 0 ? 0 : 1);
                }
    }

    // prepare_for_wall_radiation_calculation steps 5-8 (Qwall.f90:395-760) on
    // the patch list: cell centres, emissivities, areas, exhaust numbers,
    // normalised view factors and the face area of each patch's cell
    void wall_setup(const gfm_wall_spec& spec) {
        ws = spec;
        const int nb = (int)b_typ.size();
        bc_i.assign(nb, 0); bc_j.assign(nb, 0); bc_k.assign(nb, 0); b_exh.assign(nb, 0);
        emis.assign(nb, 0.0); patch_area.assign(nb, 0.0); b_face_area.assign(nb, 0.0);
        for (int n = 0; n < nb; ++n) {
            const int i = b_i[n], j = b_j[n], k = b_k[n], t = b_typ[n];
            bc_i[n] = i; bc_j[n] = j; bc_k[n] = k;
            const int s = b_direct[n] == 0 ? -1 : 1;
            if (b_orient[n] == 1) { bc_i[n] = i + s; patch_area[n] = DR[j] * DZ[k]; }
            else if (b_orient[n] == 2) { bc_j[n] = j + s; patch_area[n] = DX[i] * DZ[k]; }
            else { bc_k[n] = k + s; patch_area[n] = DX[i] * DR[j]; }
            if (t == 1) {
                const int ktop = b_orient[n] == 3 ? LP - 1 : LP;
                emis[n] = (Z[k] >= ws.height_to_ceiling || (k == ktop && ws.have_crown == 0)) ? ws.eps_c : ws.eps_w;
            } else if (t == 4 && b_orient[n] == 3) {
                emis[n] = ws.eps_m;
            } else {
                emis[n] = ONE;
            }
        }
        // step 6: exhaust numbers (Qwall.f90:534-557)
        have_frac_exh_T = 0;
        for (int m = 0; m < ws.nex; ++m) if (ws.exh_type[m] == 0) have_frac_exh_T = 1;
        for (int n = 0; n < nb; ++n) {
            if (b_typ[n] != 3) continue;
            for (int m = 0; m < ws.nex; ++m) {
                if (b_orient[n] != ws.exh_orient[m] || b_direct[n] != ws.exh_direct[m]) continue;
                bool in;
                if (b_orient[n] == 1) in = bc_j[n] >= ws.exh_j1[m] && bc_j[n] <= ws.exh_j2[m] && bc_k[n] >= ws.exh_k1[m] && bc_k[n] <= ws.exh_k2[m];
                else if (b_orient[n] == 2) in = bc_i[n] >= ws.exh_i1[m] && bc_i[n] <= ws.exh_i2[m] && bc_k[n] >= ws.exh_k1[m] && bc_k[n] <= ws.exh_k2[m];
                else in = bc_i[n] >= ws.exh_i1[m] && bc_i[n] <= ws.exh_i2[m] && bc_j[n] >= ws.exh_j1[m] && bc_j[n] <= ws.exh_j2[m];
                if (in) { b_exh[n] = m + 1; break; }
            }
        }
        // step 7: view factors, normalised per row (Qwall.f90:562-666)
        const double pi = 3.141592653589793;
        vf.assign((size_t)nb * nb, 0.0);
        for (int n = 0; n < nb; ++n) {
            double vf_sum = ZERO;
            for (int m = 0; m < nb; ++m) {
                if (n == m) continue;
                const double dx = X[b_i[n]] - X[b_i[m]], dy = R[b_j[n]] - R[b_j[m]], dz = Z[b_k[n]] - Z[b_k[m]];
                const double dd = dx * dx + dy * dy + dz * dz;
                const double denominator = pi * (dd * dd);
                // the near patch's normal offset, and the far patch's
                auto off = [&](int o, int a, int b) {
                    return o == 1 ? X[b_i[a]] - X[b_i[b]] : o == 2 ? R[b_j[a]] - R[b_j[b]] : Z[b_k[a]] - Z[b_k[b]];
                };
                const int on = b_orient[n], om = b_orient[m];
                const int cn = on == 1 ? b_i[n] : on == 2 ? b_j[n] : b_k[n];
                const int cm = on == 1 ? b_i[m] : on == 2 ? b_j[m] : b_k[m];
                if (b_direct[n] == 0 && cm <= cn) continue;
                if (b_direct[n] == 1 && cm >= cn) continue;
                double v;
                if (om == on) {
                    const double d = off(on, m, n);
                    v = d * d * patch_area[m] / denominator;
                } else {
                    v = std::fabs(off(on, m, n) * off(om, m, n)) * patch_area[m] / denominator;
                }
                vf[(size_t)n * nb + m] = v;
                vf_sum = vf_sum + v;
            }
            for (int m = 0; m < nb; ++m) {
                if (vf_sum == ZERO) continue;
                vf[(size_t)n * nb + m] = vf[(size_t)n * nb + m] / vf_sum;
            }
        }
        // step 8: the face area of the patches on one cell (Qwall.f90:684-736),
        // with the reference's chain of same-cell links as written
        std::vector<int> s1(nb, 0), s2(nb, 0), s3(nb, 0), s4(nb, 0);   // 1-based patch numbers, 0 = none
        for (int n = 1; n <= nb; ++n)
            for (int m = n + 1; m <= nb; ++m) {
                if (!(bc_i[n - 1] == bc_i[m - 1] && bc_j[n - 1] == bc_j[m - 1] && bc_k[n - 1] == bc_k[m - 1])) continue;
                if (s1[n - 1] == 0) {
                    s1[n - 1] = m; s1[m - 1] = n;
                } else if (s2[n - 1] == 0) {
                    if (s1[n - 1] == m) continue;
                    s2[n - 1] = m; s1[m - 1] = n;
                    s2[m - 1] = s1[n - 1]; s2[s1[n - 1] - 1] = m;
                } else if (s3[n - 1] == 0) {
                    if (s1[n - 1] == m || s2[n - 1] == m) continue;
                    s3[n - 1] = m; s1[m - 1] = n;
                    s2[m - 1] = s1[n - 1]; s3[s2[n - 1] - 1] = m;
                    s3[m - 1] = s2[n - 1];
                } else if (s4[n - 1] == 0) {
                    if (s1[n - 1] == m || s2[n - 1] == m || s3[n - 1] == m) continue;
                    s4[n - 1] = m; s1[m - 1] = n;
                    s2[m - 1] = s1[n - 1]; s4[s2[n - 1] - 1] = m;
                    s3[m - 1] = s2[n - 1]; s4[s3[n - 1] - 1] = m;
                    s4[m - 1] = s3[n - 1];
                }
            }
        wall_area_total = melt_area_total = inlet_area_total = exit_area_total = ZERO;
        for (int n = 0; n < nb; ++n) {
            auto pa = [&](int q) { return patch_area[q - 1]; };
            if (s1[n] == 0) b_face_area[n] = patch_area[n];
            else if (s2[n] == 0) b_face_area[n] = patch_area[n] + pa(s1[n]);
            else if (s3[n] == 0) b_face_area[n] = patch_area[n] + pa(s1[n]) + pa(s2[n]);
            else if (s4[n] == 0) b_face_area[n] = patch_area[n] + pa(s1[n]) + pa(s2[n]) + pa(s3[n]);
            else b_face_area[n] = patch_area[n] + pa(s1[n]) + pa(s2[n]) + pa(s3[n]) + pa(s4[n]);
            if (b_typ[n] == 1) wall_area_total = wall_area_total + patch_area[n];
            else if (b_typ[n] == 4) melt_area_total = melt_area_total + patch_area[n];
            else if (b_typ[n] == 2) inlet_area_total = inlet_area_total + patch_area[n];
            else exit_area_total = exit_area_total + patch_area[n];
        }
        boundary_area_total = wall_area_total + melt_area_total + inlet_area_total + exit_area_total;
        radiosity.assign(nb, 0.0); q_amb.assign(nb, 0.0); qc.assign(nb, 0.0); qeb.assign(nb, 0.0);
        qrs.assign((size_t)MP * NP, 0.0);
        radi_min = pr.sig * pow4(ws.t_mnk);   // Setup.f90:214
        avg_wall_T = 1600.0;                            // Qwall.f90:68
        wall_on = true;
    }

    // RAD_EMIS's patch temperatures and first radiosities (Rad_emis.f90:186-273),
    // with T in K
    void wall_start() {
        const int nb = (int)b_typ.size();
        if (i1st_rad_done == 0) {
            for (int n = 0; n < nb; ++n) {
                if (b_typ[n] == 1 || b_typ[n] == 2) b_T[n] = a3(T, bc_i[n], bc_j[n], bc_k[n]);
                else if (b_typ[n] == 3) {
                    const int m = b_exh[n] - 1;
                    b_T[n] = ws.exh_type[m] == 0 ? ws.exh_frac[m] * avg_wall_T : ws.exh_fixed[m];
                } else b_T[n] = a3(T, b_i[n], b_j[n], b_k[n]);
                radiosity[n] = pr.sig * pow4(b_T[n]);
            }
        } else {
            for (int n = 0; n < nb; ++n)
                if (b_typ[n] == 4) {
                    b_T[n] = a3(T, b_i[n], b_j[n], b_k[n]);
                    radiosity[n] = pr.sig * pow4(b_T[n]);
                }
        }
    }

    // get_radiation_from_boundaries (Qwall.f90:1489-1577), the preset form
    void radiation_from_boundaries(int i) {
        const int nb = (int)b_typ.size();
        rad_from_bnds = ZERO;
        const double* row = &vf[(size_t)i * nb];
        for (int j = 0; j < nb; ++j) rad_from_bnds = rad_from_bnds + radiosity[j] * row[j];
    }

    // wall_q_amb (Qwall.f90:1585-1655): one wall material (IWALL all zero)
    void wall_q_amb() {
        q_wall_loss = ZERO;
        double u_a0;
        if (ws.w_k < 1.0e-20 || ws.h_a < 1.0e-20) u_a0 = ZERO;
        else u_a0 = ONE / (ws.w_d / ws.w_k + ONE / ws.h_a);
        for (size_t n = 0; n < b_typ.size(); ++n) {
            if (b_typ[n] != 1) { q_amb[n] = ZERO; continue; }
            q_amb[n] = u_a0 * (b_T[n] - ws.t_a);
            q_wall_loss = q_wall_loss + (q_amb[n] * patch_area[n]);
        }
    }

    // wallq (Qwall.f90:990-1245), T in K; the GUI, timer and print branches
    // are left out (qrn2, which the 20-second timer calls, only rebuilds QA)
    void wallq() {
        const int nb = (int)b_typ.size();
        q_incident_total = q_incident_wall = q_incident_inlet = q_incident_exit = q_incident_melt = ZERO;
        for (int n = 0; n < nb; ++n) {
            qc[n] = QA[cix(bc_i[n] / 2, bc_j[n] / 2, bc_k[n] / 2)] / b_face_area[n];
            q_incident_total = q_incident_total + (qc[n] * patch_area[n]);
            switch (b_typ[n]) {
            case 1: q_incident_wall = q_incident_wall + (qc[n] * patch_area[n]); break;
            case 2:
                q_incident_inlet = q_incident_inlet + (qc[n] * patch_area[n]);
                qeb[n] = pr.sig * pow4(b_T[n]);
                break;
            case 3:
                q_incident_exit = q_incident_exit + (qc[n] * patch_area[n]);
                qeb[n] = pr.sig * pow4(b_T[n]);
                break;
            case 4:
                q_incident_melt = q_incident_melt + (qc[n] * patch_area[n]);
                qeb[n] = emis[n] * pr.sig * pow4(b_T[n]);
                QE[cix(bc_i[n] / 2, bc_j[n] / 2, bc_k[n] / 2)] = qeb[n];
                break;
            }
        }
        const double wall_radiosity_tolerance = 1.0e-10, radiation_boundary_tolerance = 1.0e-10;
        double prev_q_melt_chg = 1.0e6;
        int nn = 1, nnextra = ws.maxri1;
        wall_outer = 0;
        while (nn <= ws.maxri1 && nn <= nnextra) {
            const int minradi = ws.minri2;
            calc_q_conv_wall(1.0);
            int n = 1, nextra = ws.maxri2;
            while (n <= ws.maxri2 && n <= nextra) {
                double rel_rad_chg_mean = ZERO;
                ++iterw;
                for (int i = 0; i < nb; ++i) {
                    rad_from_bnds = ZERO;
                    if (b_typ[i] == 1 || emis[i] < ONE) radiation_from_boundaries(i);
                    double rel_change = radiosity[i];
                    if (b_typ[i] == 1) radiosity[i] = fmax2(qc[i] + q_conv[i] - q_amb[i] + rad_from_bnds, emis[i] * radi_min);
                    else radiosity[i] = qeb[i] + (ONE - emis[i]) * (rad_from_bnds + qc[i]);
                    if (rel_change < wall_radiosity_tolerance) {
                        rel_change = ZERO;
                    } else {
                        rel_change = std::fabs((rel_change - radiosity[i]) / rel_change);
                        rel_rad_chg_mean = rel_rad_chg_mean + rel_change;
                    }
                }
                rel_rad_chg_mean = rel_rad_chg_mean / nb;
                last_rel_rad_chg_mean = rel_rad_chg_mean;
                if (rel_rad_chg_mean < wall_radiosity_tolerance && n > minradi)
                    if (nextra == ws.maxri2) nextra = n + 3;
                ++n;
            }
            // wall temperatures and the melt-surface flux (Qwall.f90:1134-1184)
            const double prev_q_melt = q_melt;
            q_melt = ZERO;
            for (int i = 0; i < nb; ++i) {
                if (b_typ[i] == 1) {
                    b_T[i] = std::pow(fmax2(ZERO, (radiosity[i] - (q_amb[i] - q_conv[i]) * (ONE - emis[i]) / emis[i]) / pr.sig), 0.25);
                    b_T[i] = fmax2(ws.t_mnk, b_T[i]);
                } else if (b_typ[i] == 4) {
                    radiation_from_boundaries(i);
                    double& q = qrs[(size_t)(b_i[i] - 1) + (size_t)MP * (b_j[i] - 1)];
                    q = qc[i] + q_conv[i] + rad_from_bnds - radiosity[i];
                    q_melt = q_melt + (q * patch_area[i]);
                }
            }
            wall_q_amb();
            const double q_melt_chg = std::fabs((prev_q_melt - q_melt) / (q_melt + small16));
            if (q_melt_chg < radiation_boundary_tolerance)
                if (nnextra == ws.maxri1) nnextra = nn + 1;
            prev_q_melt_chg = q_melt_chg;
            ++wall_outer;
            ++nn;
        }
        (void)prev_q_melt_chg;
        // after the loop (Qwall.f90:1192-1245)
        q_rad_outlet = q_rad_inlet = ZERO;
        double wall_TxArea_total = ZERO;
        qm_flame = qm_bnds = qm_conv = ZERO;
        for (int i = 0; i < nb; ++i) {
            switch (b_typ[i]) {
            case 1:
                a3(T, b_i[i], b_j[i], b_k[i]) = b_T[i];
                wall_TxArea_total = wall_TxArea_total + (b_T[i] * patch_area[i]);
                break;
            case 2:
                radiation_from_boundaries(i);
                q_rad_inlet = q_rad_inlet + (qc[i] + rad_from_bnds - qeb[i]) * patch_area[i];
                break;
            case 3:
                radiation_from_boundaries(i);
                q_rad_outlet = q_rad_outlet + (qc[i] + rad_from_bnds - qeb[i]) * patch_area[i];
                break;
            case 4: {
                radiation_from_boundaries(i);
                const double f_melt = 1.0 - qeb[i] / (emis[i] * (qc[i] + rad_from_bnds) + q_conv[i]);
                qm_flame = qm_flame + f_melt * emis[i] * qc[i] * patch_area[i];
                qm_bnds = qm_bnds + f_melt * emis[i] * rad_from_bnds * patch_area[i];
                qm_conv = qm_conv + f_melt * q_conv[i] * patch_area[i];
                break;
            }
            }
        }
        avg_wall_T = wall_TxArea_total / wall_area_total;
        if (have_frac_exh_T == 1)
            for (int i = 0; i < nb; ++i) {
                if (b_typ[i] != 3) continue;
                const int m = b_exh[i] - 1;
                b_T[i] = ws.exh_type[m] == 0 ? ws.exh_frac[m] * avg_wall_T : ws.exh_fixed[m];
            }
    }

    void SOURCE(int MI1, int MI3, int NJ1, int NJ3, int LK1, int LK3) {
        switch (NELG) {
        case 1: case 2: case 3: {
            int IU1 = NELG;
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) SRC1(I, J, K, IU1);
            break;
        }
        case 4: case 5: {
            if (NELG == 5) { res_mass = ZERO; res_mass_max = ZERO; }
            for (int i = MI1; i <= MI3; i += 2)
                for (int j = NJ1; j <= NJ3; j += 2)
                    for (int k = LK1; k <= LK3; k += 2) {
                        if (ibcell(i, j, k) >= 1) continue;
                        double area_x = AREA_C(i, j, k, 1);
                        double frx1 = (a3(THETA, i - 1, j, k) * a3(DNST, i - 1, j, k) * ug(i - 1, j, k, 1)) * area_x;
                        double frx2 = (a3(THETA, i + 1, j, k) * a3(DNST, i + 1, j, k) * ug(i + 1, j, k, 1)) * area_x;
                        double rx = frx1 - frx2;
                        double area_y = AREA_C(i, j, k, 2);
                        double fry1 = (a3(THETA, i, j - 1, k) * a3(DNST, i, j - 1, k) * ug(i, j - 1, k, 2)) * area_y;
                        double fry2 = (a3(THETA, i, j + 1, k) * a3(DNST, i, j + 1, k) * ug(i, j + 1, k, 2)) * area_y;
                        double ry = fry1 - fry2;
                        double area_z = AREA_C(i, j, k, 3);
                        double frz1 = (a3(THETA, i, j, k - 1) * a3(DNST, i, j, k - 1) * ug(i, j, k - 1, 3)) * area_z;
                        double frz2 = (a3(THETA, i, j, k + 1) * a3(DNST, i, j, k + 1) * ug(i, j, k + 1, 3)) * area_z;
                        double rz = frz1 - frz2;
                        const double evms = ZERO;
                        a3(BS, i, j, k) = (rx + ry + rz + evms) / pr.eun;
                        a3(SFP, i, j, k) = ZERO;
                        if (NELG == 5) {
                            double r_mass;
                            if (ibcell(i - 1, j, k) == 3 || ibcell(i + 1, j, k) == 3 || ibcell(i, j - 1, k) == 3 ||
                                ibcell(i, j + 1, k) == 3 || ibcell(i, j, k - 1) == 3 || ibcell(i, j, k + 1) == 3) {
                                continue;
                            } else {
                                double fmax = fmax2(fmax2(fmax2(fmax2(fmax2(fmax2(std::fabs(frx1), std::fabs(frx2)), std::fabs(fry1)),
                                                                   std::fabs(fry2)), std::fabs(frz1)), std::fabs(frz2)), evms);
                                if (fmax == ZERO) r_mass = ZERO;
                                else r_mass = std::fabs(a3(BS, i, j, k)) * pr.eun / fmax;
                            }
                            if (res_mass_max < r_mass) res_mass_max = r_mass;
                            res_mass = res_mass + r_mass;
                        }
                    }
            if (NELG == 5) res_mass = res_mass / NCELLS;
            break;
        }
        case 6: {
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        if (ibcell(I, J, K) >= 1) {
                            a3(BS, I, J, K) = a3(FZ, I, J, K); a3(SFP, I, J, K) = ZERO;
                            a3(CRATE, I, J, K) = ZERO; a3(HRATE, I, J, K) = ZERO;
                            continue;
                        }
                        const double SC = ZERO;
                        double D11 = std::fabs(ug(I + 1, J, K, 1) / DX[I]);
                        double D12 = std::fabs(ug(I - 1, J, K, 1) / DX[I]);
                        double D21 = 0, D22 = 0, D31 = 0, D32 = 0;
                        if (NJ3 > 6) { D21 = std::fabs(ug(I, J + 1, K, 2) / DR[J]); D22 = std::fabs(ug(I, J - 1, K, 2) / DR[J]); }
                        if (LK3 > 6) { D31 = std::fabs(ug(I, J, K + 1, 3) / DZ[K]); D32 = std::fabs(ug(I, J, K - 1, 3) / DZ[K]); }
                        double DTIME = fmax2(fmax2(fmax2(fmax2(fmax2(fmax2(D11, D12), D21), D22), D31), D32), SMX0);
                        DTIME = ONE / DTIME;
                        double DRTIME = DTIME * pr.r0 / pr.ug0;
                        double AYF = fmin2(gf(I, J, K, IYF), gf(I, J, K, IYO2) / pr.stoich);
                        if (AYF < 1.0e-5) {
                            a3(CRATE, I, J, K) = ZERO; a3(HRATE, I, J, K) = ZERO; a3(SFP, I, J, K) = ZERO; a3(BS, I, J, K) = ZERO;
                            continue;
                        }
                        double ZP1 = gf(I, J, K, IYCO2) / WCO2, DELR1;
                        if (ZP1 <= small20) DELR1 = ZERO;
                        else { double ZF = gf(I, J, K, IYF) / WF; DELR1 = ZP1 / (ZF + ZP1); }
                        double TIME1 = ZY1(DELR.data(), TIMED.data(), DELR1, NR0);
                        double TIME2 = TIME1 + DRTIME;
                        double DELR2 = ZY1(RTIM.data(), DELRT.data(), TIME2, NR0);
                        double AYF0 = AYF / (ONE - DELR1) * a3(DNST, I, J, K) * a3(THETA, I, J, K);
                        double SR = AYF0 * (DELR2 - DELR1) / DTIME;
                        if (SR <= ZERO) {
                            a3(CRATE, I, J, K) = ZERO; a3(HRATE, I, J, K) = ZERO; a3(SFP, I, J, K) = ZERO; a3(BS, I, J, K) = SC;
                            continue;
                        }
                        a3(CRATE, I, J, K) = SR;
                        a3(SFP, I, J, K) = -a3(CRATE, I, J, K) / (gf(I, J, K, IYF) + small20);
                        a3(BS, I, J, K) = SC;
                        a3(HRATE, I, J, K) = a3(CRATE, I, J, K) * pr.q0;
                    }
            break;
        }
        case 7: {
            double G0 = WCO2 / WF;
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        a3(SFP, I, J, K) = ZERO;
                        if (ibcell(I, J, K) >= 1) { a3(BS, I, J, K) = a3(FZ, I, J, K); continue; }
                        if (!pr.react) { a3(BS, I, J, K) = ZERO; continue; }
                        a3(BS, I, J, K) = a3(CRATE, I, J, K) * G0;
                    }
            break;
        }
        case 8: case 9: {
            if (NELG == 8) {
                q_rad_vol_tot = ZERO; q_react = ZERO;
                for (int I = MI1; I <= MI3; I += 2)
                    for (int J = NJ1; J <= NJ3; J += 2)
                        for (int K = LK1; K <= LK3; K += 2) {
                            if (ibcell(I, J, K) >= 1) continue;
                            double DUDX, DVDX, DWDX, DUDR, DVDR, DWDR, DUDZ, DVDZ, DWDZ;
                            if (ibcell(I + 1, J, K) == 3 || ibcell(I - 1, J, K) == 3) { DUDX = DVDX = DWDX = ZERO; }
                            else {
                                DUDX = (ug(I + 1, J, K, 1) - ug(I - 1, J, K, 1)) / DX[I];
                                DVDX = (ug(I + 1, J, K, 2) - ug(I - 1, J, K, 2)) / DX[I];
                                DWDX = (ug(I + 1, J, K, 3) - ug(I - 1, J, K, 3)) / DX[I];
                            }
                            if (NJ3 < 6 || ibcell(I, J + 1, K) == 3 || ibcell(I, J - 1, K) == 3) { DUDR = DVDR = DWDR = ZERO; }
                            else {
                                DUDR = (ug(I, J + 1, K, 1) - ug(I, J - 1, K, 1)) / DR[J];
                                DVDR = (ug(I, J + 1, K, 2) - ug(I, J - 1, K, 2)) / DR[J];
                                DWDR = (ug(I, J + 1, K, 3) - ug(I, J - 1, K, 3)) / DR[J];
                            }
                            if (LK3 < 6 || ibcell(I, J, K + 1) == 3 || ibcell(I, J, K - 1) == 3) { DUDZ = DVDZ = DWDZ = ZERO; }
                            else {
                                DUDZ = (ug(I, J, K + 1, 1) - ug(I, J, K - 1, 1)) / DZ[K];
                                DVDZ = (ug(I, J, K + 1, 2) - ug(I, J, K - 1, 2)) / DZ[K];
                                DWDZ = (ug(I, J, K + 1, 3) - ug(I, J, K - 1, 3)) / DZ[K];
                            }
                            const double VR = ZERO;
                            double s1 = DUDR + DVDX, s2 = DWDR + DVDZ, s3 = DUDZ + DWDX, s4 = DUDX + DVDR + DWDZ;
                            a3(GTE, I, J, K) = TWO * (DUDX * DUDX + DVDR * DVDR + VR * VR + DWDZ * DWDZ) + s1 * s1 + s2 * s2 +
                                               s3 * s3 - s4 * s4 / 1.5;
                        }
                for (int I = MI1; I <= MI3; I += 2) {
                    int ID2 = I / 2;
                    for (int J = NJ1; J <= NJ3; J += 2) {
                        int JD2 = J / 2;
                        for (int K = LK1; K <= LK3; K += 2) {
                            if (ibcell(I, J, K) >= 1) { a3(BS, I, J, K) = a3(FZ, I, J, K); a3(SFP, I, J, K) = ZERO; continue; }
                            int KD2 = K / 2;
                            const double GDZ = ZERO, GDZH = ZERO;
                            double CPMIX1 = CPF1 * gf(I, J, K, IYF) + CPCO21 * gf(I, J, K, IYCO2) + CPH2O1 * gf(I, J, K, IYH2O) +
                                            CPO21 * gf(I, J, K, IYO2) + CPN21 * gf(I, J, K, IYN2);
                            a3(BS, I, J, K) = GDZH + a3(HRATE, I, J, K);
                            a3(SFP, I, J, K) = -GDZ / CPMIX1;
                            double vol = VOL_C(I, J, K) * 1.0;   // *vol0
                            q_react = q_react + a3(HRATE, I, J, K) * pr.qr0 * vol;
                            if (i1st_rad_qe_done > 0) {
                                double q_rad = QA[cix(ID2, JD2, KD2)] - QE[cix(ID2, JD2, KD2)];
                                a3(BS, I, J, K) = a3(BS, I, J, K) + q_rad / (vol * pr.qr0);
                                q_rad_vol_tot = q_rad_vol_tot - q_rad;
                            }
                        }
                    }
                }
                if (pr.wall_sink) {
                    // q_conv was evaluated at the start of GSLV3G (see GSLV3G)
                    for (size_t n = 0; n < b_typ.size(); ++n) {
                        if (b_typ[n] == 1 || b_typ[n] == 4) {
                            int inc = b_i[n], jnc = b_j[n], knc = b_k[n];
                            double ds;
                            if (b_orient[n] == 1) { inc = b_direct[n] == 0 ? inc + 1 : inc - 1; ds = DX[inc]; }
                            else if (b_orient[n] == 2) { jnc = b_direct[n] == 0 ? jnc + 1 : jnc - 1; ds = DR[jnc]; }
                            else { knc = b_direct[n] == 0 ? knc + 1 : knc - 1; ds = DZ[knc]; }
                            a3(BS, inc, jnc, knc) = a3(BS, inc, jnc, knc) - q_conv[n] / (ds * pr.r0 * pr.qr0);
                        }
                    }
                }
                if (itr_gas > 1) {
                    for (int i = MI1; i <= MI3; i += 2)
                        for (int j = NJ1; j <= NJ3; j += 2)
                            for (int k = LK1; k <= LK3; k += 2) {
                                if (ibcell(i, j, k) >= 1) continue;
                                a3(BS, i, j, k) = pr.rf_hsource * a3(BS, i, j, k) + (ONE - pr.rf_hsource) * a3(bs_hprev, i, j, k);
                            }
                }
                bs_hprev = BS;
                break;
            }
            // NELG == 9: turbulent kinetic energy (LSTAR<=3: GTE from the enthalpy call)
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        if (ibcell(I, J, K) >= 1) { a3(BS, I, J, K) = a3(FZ, I, J, K); a3(SFP, I, J, K) = ZERO; continue; }
                        const double SUM = ZERO;
                        a3(BS, I, J, K) = TWO / (pr.reyg * pr.epsr) * a3(THETA, I, J, K) * a3(TMU, I, J, K) * a3(GTE, I, J, K) - SUM;
                        a3(SFP, I, J, K) = -(pr.taur * a3(THETA, I, J, K) * a3(DNST, I, J, K) * gf(I, J, K, IEPS) /
                                             (gf(I, J, K, IK) + small20));
                    }
            break;
        }
        case 10: {
            double CBL0 = 2.5 * std::sqrt(pr.epsr) / pr.taur * std::pow(pr.cmu, 0.75);
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        a3(SFP, I, J, K) = ZERO;
                        if (ibcell(I, J, K) >= 1) { a3(BS, I, J, K) = a3(FZ, I, J, K); continue; }
                        double CBL = CBL0 * std::pow(gf(I, J, K, IK), 1.5);
                        a3(BS, I, J, K) = ZERO;
                        if (MP > 8 && ibcell(I + 1, J, K) == 1) { a3(BS, I, J, K) = a3(BS, I, J, K) + BIG * CBL / (X[I + 1] - X[I]); a3(SFP, I, J, K) = -BIG; }
                        if (MP > 8 && ibcell(I - 1, J, K) == 1) { a3(BS, I, J, K) = a3(BS, I, J, K) + BIG * CBL / (X[I] - X[I - 1]); a3(SFP, I, J, K) = -BIG; }
                        if (NP > 8 && ibcell(I, J + 1, K) == 1) { a3(BS, I, J, K) = a3(BS, I, J, K) + BIG * CBL / (R[J + 1] - R[J]); a3(SFP, I, J, K) = -BIG; }
                        if (NP > 8 && ibcell(I, J - 1, K) == 1) { a3(BS, I, J, K) = a3(BS, I, J, K) + BIG * CBL / (R[J] - R[J - 1]); a3(SFP, I, J, K) = -BIG; }
                        if (LP > 8 && ibcell(I, J, K + 1) == 1) { a3(BS, I, J, K) = a3(BS, I, J, K) + BIG * CBL / (Z[K + 1] - Z[K]); a3(SFP, I, J, K) = -BIG; }
                        if (LP > 8 && ibcell(I, J, K - 1) == 1) { a3(BS, I, J, K) = a3(BS, I, J, K) + BIG * CBL / (Z[K] - Z[K - 1]); a3(SFP, I, J, K) = -BIG; }
                        if (a3(SFP, I, J, K) <= -BIG) continue;
                        double BT = a3(THETA, I, J, K);
                        a3(BS, I, J, K) = pr.ct1 * pr.cmu * BT / pr.taur * a3(DNST, I, J, K) * a3(GTE, I, J, K) * gf(I, J, K, IK);
                        a3(SFP, I, J, K) = -(pr.ct2 * pr.taur * BT * a3(DNST, I, J, K) * gf(I, J, K, IEPS) / (gf(I, J, K, IK) + small20));
                    }
            break;
        }
        case 11: {
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        if (ibcell(I, J, K) >= 1) { a3(BS, I, J, K) = a3(FZ, I, J, K); a3(SFP, I, J, K) = ZERO; continue; }
                        a3(BS, I, J, K) = ZERO; a3(SFP, I, J, K) = ZERO;
                    }
            break;
        }
        case 12: {
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        a3(SFP, I, J, K) = ZERO;
                        if (ibcell(I, J, K) >= 1) { a3(BS, I, J, K) = a3(FZ, I, J, K); continue; }
                        if (!pr.react) { a3(BS, I, J, K) = ZERO; continue; }
                        a3(BS, I, J, K) = -a3(CRATE, I, J, K) * pr.stoich;
                    }
            break;
        }
        default: break;
        }
    }

    // ---- Adlbl3.f90 ----------------------------------------------------------------
    // XT2/XT3 are (NP,LP) planes, 1-based
    vec XT2, XT3;
    int JBML, JEPL, IPL, IML;
    double& p2(vec& v, int j, int k) { return v[(long)(j - 1) + (long)NP * (k - 1)]; }

    void ADLZY(vec& XT, int LD, int I, int JB, int JE, int K) {
        if (JE == 2) return;
        int KPL = K + LD, KML = K - LD;
        std::vector<double> PT(NP + 2, 0.0), QT(NP + 2, 0.0);
        PT[JBML] = ZERO;
        QT[JBML] = XT[ix(I, JBML, K)];
        for (int J = JB; J <= JE; J += LD) {
            int JML = J - LD;
            double ALP = a3(AP, I, J, K) - PT[JML] * as(I, J, K, 2, 1);
            double BSY = a3(BS, I, J, K);
            if (std::fabs(ALP) <= small20 || ibcell(I * 2 / LD, J * 2 / LD, K * 2 / LD) >= 1) {
                PT[J] = ZERO;
                QT[J] = XT[ix(I, J, K)];
            } else {
                PT[J] = as(I, J, K, 2, 2) / ALP;
                BSY = BSY + as(I, J, K, 1, 2) * XT[ix(IPL, J, K)] + as(I, J, K, 1, 1) * XT[ix(IML, J, K)];
                if (LP >= 6) BSY = BSY + as(I, J, K, 3, 2) * XT[ix(I, J, KPL)] + as(I, J, K, 3, 1) * XT[ix(I, J, KML)];
                QT[J] = (BSY + as(I, J, K, 2, 1) * QT[JML]) / ALP;
            }
        }
        for (int J = JE; J >= JB; J -= LD) p2(XT2, J, K) = p2(XT2, J + LD, K) * PT[J] + QT[J];
    }
    void ADLYZ(vec& XT, int LD, int I, int J, int KB, int KE) {
        if (LP == 2) return;
        int JPL = J + LD, JML = J - LD, KBML = KB - LD;
        std::vector<double> PT(LP + 2, 0.0), QT(LP + 2, 0.0);
        PT[KBML] = ZERO;
        QT[KBML] = XT[ix(I, J, KBML)];
        for (int K = KB; K <= KE; K += LD) {
            int KML = K - LD;
            double ALP = a3(AP, I, J, K) - PT[KML] * as(I, J, K, 3, 1);
            double BSY = a3(BS, I, J, K);
            if (std::fabs(ALP) <= small20 || ibcell(I * 2 / LD, J * 2 / LD, K * 2 / LD) >= 1) {
                PT[K] = ZERO;
                QT[K] = XT[ix(I, J, K)];
            } else {
                PT[K] = as(I, J, K, 3, 2) / ALP;
                BSY = BSY + as(I, J, K, 1, 2) * XT[ix(IPL, J, K)] + as(I, J, K, 1, 1) * XT[ix(IML, J, K)];
                if (NP >= 6) BSY = BSY + as(I, J, K, 2, 2) * XT[ix(I, JPL, K)] + as(I, J, K, 2, 1) * XT[ix(I, JML, K)];
                QT[K] = (BSY + as(I, J, K, 3, 1) * QT[KML]) / ALP;
            }
        }
        for (int K = KE; K >= KB; K -= LD) p2(XT3, J, K) = p2(XT3, J, K + LD) * PT[K] + QT[K];
    }
    void ADLZ(vec& XT, int LD, int I, int JB, int JE, int KB, int KE) {
        int KEPL = (LP == 2) ? KE : KE + LD;
        for (int K = KB; K <= KEPL; K += LD)
            for (int J = JB; J <= JEPL; J += LD) { p2(XT2, J, K) = XT[ix(I, J, K)]; p2(XT3, J, K) = XT[ix(I, J, K)]; }
        for (int L = 1; L <= 2; ++L) {
            for (int K = KB; K <= KE; K += LD) ADLZY(XT, LD, I, JB, JE, K);
            if (KB >= KE) {
                for (int K = KB; K <= KE; K += LD)
                    for (int J = JB; J <= JE; J += LD) XT[ix(I, J, K)] = p2(XT2, J, K);
                return;
            }
            for (int J = JB; J <= JE; J += LD) ADLYZ(XT, LD, I, J, KB, KE);
            for (int K = KB; K <= KE; K += LD)
                for (int J = JB; J <= JE; J += LD) XT[ix(I, J, K)] = (p2(XT2, J, K) + p2(XT3, J, K)) / TWO;
        }
    }
    // Plane order of the sweeps.  GFM_ADI_MARCH is the reference's (Adlbl3.f90:39-51):
    // planes IB..IE, then IE..IB, NIM times.  GFM_ADI_REDBLACK is the order the GPU's
    // production line solver uses: per sweep, twice, first every plane IB, IB+4, ..
    // ("colour 0"), then every plane IB+2, IB+6, .. ("colour 1").  Planes of one
    // colour are not neighbours (a plane update reads the planes I-2 and I+2 only),
    // so visiting them one after another here equals visiting them all at once.  Each
    // visit is the reference's ADLZ unchanged; only the order of the visits differs.
    void ADLBL3(vec& XT, int IB, int IE, int JB, int JE, int KB, int KE, int NIM) {
        const int LD = 2;
        if (JE == 2) { JBML = JB; JEPL = JE; } else { JBML = JB - LD; JEPL = JE + LD; }
        XT2.assign((long)NP * LP, 0.0);
        XT3.assign((long)NP * LP, 0.0);
        for (int Ns = 1; Ns <= NIM; ++Ns) {
            if (pr.adi_mode == GFM_ADI_REDBLACK) {
                for (int half = 0; half < 2; ++half)
                    for (int colour = 0; colour < 2; ++colour)
                        for (int I = IB + LD * colour; I <= IE; I += 2 * LD) {
                            IPL = I + LD; IML = I - LD; ADLZ(XT, LD, I, JB, JE, KB, KE);
                        }
                continue;
            }
            for (int I = IB; I <= IE; I += LD) { IPL = I + LD; IML = I - LD; ADLZ(XT, LD, I, JB, JE, KB, KE); }
            for (int I = IE; I >= IB; I -= LD) { IPL = I + LD; IML = I - LD; ADLZ(XT, LD, I, JB, JE, KB, KE); }
        }
        // end-of-call RESG residual (Adlbl3.f90:60-94) only feeds the final print (Sprint.f90:33): not kept
    }

    double calc_residual(vec& xt, int ib, int ie, int jb, int je, int kb, int ke) {   // Adlbl3.f90:239-271
        double resid = ZERO;
        for (int k = kb; k <= ke; k += 2)
            for (int j = jb; j <= je; j += 2)
                for (int i = ib; i <= ie; i += 2) {
                    if (ibcell(i, j, k) > 0) continue;
                    double t1 = as(i, j, k, 1, 1) * xt[ix(i - 2, j, k)], t2 = as(i, j, k, 1, 2) * xt[ix(i + 2, j, k)];
                    double t3 = as(i, j, k, 2, 1) * xt[ix(i, j - 2, k)], t4 = as(i, j, k, 2, 2) * xt[ix(i, j + 2, k)];
                    double t5 = as(i, j, k, 3, 1) * xt[ix(i, j, k - 2)], t6 = as(i, j, k, 3, 2) * xt[ix(i, j, k + 2)];
                    double t7 = a3(AP, i, j, k) * xt[ix(i, j, k)], t8 = a3(BS, i, j, k);
                    double eq_max = fmax2(fmax2(fmax2(fmax2(fmax2(fmax2(fmax2(std::fabs(t1), std::fabs(t2)), std::fabs(t3)),
                                                                  std::fabs(t4)), std::fabs(t5)), std::fabs(t6)), std::fabs(t7)),
                                          std::fabs(t8));
                    resid = resid + std::fabs(t1 + t2 + t3 + t4 + t5 + t6 + t8 - t7) / eq_max;
                }
        resid = resid / NCELLS;
        return resid > 1.0e-16 ? resid : 1.0e-16;   // MAX(resid,1d-16): a NaN sum gives 1d-16
    }

    // ---- Gslv3v.f90 --------------------------------------------------------------
    void GSLV3V_momasm() {
        SGM = ONE;
        std::fill(AP.begin(), AP.end(), ONE);
        std::fill(AS.begin(), AS.end(), ZERO);
        for (int IU1 = 1; IU1 <= 3; ++IU1) {
            int NX[4] = {0, 0, 0, 0}; NX[IU1] = 1;
            for (int I = 2 + NX[1]; I <= MP - NX[1]; I += 2)
                for (int J = 2 + NX[2]; J <= NP - NX[2]; J += 2)
                    for (int K = 2 + NX[3]; K <= LP - NX[3]; K += 2) a3(FZ, I, J, K) = ug(I, J, K, IU1);
        }
        for (int IU1 = 1; IU1 <= 3; ++IU1) { NELG = IU1; GSLVX1(IU1); }
    }
    void GSLV3V_psolve() {
        NELG = 4;
        int MI1 = 4, MI3 = MPM2, NJ1 = NJY1, NJ3 = NJY2, LK1 = LKZ1, LK3 = LKZ2;
        SOURCE(MI1, MI3, NJ1, NJ3, LK1, LK3);
        for (int I = MI1; I <= MI3; I += 2)
            for (int J = NJ1; J <= NJ3; J += 2)
                for (int K = LK1; K <= LK3; K += 2) {
                    if (ibcell(I, J, K) >= 1) { a3(BS, I, J, K) = a3(P, I, J, K); continue; }
                    a3(AP, I, J, K) = -a3(SFP, I, J, K);
                    int I1 = I - 1;
                    for (int M = 1; M <= 2; ++M) {
                        if (M == 2) I1 = I + 1;
                        int IBC1 = ibcell(I1, J, K);
                        if (IBC1 <= 0 && std::fabs(a3(AP, I1, J, K)) > small20) {
                            double AREA = AREA_C(I, J, K, 1);
                            double th = a3(THETA, I1, J, K);
                            as(I, J, K, 1, M) = th * th * a3(DNST, I1, J, K) * (AREA * AREA) / a3(AP, I1, J, K) * DXAV(I1, J, K) / DX[I1];
                        }
                        a3(AP, I, J, K) = a3(AP, I, J, K) + as(I, J, K, 1, M);
                    }
                    int J1 = J - 1;
                    for (int M = 1; M <= 2; ++M) {
                        if (M == 2) J1 = J + 1;
                        int IBC1 = ibcell(I, J1, K);
                        if (IBC1 <= 0 && std::fabs(a3(AP, I, J1, K)) > small20) {
                            double AREA = AREA_C(I, J, K, 2);
                            double th = a3(THETA, I, J1, K);
                            as(I, J, K, 2, M) = th * th * a3(DNST, I, J1, K) * (AREA * AREA) / a3(AP, I, J1, K) * DRAV(I, J1, K) / DR[J1];
                        }
                        a3(AP, I, J, K) = a3(AP, I, J, K) + as(I, J, K, 2, M);
                    }
                    int K1 = K - 1;
                    for (int M = 1; M <= 2; ++M) {
                        if (M == 2) K1 = K + 1;
                        int IBC1 = ibcell(I, J, K1);
                        if (IBC1 <= 0 && std::fabs(a3(AP, I, J, K1)) > small20) {
                            double AREA = AREA_C(I, J, K, 3);
                            double th = a3(THETA, I, J, K1);
                            as(I, J, K, 3, M) = th * th * a3(DNST, I, J, K1) * (AREA * AREA) / a3(AP, I, J, K1) * DZAV(I, J, K1) / DZ[K1];
                        }
                        a3(AP, I, J, K) = a3(AP, I, J, K) + as(I, J, K, 3, M);
                    }
                }
        p_resid_pre = calc_residual(P, MI1, MI3, NJ1, NJ3, LK1, LK3);
        ADLBL3(P, MI1, MI3, NJ1, NJ3, LK1, LK3, pr.ntimesg[NELG - 1]);
        p_resid = calc_residual(P, MI1, MI3, NJ1, NJ3, LK1, LK3);
        for (int I = MI1; I <= MI3; I += 2)
            for (int J = NJ1; J <= NJ3; J += 2)
                for (int K = LK1; K <= LK3; K += 2) {
                    if (ibcell(I, J, K) >= 1) continue;
                    BOUND(a3(P, I, J, K), 0, 1);
                }
    }
    void GSLV3V_momsolve() {
        for (int IU1 = 1; IU1 <= 3; ++IU1) {
            NELG = IU1;
            int NX[4] = {0, 0, 0, 0}; NX[IU1] = 1;
            int MI1 = 4 + NX[1], MI3 = MPM2 - NX[1], NJ1 = NJY1V[IU1], NJ3 = NJY2V[IU1], LK1 = LKZ1V[IU1], LK3 = LKZ2V[IU1];
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        if (ibcell(I, J, K) >= 1) continue;
                        a3(AP, I, J, K) = a3(AP, I, J, K) / pr.rf[NELG - 1];
                        double VOL = VOL_C(I, J, K), DPDX;
                        if (IU1 == 1) DPDX = (a3(P, I - 1, J, K) - a3(P, I + 1, J, K)) / DX[I];
                        else if (IU1 == 2) DPDX = (a3(P, I, J - 1, K) - a3(P, I, J + 1, K)) / DR[J] / RS[J];
                        else DPDX = (a3(P, I, J, K - 1) - a3(P, I, J, K + 1)) / DZ[K];
                        a3(BS, I, J, K) = a3(BS, I, J, K) + pr.eun * a3(THETA, I, J, K) * VOL * DPDX +
                                          RFC[NELG - 1] * a3(AP, I, J, K) * a3(FZ, I, J, K);
                    }
            u_resid_pre[IU1 - 1] = calc_residual(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3);
            ADLBL3(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3, pr.ntimesg[NELG - 1]);
            u_resid[IU1 - 1] = calc_residual(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3);
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        if (ibcell(I, J, K) >= 1) continue;
                        BOUND(a3(FZ, I, J, K), IU1, 1);
                        ug(I, J, K, IU1) = a3(FZ, I, J, K);
                    }
        }
    }
    void GSLV3V_pcorr() {
        NELG = 5;
        int MI1 = 4, MI3 = MPM2, NJ1 = NJY1, NJ3 = NJY2, LK1 = LKZ1, LK3 = LKZ2;
        SOURCE(MI1, MI3, NJ1, NJ3, LK1, LK3);
        for (int I = 2; I <= MP; I += 2)
            for (int J = 2; J <= NP; J += 2)
                for (int K = 2; K <= LP; K += 2) a3(FZ, I, J, K) = ZERO;
        ADLBL3(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3, pr.ntimesg[NELG - 1]);
        pcorr_resid = calc_residual(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3);
    }
    void GSLV3V_velcorr() {
        for (int IU1 = 1; IU1 <= 3; ++IU1) {
            int NX[4] = {0, 0, 0, 0}; NX[IU1] = 1;
            int MI1 = 4 + NX[1], MI3 = MPM2 - NX[1], NJ1 = NJY1V[IU1], NJ3 = NJY2V[IU1], LK1 = LKZ1V[IU1], LK3 = LKZ2V[IU1];
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        if (ibcell(I, J, K) >= 1 || std::fabs(a3(AP, I, J, K)) < small20) continue;
                        double VOL = VOL_C(I, J, K), DPDX;
                        if (IU1 == 1) DPDX = (a3(FZ, I - 1, J, K) - a3(FZ, I + 1, J, K)) / DX[I];
                        else if (IU1 == 2) DPDX = (a3(FZ, I, J - 1, K) - a3(FZ, I, J + 1, K)) / DR[J] / RS[J];
                        else DPDX = (a3(FZ, I, J, K - 1) - a3(FZ, I, J, K + 1)) / DZ[K];
                        double G0 = pr.eun * a3(THETA, I, J, K) * DPDX * VOL / (a3(AP, I, J, K) * pr.rf[IU1 - 1]);
                        ug(I, J, K, IU1) = ug(I, J, K, IU1) + G0;
                        BOUND(ug(I, J, K, IU1), IU1, 1);
                    }
        }
    }
    void GSLV3V_exits() {
        EXTRV(0);
        GFIN = GFIN0 * pr.gmfr;   // FLX1D, NPHAS=1 (Flx1d.f90:75-77)
        if (itr_gas > 10) {
            if (GFEX < small20) { FACTOR = ONE; FADJ = ZERO; }
            else {
                FACTOR = GFIN / GFEX;
                if (FACTOR > pr.f_mx) { FACTOR = pr.f_mx; FADJ = ZERO; }
                else if (FACTOR < pr.f_mn) { FACTOR = pr.f_mn; FADJ = ZERO; }
            }
        }
        EXTRV(1);
        INTPV();
    }

    // ---- Extr.f90 ----------------------------------------------------------------
    void EXTR1(double& F1, double& F2, int I, int J, int K, int I1, int J1, int K1, int I2, int J2, int K2, int IXD) {
        F2 = ZERO;
        int IBC0 = ibcell(I, J, K) % 10;
        if (IXD == 3) {
            double DZK = Z[K2] - Z[K1];
            if (DZK != ZERO) { int K0 = IBC0 == 2 ? (K + K1) / 2 : K; F2 = (Z[K0] - Z[K1]) / DZK; }
        } else if (IXD == 2) {
            double DRJ = R[J2] - R[J1];
            if (DRJ != ZERO) { int J0 = IBC0 == 2 ? (J + J1) / 2 : J; F2 = (R[J0] - R[J1]) / DRJ; }
        } else if (IXD == 1) {
            double DXI = X[I2] - X[I1];
            if (DXI != ZERO) { int I0 = IBC0 == 2 ? (I + I1) / 2 : I; F2 = (X[I0] - X[I1]) / DXI; }
        }
        F1 = ONE - F2;
    }
    // EXT0 / EXT1 (Extr.f90:575-661).  Returns false when no neighbour was
    // found (the reference then keeps the loop's last indices and IX=4).
    bool EXT01(bool wall, int I, int J, int K, int& I1, int& J1, int& K1, int& I2, int& J2, int& K2, int& IXD) {
        for (IXD = 1; IXD <= 3; ++IXD) {
            int NX[4] = {0, 0, 0, 0}; NX[IXD] = 1;
            for (int M = -2; M <= 2; M += 4) {
                I1 = std::max(2, std::min(MP, I + M * NX[1]));
                J1 = std::max(2, std::min(NP, J + M * NX[2]));
                K1 = std::max(2, std::min(LP, K + M * NX[3]));
                bool hit = wall ? (ibcell(I1, J1, K1) % 10 != 1) : (ibcell(I1, J1, K1) <= 0);
                if (hit) {
                    I2 = std::max(2, std::min(MP, I1 + M * NX[1]));
                    J2 = std::max(2, std::min(NP, J1 + M * NX[2]));
                    K2 = std::max(2, std::min(LP, K1 + M * NX[3]));
                    if (ibcell(I2, J2, K2) % 10 == 1) { I2 = I1; J2 = J1; K2 = K1; }
                    return true;
                }
            }
        }
        // fall-through: last tried indices are (I,J,min(LP,K+2)); I2 keeps a
        // stale value in the reference and enters only with weight F2=0
        IXD = 4;
        I2 = I1; J2 = J1; K2 = K1;
        return false;
    }
    void SBC4(int I1, int J1, int K1, int I, int J, int K) {
        a3(P, I, J, K) = a3(P, I1, J1, K1);
        a3(T, I, J, K) = a3(T, I1, J1, K1);
        for (int L = 1; L <= 9; ++L) gf(I, J, K, L) = gf(I1, J1, K1, L);
        a3(DNST, I, J, K) = a3(DNST, I1, J1, K1);
        a3(THETA, I, J, K) = a3(THETA, I1, J1, K1);
        a3(TMU, I, J, K) = a3(TMU, I1, J1, K1);
        a3(GAMA, I, J, K) = a3(GAMA, I1, J1, K1);
    }
    void EXTR() {   // EXTR(1): gas-phase variables
        GFIN0 = ZERO;
        q_exhaust = ZERO;
        for (int I = 2; I <= MP; I += 2)
            for (int J = 2; J <= NP; J += 2)
                for (int K = 2; K <= LP; K += 2) {
                    int IBC0 = ibcell(I, J, K) % 10;
                    if (IBC0 != 2 && IBC0 != 3) continue;
                    int I1, J1, K1, I2, J2, K2, IXD;
                    EXT01(false, I, J, K, I1, J1, K1, I2, J2, K2, IXD);
                    double F1, F2;
                    EXTR1(F1, F2, I, J, K, I1, J1, K1, I2, J2, K2, IXD);
                    gf(I, J, K, IEPS) = gf(I1, J1, K1, IEPS);
                    a3(P, I, J, K) = a3(P, I1, J1, K1) * F1 + a3(P, I2, J2, K2) * F2;
                    if (IBC0 == 2) {
                        double G0 = a3(TMU, I, J, K);
                        THER(I, J, K);
                        a3(TMU, I, J, K) = G0;
                        a3(GAMA, I, J, K) = a3(GAMA, I1, J1, K1);
                        double AREA = AREA_C(I, J, K, IXD);
                        G0 = a3(THETA, I, J, K) * a3(DNST, I, J, K) * ug(I, J, K, IXD) * AREA;
                        GFIN0 = GFIN0 + std::fabs(G0);
                        continue;
                    }
                    a3(TMU, I, J, K) = a3(TMU, I1, J1, K1);
                    a3(GAMA, I, J, K) = a3(GAMA, I1, J1, K1);
                    for (int L = LSTAR; L <= LEND; ++L) {
                        if (L == IEPS) continue;
                        double G0 = gf(I1, J1, K1, L) * F1 + gf(I2, J2, K2, L) * F2;
                        if (L == IK) gf(I, J, K, IK) = fmax2(G0, 1.0e-6);
                        else if (L == IH) gf(I, J, K, L) = G0;
                        else gf(I, J, K, L) = fmax2(G0, ZERO);
                    }
                    enth_to_T_at(I, J, K);
                    dnst_calc(I, J, K);
                    double AREA = AREA_C(I, J, K, IXD) * 1.0;
                    double G0 = std::fabs(ug(I, J, K, IXD)) * pr.ug0 * AREA;
                    G0 = G0 * a3(THETA, I, J, K) * a3(DNST, I, J, K) * pr.dnst0;
                    q_exhaust = q_exhaust + gf(I, J, K, IH) * pr.h_0 * G0;
                    if (IBC0 == 3) SBC4(I, J, K, (I + I1) / 2, (J + J1) / 2, (K + K1) / 2);
                }
        for (int I = 2; I <= MP; I += 2)
            for (int J = 2; J <= NP; J += 2)
                for (int K = 2; K <= LP; K += 2) {
                    int IBC0 = ibcell(I, J, K) % 10;
                    if (IBC0 != 1) continue;
                    int I1, J1, K1, I2, J2, K2, IXD;
                    EXT01(true, I, J, K, I1, J1, K1, I2, J2, K2, IXD);
                    double F1, F2;
                    EXTR1(F1, F2, I, J, K, I1, J1, K1, I2, J2, K2, IXD);
                    a3(P, I, J, K) = a3(P, I1, J1, K1) * F1 + a3(P, I2, J2, K2) * F2;
                    a3(TMU, I, J, K) = a3(TMU, I2, J2, K2);
                    a3(GAMA, I, J, K) = a3(GAMA, I2, J2, K2);
                    for (int L = LSTAR; L <= LEND; ++L)
                        if (L != IH) gf(I, J, K, L) = gf(I1, J1, K1, L);
                    // walls adiabatic until the first full radiation call (Extr.f90:194-197)
                    if (i1st_rad_done == 0) {
                        gf(I, J, K, IH) = gf(I1, J1, K1, IH);
                        a3(T, I, J, K) = a3(T, I1, J1, K1);
                    }
                    dnst_calc(I, J, K);
                }
    }
    void EXTRV(int MEX) {   // Extr.f90:358-567
        double Tarea_mean = 0, area_ex = 0;
        if (MEX == 0) { GFEX = ZERO; Tmean_ex = ZERO; }
        int IU = 1;
        for (int I = 3; I <= MPM1; I += 2)
            for (int J = 2; J <= NP; J += 2)
                for (int K = 2; K <= LP; K += 2) {
                    if (ibcell(I, J, K) % 10 != 3) continue;
                    bool done = false;
                    for (int M = -1; M <= 1 && !done; M += 2) {
                        if (ibcell(I + M, J, K) >= 1) continue;
                        int I0 = I - M, I1 = I + 2 * M;
                        if (ug(I1, J, K, IU) * M > ZERO) ug(I1, J, K, IU) = ZERO;
                        double AREA = AREA_C(I, J, K, IU);
                        area_ex = area_ex + AREA;
                        double G0 = a3(THETA, I1, J, K) * a3(DNST, I1, J, K) * ug(I1, J, K, IU) * AREA;
                        if (MEX == 0) {
                            GFEX = GFEX + std::fabs(G0);
                            Tmean_ex = Tmean_ex + a3(T, I, J, K) * std::fabs(G0);
                            Tarea_mean = Tarea_mean + a3(T, I, J, K) * AREA;
                            done = true; break;
                        }
                        ug(I1, J, K, IU) = ug(I1, J, K, IU) * FACTOR;
                        G0 = G0 * FACTOR;
                        ug(I, J, K, IU) = G0 / (a3(THETA, I, J, K) * a3(DNST, I, J, K) * AREA);
                        BOUND(ug(I, J, K, IU), IU, 1);
                        ug(I0, J, K, IU) = ug(I, J, K, IU);
                        done = true; break;
                    }
                    if (done) continue;
                    if (J > 2 && ibcell(I, J - 2, K) <= 0) ug(I, J, K, IU) = ug(I, J - 2, K, IU);
                    else if (J < NP && ibcell(I, J + 2, K) <= 0) ug(I, J, K, IU) = ug(I, J + 2, K, IU);
                    else if (K > 2 && ibcell(I, J, K - 2) <= 0) ug(I, J, K, IU) = ug(I, J, K - 2, IU);
                    else if (K < LP && ibcell(I, J, K + 2) <= 0) ug(I, J, K, IU) = ug(I, J, K + 2, IU);
                }
        IU = 2;
        for (int J = 3; J <= NPM1; J += 2)
            for (int K = 2; K <= LP; K += 2)
                for (int I = 2; I <= MP; I += 2) {
                    if (ibcell(I, J, K) % 10 != 3) continue;
                    bool done = false;
                    for (int M = -1; M <= 1 && !done; M += 2) {
                        if (ibcell(I, J + M, K) >= 1) continue;
                        int J0 = J - M, J1 = J + 2 * M;
                        if (ug(I, J1, K, IU) * M > ZERO) ug(I, J1, K, IU) = ZERO;
                        double AREA = AREA_C(I, J, K, IU);
                        area_ex = area_ex + AREA;
                        double G0 = a3(THETA, I, J1, K) * a3(DNST, I, J1, K) * ug(I, J1, K, IU) * AREA;
                        if (MEX == 0) {
                            GFEX = GFEX + std::fabs(G0);
                            Tmean_ex = Tmean_ex + a3(T, I, J, K) * std::fabs(G0);
                            Tarea_mean = Tarea_mean + a3(T, I, J, K) * AREA;
                            done = true; break;
                        }
                        ug(I, J1, K, IU) = ug(I, J1, K, IU) * FACTOR;
                        G0 = G0 * FACTOR;
                        ug(I, J, K, IU) = G0 / (a3(THETA, I, J, K) * a3(DNST, I, J, K) * AREA);
                        BOUND(ug(I, J, K, IU), IU, 1);
                        ug(I, J0, K, IU) = ug(I, J, K, IU);
                        done = true; break;
                    }
                    if (done) continue;
                    if (K > 2 && ibcell(I, J, K - 2) <= 0) ug(I, J, K, IU) = ug(I, J, K - 2, IU);
                    else if (K < LP && ibcell(I, J, K + 2) <= 0) ug(I, J, K, IU) = ug(I, J, K + 2, IU);
                    else if (I > 2 && ibcell(I - 2, J, K) <= 0) ug(I, J, K, IU) = ug(I - 2, J, K, IU);
                    else if (I < MP && ibcell(I + 2, J, K) <= 0) ug(I, J, K, IU) = ug(I + 2, J, K, IU);
                }
        IU = 3;
        for (int K = 3; K <= LPM1; K += 2)
            for (int I = 2; I <= MP; I += 2)
                for (int J = 2; J <= NP; J += 2) {
                    if (ibcell(I, J, K) % 10 != 3) continue;
                    bool done = false;
                    for (int M = -1; M <= 1 && !done; M += 2) {
                        if (ibcell(I, J, K + M) >= 1) continue;
                        int K1 = K + 2 * M;
                        if (ug(I, J, K1, IU) * M > ZERO) ug(I, J, K1, IU) = ZERO;
                        double AREA = AREA_C(I, J, K, IU);
                        area_ex = area_ex + AREA;
                        double G0 = a3(THETA, I, J, K1) * a3(DNST, I, J, K1) * ug(I, J, K1, IU) * AREA;
                        if (MEX == 0) {
                            GFEX = GFEX + std::fabs(G0);
                            Tmean_ex = Tmean_ex + a3(T, I, J, K) * std::fabs(G0);
                            Tarea_mean = Tarea_mean + a3(T, I, J, K) * AREA;
                            done = true; break;
                        }
                        ug(I, J, K1, IU) = ug(I, J, K1, IU) * FACTOR;
                        done = true; break;   // GOTO 160 (Extr.f90:529)
                    }
                    if (done) continue;
                    if (I > 2 && ibcell(I - 2, J, K) <= 0) ug(I, J, K, IU) = ug(I - 2, J, K, IU);
                    else if (I < MP && ibcell(I + 2, J, K) <= 0) ug(I, J, K, IU) = ug(I + 2, J, K, IU);
                    else if (J > 2 && ibcell(I, J - 2, K) <= 0) ug(I, J, K, IU) = ug(I, J - 2, K, IU);
                    else if (J < NP && ibcell(I, J + 2, K) <= 0) ug(I, J, K, IU) = ug(I, J + 2, K, IU);
                }
        if (MEX == 0) {
            GFEX = GFEX * pr.gmfr;
            if (GFEX < small16) Tmean_ex = Tarea_mean * pr.t0 / area_ex;
            else Tmean_ex = Tmean_ex * pr.t0 * pr.gmfr / GFEX;
        }
    }

    // ---- Intp.f90 ------------------------------------------------------------------
    double INTP1(int I, int J, int K, int IXD) {
        double F1;
        if (IXD == 3) F1 = (DZ[K] <= ZERO || K > LP) ? ZERO : (Z[K] - Z[K - 1]) / DZ[K];
        else if (IXD == 2) F1 = (DR[J] <= ZERO || J > NP) ? ZERO : (R[J] - R[J - 1]) / DR[J];
        else F1 = (DX[I] <= ZERO || I > MP) ? ZERO : (X[I] - X[I - 1]) / DX[I];
        return F1;
    }
    // F1 is the caller's variable (Fortran pass by reference): INTP0 may
    // overwrite it and the caller keeps the new value for later positions.
    void INTP0(double& F1, int I, int J, int K, int I1, int J1, int K1, int I2, int J2, int K2) {
        if (ibcell(I, J, K) == 3) return;
        if (ibcell(I, J, K) == 2) {
            if (ibcell(I1, J1, K1) == 2 && ibcell(I2, J2, K2) == 0) F1 = ONE;
            else if (ibcell(I1, J1, K1) == 0 && ibcell(I2, J2, K2) == 2) F1 = ZERO;
        }
        double F2 = ONE - F1;
        a3(P, I, J, K) = F1 * a3(P, I1, J1, K1) + F2 * a3(P, I2, J2, K2);
        a3(T, I, J, K) = F1 * a3(T, I1, J1, K1) + F2 * a3(T, I2, J2, K2);
        for (int L = LSTAR; L <= LEND; ++L) gf(I, J, K, L) = F1 * gf(I1, J1, K1, L) + F2 * gf(I2, J2, K2, L);
        CONC(I, J, K);
        a3(TMU, I, J, K) = F1 * a3(TMU, I1, J1, K1) + F2 * a3(TMU, I2, J2, K2);
        a3(GAMA, I, J, K) = F1 * a3(GAMA, I1, J1, K1) + F2 * a3(GAMA, I2, J2, K2);
        a3(THETA, I, J, K) = F1 * a3(THETA, I1, J1, K1) + F2 * a3(THETA, I2, J2, K2);
        dnst_calc(I, J, K);
    }
    void INTP() {
        for (int I = 2; I <= MP; I += 2) {
            for (int K = 3; K <= LPM1; K += 2) {
                double F1 = INTP1(I, 0, K, 3);
                for (int J = 2; J <= NP; J += 2) {
                    if (ibcell(I, J, K) == 1) continue;
                    INTP0(F1, I, J, K, I, J, K + 1, I, J, K - 1);
                }
            }
            for (int J = 3; J <= NPM1; J += 2) {
                double F1 = INTP1(I, J, 0, 2);
                for (int K = 2; K <= LP; ++K) {
                    if (ibcell(I, J, K) == 1) continue;
                    INTP0(F1, I, J, K, I, J + 1, K, I, J - 1, K);
                }
            }
        }
        for (int I = 3; I <= MPM1; I += 2) {
            double F1 = INTP1(I, 0, 0, 1);
            for (int K = 2; K <= LP; ++K)
                for (int J = 2; J <= NP; ++J) {
                    if (ibcell(I, J, K) == 1) continue;
                    INTP0(F1, I, J, K, I + 1, J, K, I - 1, J, K);
                }
        }
    }
    void INTPV1(int M, int Nn, int L, int IU, int IXD) {
        int I, J, K;
        if (IU == 1) { I = M; J = Nn; K = L; } else if (IU == 2) { J = M; K = Nn; I = L; } else { K = M; I = Nn; J = L; }
        int b = ibcell(I, J, K);
        if (b >= 1 && b != 4) return;
        double F1 = INTP1(I, J, K, IXD), F2 = ONE - F1;
        if (IXD == 1) {
            ug(I, J, K, IU) = ug(I + 1, J, K, IU) * F1 + ug(I - 1, J, K, IU) * F2;
        } else if (IXD == 2) {
            if (ibcell(I, J + 1, K) == 2 && b == 0) { F1 = 0; F2 = 1; }
            else if (ibcell(I, J - 1, K) == 2 && b == 0) { F1 = 1; F2 = 0; }
            ug(I, J, K, IU) = ug(I, J + 1, K, IU) * F1 + ug(I, J - 1, K, IU) * F2;
        } else {
            if (ibcell(I, J, K + 1) == 2 && b == 0) { F1 = 0; F2 = 1; }
            else if (ibcell(I, J, K - 1) == 2 && b == 0) { F1 = 1; F2 = 0; }
            ug(I, J, K, IU) = ug(I, J, K + 1, IU) * F1 + ug(I, J, K - 1, IU) * F2;
        }
        BOUND(ug(I, J, K, IU), IU, 1);
    }
    void INTPV() {
        for (int IU = 1; IU <= 3; ++IU) {
            int M3, N3, L3;
            if (IU == 1) { M3 = MP; N3 = NP; L3 = LP; } else if (IU == 2) { M3 = NP; N3 = LP; L3 = MP; } else { M3 = LP; N3 = MP; L3 = NP; }
            for (int M = 3; M <= M3 - 1; M += 2) {
                if (N3 > 3) {
                    for (int L = 2; L <= L3; L += 2)
                        for (int Nn = 3; Nn <= N3 - 1; Nn += 2) INTPV1(M, Nn, L, IU, IU == 1 ? 2 : (IU == 2 ? 3 : 1));
                }
                if (L3 <= 3) continue;
                for (int L = 3; L <= L3 - 1; L += 2)
                    for (int Nn = 2; Nn <= N3; ++Nn) INTPV1(M, Nn, L, IU, IU == 1 ? 3 : (IU == 2 ? 1 : 2));
            }
            for (int M = 4; M <= M3; M += 2)
                for (int Nn = 2; Nn <= N3; ++Nn)
                    for (int L = 2; L <= L3; ++L) INTPV1(M, Nn, L, IU, IU);
        }
    }

    // ---- Gflow.f90 -----------------------------------------------------------------
    void wall_functions() {   // Gflow.f90:16-130
        for (int I = 2; I <= MP; ++I)
            for (int J = 2; J <= NP; ++J)
                for (int K = 2; K <= LP; ++K) {
                    if (ibcell(I, J, K) >= 1) continue;
                    if (ibcell(I - 1, J, K) == 1) {
                        double G1 = (X[I] - X[I - 1]) * (X[I] - X[I - 1]), G2 = (X[I + 2] - X[I - 1]) * (X[I + 2] - X[I - 1]);
                        double X01 = G2 / (G2 - G1), X02 = G1 / (G1 - G2);
                        a3(THETA, I - 1, J, K) = a3(THETA, I, J, K) * X01 + a3(THETA, I + 2, J, K) * X02;
                    }
                    if (ibcell(I + 1, J, K) == 1) {
                        double G1 = (X[I] - X[I + 1]) * (X[I] - X[I + 1]), G2 = (X[I - 2] - X[I + 1]) * (X[I - 2] - X[I + 1]);
                        double X01 = G2 / (G2 - G1), X02 = G1 / (G1 - G2);
                        a3(THETA, I + 1, J, K) = a3(THETA, I, J, K) * X01 + a3(THETA, I - 2, J, K) * X02;
                    }
                    if (ibcell(I, J - 1, K) == 1) {
                        double G1 = (R[J] - R[J - 1]) * (R[J] - R[J - 1]), G2 = (R[J + 2] - R[J - 1]) * (R[J + 2] - R[J - 1]);
                        double X01 = G2 / (G2 - G1), X02 = G1 / (G1 - G2);
                        a3(THETA, I, J - 1, K) = a3(THETA, I, J, K) * X01 + a3(THETA, I, J + 2, K) * X02;
                    }
                    if (ibcell(I, J + 1, K) == 1) {
                        double G1 = (R[J] - R[J + 1]) * (R[J] - R[J + 1]), G2 = (R[J - 2] - R[J + 1]) * (R[J - 2] - R[J + 1]);
                        double X01 = G2 / (G2 - G1), X02 = G1 / (G1 - G2);
                        a3(THETA, I, J + 1, K) = a3(THETA, I, J, K) * X01 + a3(THETA, I, J - 2, K) * X02;
                    }
                    if (ibcell(I, J, K - 1) == 1) {
                        double G1 = (Z[K] - Z[K - 1]) * (Z[K] - Z[K - 1]), G2 = (Z[K + 2] - Z[K - 1]) * (Z[K + 2] - Z[K - 1]);
                        double X01 = G2 / (G2 - G1), X02 = G1 / (G1 - G2);
                        a3(THETA, I, J, K - 1) = a3(THETA, I, J, K) * X01 + a3(THETA, I, J, K + 2) * X02;
                    }
                    if (ibcell(I, J, K + 1) == 1) {
                        double G1 = (Z[K] - Z[K + 1]) * (Z[K] - Z[K + 1]), G2 = (Z[K - 2] - Z[K + 1]) * (Z[K - 2] - Z[K + 1]);
                        double X01 = G2 / (G2 - G1), X02 = G1 / (G1 - G2);
                        a3(THETA, I, J, K + 1) = a3(THETA, I, J, K) * X01 + a3(THETA, I, J, K - 2) * X02;
                    }
                }
        for (int I = 2; I <= MP; ++I)
            for (int J = 2; J <= NP; ++J)
                for (int K = 2; K <= LP; ++K)
                    if (ibcell(I, J, K) == 1) a3(GAMA, I, J, K) = ZERO;
        double RT20 = pr.reyg2 * std::sqrt(pr.epsr) * std::pow(pr.cmu, 0.25);
        for (int I = 2; I <= MP; ++I)
            for (int J = 2; J <= NP; ++J)
                for (int K = 2; K <= LP; ++K) {
                    if (ibcell(I, J, K) >= 1) continue;
                    double C = std::pow(a3(T, I, J, K) / pr.trdg, pr.amu);
                    double BLVM = RT20 * a3(DNST, I, J, K) * std::sqrt(gf(I, J, K, IK)) / C;
                    double VGAM = C / pr.reyg2;
                    auto upd = [&](int i1, int j1, int k1, int i2, int j2, int k2, double dist) {
                        double BLV = BLVM * dist;
                        double GAMA0 = VGAM * TGAMF(BLV);
                        a3(GAMA, i1, j1, k1) = fmax2(GAMA0, a3(GAMA, i1, j1, k1));
                        a3(TMU, i1, j1, k1) = pr.reyg2 * a3(GAMA, i1, j1, k1);
                        a3(TMU, i2, j2, k2) = a3(TMU, i1, j1, k1);
                    };
                    if (ibcell(I - 1, J, K) == 1) upd(I - 1, J, K, I - 2, J, K, X[I] - X[I - 1]);
                    if (ibcell(I + 1, J, K) == 1) upd(I + 1, J, K, I + 2, J, K, X[I + 1] - X[I]);
                    if (ibcell(I, J - 1, K) == 1) upd(I, J - 1, K, I, J - 2, K, R[J] - R[J - 1]);
                    if (ibcell(I, J + 1, K) == 1) upd(I, J + 1, K, I, J + 2, K, R[J + 1] - R[J]);
                    if (ibcell(I, J, K - 1) == 1) upd(I, J, K - 1, I, J, K - 2, Z[K] - Z[K - 1]);
                    if (ibcell(I, J, K + 1) == 1) upd(I, J, K + 1, I, J, K + 2, Z[K + 1] - Z[K]);
                }
    }
    double pref_g0() {   // Gflow.f90:182-242
        int I = I_REF, J = J_REF, K = K_REF, I1 = I, J1 = J, K1 = K, I2 = I, J2 = J, K2 = K, NXd = 0;
        if (I < MPM2 && ibcell(I + 2, J, K) == 0) { NXd = 1; I1 = I + 2; I2 = ibcell(I + 4, J, K) == 0 ? I + 4 : I1; }
        else if (I > 2 && ibcell(I - 2, J, K) == 0) { NXd = 1; I1 = I - 2; I2 = ibcell(I - 4, J, K) == 0 ? I - 4 : I1; }
        else if (J < NPM2 && ibcell(I, J + 2, K) == 0) { NXd = 2; J1 = J + 2; J2 = (J < NPM2 && ibcell(I, J + 4, K) <= 0) ? J + 4 : J1; }
        else if (J > 2 && ibcell(I, J - 2, K) <= 0) { NXd = 2; J1 = J - 2; J2 = (J > 4 && ibcell(I, J - 4, K) <= 0) ? J - 4 : J1; }
        else if (K < LPM2 && ibcell(I, J, K + 2) <= 0) { NXd = 3; K1 = K + 2; K2 = (K < LPM2 && ibcell(I, J, K + 4) <= 0) ? K + 4 : K1; }
        else if (K > 2 && ibcell(I, J, K - 2) <= 0) { NXd = 3; K1 = K - 2; K2 = (K > 4 && ibcell(I, J, K - 4) <= 0) ? K - 4 : K1; }
        double F1, F2;
        EXTR1(F1, F2, I, J, K, I1, J1, K1, I2, J2, K2, NXd);
        a3(P, I, J, K) = a3(P, I1, J1, K1) * F1 + a3(P, I2, J2, K2) * F2;
        return a3(P, I1, J1, K1) - P_REF;
    }
    void GSLV3G() {   // Gslv3g.f90:6-115
        int MI1 = 4, MI3 = MPM2, NJ1 = NJY1, NJ3 = NJY2, LK1 = LKZ1, LK3 = LKZ2;
        // Fixed-temperature wall sink (configuration deviation): the reference
        // evaluates q_conv inside its full radiation call; here it is evaluated
        // once per iteration from the state at the start of the scalar loop.
        if (pr.wall_sink) calc_q_conv_wall();
        for (int L = LSTAR; L <= LEND; ++L) {
            if (L == IYF) NELG = 6;
            else if (L == IYCO2) NELG = 7;
            else if (L == IH) NELG = 8;
            else if (L == IK) NELG = 9;
            else if (L == IEPS) NELG = 10;
            else if (L == IYN2) NELG = 11;
            else if (L == IYO2) NELG = 12;
            else continue;
            for (int I = 2; I <= MP; I += 2)
                for (int J = 2; J <= NP; J += 2)
                    for (int K = 2; K <= LP; K += 2) a3(FZ, I, J, K) = gf(I, J, K, L);
            SOURCE(MI1, MI3, NJ1, NJ3, LK1, LK3);
            if (L == LSTAR || SGM != pr.sigma[L - 1]) { SGM = pr.sigma[L - 1]; GSLV3G0(MI1, MI3, NJ1, NJ3, LK1, LK3, 0); }
            else GSLV3G0(MI1, MI3, NJ1, NJ3, LK1, LK3, 1);
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        if (ibcell(I, J, K) >= 1) continue;
                        if (std::fabs(a3(AP, I, J, K)) <= small20) { a3(AP, I, J, K) = ONE; a3(BS, I, J, K) = a3(FZ, I, J, K); continue; }
                        double VOL = VOL_C(I, J, K);
                        a3(BS, I, J, K) = a3(BS, I, J, K) * VOL;
                        a3(AP, I, J, K) = a3(AP, I, J, K) - (a3(SFP, I, J, K) * VOL);
                        a3(AP, I, J, K) = a3(AP, I, J, K) / pr.rfl[L - 1];
                        a3(BS, I, J, K) = a3(BS, I, J, K) + RFLC[L - 1] * a3(FZ, I, J, K) * a3(AP, I, J, K);
                    }
            if (NELG == 8) h_resid_pre = calc_residual(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3);
            gf_resid_pre[L - 1] = calc_residual(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3);
            ADLBL3(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3, pr.ntimesg[NELG - 1]);
            gf_resid[L - 1] = calc_residual(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3);
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        if (ibcell(I, J, K) >= 1) continue;
                        BOUND(a3(FZ, I, J, K), L, 2);
                        gf(I, J, K, L) = a3(FZ, I, J, K);
                    }
        }
    }
    void GSLV3G0(int MI1, int MI3, int NJ1, int NJ3, int LK1, int LK3, int IGS) {
        for (int I = MI1; I <= MI3; I += 2)
            for (int J = NJ1; J <= NJ3; J += 2)
                for (int K = LK1; K <= LK3; K += 2) {
                    if (ibcell(I, J, K) >= 1) continue;
                    a3(AP, I, J, K) = ZERO;
                    for (int IU = 1; IU <= 3; ++IU)
                        for (int M = -1; M <= 1; M += 2) {
                            int M1 = (M + 3) / 2;
                            if (IGS != 1) {
                                int I1, J1, K1, I2, J2, K2;
                                VINDX(IU, M, I, J, K, I1, J1, K1, I2, J2, K2);
                                int IBC0 = ibcell(I2, J2, K2);
                                if (IBC0 <= 0) as(I, J, K, IU, M1) = FLWD(I1, J1, K1, IU, M1);
                                else if (IBC0 == 2) as(I, J, K, IU, M1) = FLW(I2, J2, K2, IU, M1);
                                else as(I, J, K, IU, M1) = ZERO;
                            }
                            a3(AP, I, J, K) = a3(AP, I, J, K) + as(I, J, K, IU, M1);
                        }
                }
    }
    // ---- minor species and soot (Initsv.f90:329-378, Msflow.f90, Gslv3m.f90,
    //      Sourcem.f90, Extr.f90:258-300, Intp.f90:348-420, Flx1d.f90:114-160) ----
    void minor_alloc() {   // allocate_ms (Setup.f90:904-929): zeros
        if (minor_on) return;
        GFMS.assign(7 * N, 0.0); SMF.assign(N, 0.0); BS_SOOT_PREV.assign(N, 0.0); SFP_SOOT_PREV.assign(N, 0.0);
        RRMS.assign(5L * MZ * NZ * LZ, 0.0);
        for (int l = 0; l <= 8; ++l) { resid_ms[l] = 1.0e-16; resid_ms_pre[l] = 1.0e-16; }
        minor_on = 1;
    }
    // INITSVM: a new start from the major species, or the restart state
    // (already in place) with the inlets reset and the exits extrapolated
    void INITSVM(int restart) {
        minor_alloc();
        if (!restart) {
            std::fill(SMF.begin(), SMF.end(), 0.0);
            std::fill(GFMS.begin(), GFMS.end(), 0.0);
            for (int I = 2; I <= MP; I += 2)
                for (int J = 2; J <= NP; J += 2)
                    for (int K = 2; K <= LP; K += 2) {
                        gfm(I, J, K, 1) = gf(I, J, K, IYF);
                        gfm(I, J, K, 2) = gf(I, J, K, IYO2);
                        gfm(I, J, K, 4) = gf(I, J, K, IYH2O);
                        gfm(I, J, K, 5) = gf(I, J, K, IYCO2);
                        gfm(I, J, K, 6) = gf(I, J, K, IYN2);
                    }
        } else {
            for (int I = 2; I <= MP; I += 2)
                for (int J = 2; J <= NP; J += 2)
                    for (int K = 2; K <= LP; K += 2) {
                        if (ibcell(I, J, K) != 2) continue;
                        gfm(I, J, K, 1) = gf(I, J, K, IYF);
                        gfm(I, J, K, 2) = gf(I, J, K, IYO2);
                        gfm(I, J, K, 4) = gf(I, J, K, IYH2O);
                        gfm(I, J, K, 5) = gf(I, J, K, IYCO2);
                        gfm(I, J, K, 6) = gf(I, J, K, IYN2);
                        gfm(I, J, K, 3) = ZERO;
                        gfm(I, J, K, 7) = ZERO;
                    }
            EXTRM();
        }
        IGS0 = 0;
        INTPM();
    }
    void EXTRM() {   // Extr.f90:258-300
        for (int i = 2; i <= MP; i += 2)
            for (int j = 2; j <= NP; j += 2)
                for (int k = 2; k <= LP; k += 2) {
                    if (ibcell(i, j, k) % 10 != 3) continue;
                    int i1, j1, k1, i2, j2, k2, ixd;
                    EXT01(false, i, j, k, i1, j1, k1, i2, j2, k2, ixd);
                    double f1, f2;
                    EXTR1(f1, f2, i, j, k, i1, j1, k1, i2, j2, k2, ixd);
                    for (int L = 1; L <= 7; ++L) {
                        double g0 = gfm(i1, j1, k1, L) * f1 + gfm(i2, j2, k2, L) * f2;
                        gfm(i, j, k, L) = fmax2(g0, ZERO);
                        const int jj = (j + j1) / 2;   // the y-face, whatever the exit's direction
                        gfm(i, jj, k, L) = gfm(i, j, k, L);
                    }
                    a3(SMF, i, j, k) = a3(SMF, i1, j1, k1);
                }
        for (int i = 2; i <= MP; i += 2)
            for (int j = 2; j <= NP; j += 2)
                for (int k = 2; k <= LP; k += 2) {
                    if (ibcell(i, j, k) % 10 != 1) continue;
                    int i1, j1, k1, i2, j2, k2, ixd;
                    EXT01(true, i, j, k, i1, j1, k1, i2, j2, k2, ixd);
                    for (int L = 1; L <= 7; ++L) {
                        gfm(i, j, k, L) = gfm(i1, j1, k1, L);
                        if (ixd == 1) gfm((i + i1) / 2, j, k, L) = gfm(i, j, k, L);
                        else if (ixd == 2) gfm(i, (j + j1) / 2, k, L) = gfm(i, j, k, L);
                        else gfm(i, j, (k + k1) / 2, L) = gfm(i, j, k, L);
                    }
                }
    }
    // INTP0M (Intp.f90:404-420): F1 is the caller's variable, as in INTP0
    void INTP0M(double& F1, int I, int J, int K, int I1, int J1, int K1, int I2, int J2, int K2) {
        if (ibcell(I, J, K) == 3) return;
        if (ibcell(I, J, K) == 2) {
            if (ibcell(I1, J1, K1) == 2 && ibcell(I2, J2, K2) == 0) F1 = ONE;
            else if (ibcell(I1, J1, K1) == 0 && ibcell(I2, J2, K2) == 2) F1 = ZERO;
        }
        const double F2 = ONE - F1;
        for (int L = 1; L <= 7; ++L) gfm(I, J, K, L) = F1 * gfm(I1, J1, K1, L) + F2 * gfm(I2, J2, K2, L);
    }
    void INTPM() {   // Intp.f90:348-400
        for (int I = 2; I <= MP; I += 2) {
            for (int K = 3; K <= LPM1; K += 2) {
                double F1 = INTP1(I, 0, K, 3);
                for (int J = 2; J <= NP; J += 2) {
                    if (ibcell(I, J, K) == 1) continue;
                    INTP0M(F1, I, J, K, I, J, K + 1, I, J, K - 1);
                }
            }
            for (int J = 3; J <= NPM1; J += 2) {
                double F1 = INTP1(I, J, 0, 2);
                for (int K = 2; K <= LP; ++K) {
                    if (ibcell(I, J, K) == 1) continue;
                    INTP0M(F1, I, J, K, I, J + 1, K, I, J - 1, K);
                }
            }
        }
        for (int I = 3; I <= MPM1; I += 2) {
            double F1 = INTP1(I, 0, 0, 1);
            for (int K = 2; K <= LP; ++K)
                for (int J = 2; J <= NP; ++J) {
                    if (ibcell(I, J, K) == 1) continue;
                    INTP0M(F1, I, J, K, I + 1, J, K, I - 1, J, K);
                }
        }
    }
    // FLX1DM (Flx1d.f90:114-160): species flow through the x-face plane I
    // (id 1: positive, 2: negative) or the y-face plane J
    double flxm(int I, int L, int id) {
        double s = ZERO;
        for (int j = 4; j <= NPM2; j += 2)
            for (int k = LKZ1; k <= LKZ2; k += 2) {
                if (ibcell(I, j, k) == 1) continue;
                const double g0 = a3(THETA, I, j, k) * a3(DNST, I, j, k) * ug(I, j, k, 1) * AREA_C(I, j, k, 1) * pr.gmfr;
                if ((g0 >= ZERO ? 1 : 2) == id) s = s + std::fabs(g0) * gfm(I, j, k, L);
            }
        return s;
    }
    double flym(int J, int L, int id) {
        double s = ZERO;
        for (int i = 4; i <= MPM2; i += 2)
            for (int k = LKZ1; k <= LKZ2; k += 2) {
                if (ibcell(i, J, k) == 1) continue;
                const double g0 = a3(THETA, i, J, k) * a3(DNST, i, J, k) * ug(i, J, k, 2) * AREA_C(i, J, k, 2) * pr.gmfr;
                if ((g0 >= ZERO ? 1 : 2) == id) s = s + std::fabs(g0) * gfm(i, J, k, L);
            }
        return s;
    }
    // SPIN (Gslv3m.f90:292-305): inflow of species LSP into the cell (kmol/s)
    double SPIN(int I, int J, int K, int LSP) {
        const double G11 = as(I, J, K, 1, 1) * gfm(I - 2, J, K, LSP), G12 = as(I, J, K, 1, 2) * gfm(I + 2, J, K, LSP);
        const double G21 = as(I, J, K, 2, 1) * gfm(I, J - 2, K, LSP), G22 = as(I, J, K, 2, 2) * gfm(I, J + 2, K, LSP);
        const double G31 = as(I, J, K, 3, 1) * gfm(I, J, K - 2, LSP), G32 = as(I, J, K, 3, 2) * gfm(I, J, K + 2, LSP);
        double FXMS = G11 + G12 + G21 + G22 + G31 + G32;
        return FXMS * pr.gmfr / WMS[LSP - 1];
    }
    // RR2 of GSLV3M keeps its value from cell to cell: a cell whose first
    // reaction is off subtracts the previous cell's last RR2 (its reaction 4
    // and 5 rate) from its O2 inflow.  It is kept from call to call here
    // (zero before the first), a local the reference leaves undefined there.
    double rr2_carry = 0.0;
    double soot_tot = 0, smf_max = 0, smf_max_noclip = 0, bal_ms = 0;
    void GSLV3M() {
        const int MI1 = 4, MI3 = MPM2, NJ1 = NJY1, NJ3 = NJY2, LK1 = LKZ1, LK3 = LKZ2;
        const double SML1 = 1.0e-25;
        // CK0_M, BETA, ODR, ERC (Var_mod.f90:231-235)
        const double CK0M[5] = {1.66e15, 7.94e14, 2.24e14, 7.94e22, 9.33e14};
        const double BETA5 = -0.5;
        const double ODR1[5] = {1.46, 1.6904, 1.0, 0.721, 1.0}, ODR2[5] = {0.5217, 1.57, 0.0, 4.0111, 0.5};
        const double ERC[5] = {20643.0, 11613.0, 62281.0, 44369.0, 68899.0};
        double RR2 = rr2_carry;
        for (int I = MI1; I <= MI3; I += 2)
            for (int J = NJ1; J <= NJ3; J += 2)
                for (int K = LK1; K <= LK3; K += 2) {
                    if (ibcell(I, J, K) > 0) continue;
                    const int ID2 = I / 2, JD2 = J / 2, KD2 = K / 2;
                    const double TMP = a3(T, I, J, K) * pr.t0;
                    const double DNST1 = a3(DNST, I, J, K) * pr.dnst0;
                    const double VOL = DX[I] * DR[J] * DZ[K] * 1.0;   // *VOL0
                    double G[8];
                    for (int L = 1; L <= 7; ++L) G[L] = gfm(I, J, K, L) / WMS[L - 1] * DNST1;
                    // reaction 1
                    const double FXMS1 = SPIN(I, J, K, 1);
                    double FXMS2 = SPIN(I, J, K, 2);
                    if (G[1] <= SML1 || G[2] <= SML1) {
                        rrms(ID2, JD2, KD2, 1) = 0;
                    } else {
                        const double RR1 = std::pow(G[1], ODR1[0]) * std::pow(G[2], ODR2[0]);
                        RR2 = CK0M[0] * RR1 * std::exp(-ERC[0] / TMP) * VOL;
                        if (RR2 > FXMS1) RR2 = FXMS1;
                        if (FXMS2 / 1.5 < RR2) RR2 = FXMS2 / 1.5;
                        rrms(ID2, JD2, KD2, 1) = RR2 * 0.3 + rrms(ID2, JD2, KD2, 1) * 0.7;
                    }
                    // reaction 2
                    FXMS2 = FXMS2 - RR2 * 1.5;
                    if (FXMS2 > small20 && G[3] > small20) {
                        const double RR1 = std::pow(G[3], ODR1[1]) * std::pow(G[2], ODR2[1]);
                        RR2 = CK0M[1] * RR1 * std::exp(-ERC[1] / TMP) * VOL;
                        if (FXMS2 * 2 < RR2) RR2 = FXMS2 * 2;
                        const double FXMS3 = SPIN(I, J, K, 3);
                        RR2 = fmin2(RR2, FXMS3);
                    } else {
                        RR2 = 0;
                    }
                    // reaction 3
                    double RR3;
                    if (G[5] > small20) {
                        const double RR1 = std::pow(G[5], ODR1[2]);
                        RR3 = CK0M[2] * RR1 * std::exp(-ERC[2] / TMP) * VOL;
                        const double FXMS5 = SPIN(I, J, K, 5);
                        RR3 = fmin2(RR3, FXMS5);
                    } else {
                        RR3 = 0;
                    }
                    double RR1 = RR2 - RR3;
                    if (RR1 < 0) RR1 = 0;
                    rrms(ID2, JD2, KD2, 2) = RR1 * 0.3 + rrms(ID2, JD2, KD2, 2) * 0.7;
                    // reactions 4 and 5
                    if (G[2] > small20 && G[3] > small20 && G[6] > small20) {
                        const double R1 = std::pow(G[3], ODR1[3]) * std::pow(G[2], ODR2[3]) * gfm(I, J, K, 6) / 0.725;
                        RR2 = CK0M[3] * R1 * std::exp(-ERC[3] / TMP) * VOL;
                    } else {
                        RR2 = 0;
                    }
                    if (G[2] > small20 && G[6] > small20) {
                        const double R1 = std::pow(G[6], ODR1[4]) * std::pow(G[2], ODR2[4]);
                        RR3 = CK0M[4] * R1 * std::exp(-ERC[4] / TMP) * std::pow(TMP, BETA5);
                        RR3 = RR3 * VOL;
                    } else {
                        RR3 = 0;
                    }
                    RR2 = RR2 + RR3;
                    rrms(ID2, JD2, KD2, 4) = RR2;
                }
        rr2_carry = RR2;
        // the seven species (Gslv3m.f90:131-192)
        for (int L = 1; L <= 7; ++L) {
            for (int I = 2; I <= MP; I += 2)
                for (int J = 2; J <= NP; J += 2)
                    for (int K = 2; K <= LP; K += 2) a3(FZ, I, J, K) = gfm(I, J, K, L);
            SOURCEM(L, MI1, MI3, NJ1, NJ3, LK1, LK3);
            SGM = pr.ssigma;
            if (IGS0 == 0) {
                GSLV3G0(MI1, MI3, NJ1, NJ3, LK1, LK3, 0);
                AP1 = AP;
                IGS0 = 1;
            } else {
                AP = AP1;
            }
            const double RFM = pr.rfm, RFMC = ONE - pr.rfm;
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        if (ibcell(I, J, K) >= 1) continue;
                        const double VOL = VOL_C(I, J, K);
                        a3(AP, I, J, K) = a3(AP, I, J, K) - (a3(SFP, I, J, K) * VOL);
                        a3(AP, I, J, K) = a3(AP, I, J, K) / RFM;
                        a3(BS, I, J, K) = a3(BS, I, J, K) + RFMC * a3(FZ, I, J, K) * a3(AP, I, J, K);
                    }
            resid_ms_pre[L] = calc_residual(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3);
            ADLBL3(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3, pr.ntimesm);
            resid_ms[L] = calc_residual(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3);
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        if (ibcell(I, J, K) >= 1) continue;
                        double& z = a3(FZ, I, J, K);
                        if (z > ONE) z = ONE;
                        if (z < 0) z = 0;
                        if (L == 3 && z > 0.1) z = 0.1;
                        if (L == 7 && z > 1.0e-2) z = 1.0e-2;
                        gfm(I, J, K, L) = RFMC * gfm(I, J, K, L) + RFM * z;
                        if (gfm(I, J, K, L) < small20) gfm(I, J, K, L) = 0;
                    }
        }
        // mass balance of the species (Gslv3m.f90:196-218)
        double vol_tot = ZERO;
        for (int i = 2; i <= MP; i += 2)
            for (int j = 2; j <= NP; j += 2)
                for (int k = 2; k <= LP; k += 2)
                    if (ibcell(i, j, k) == 0) vol_tot = vol_tot + VOL_C(i, j, k) * 1.0;
        bal_ms = 0;
        for (int I = MI1; I <= MI3; I += 2)
            for (int J = NJ1; J <= NJ3; J += 2)
                for (int K = LK1; K <= LK3; K += 2) {
                    if (ibcell(I, J, K) >= 1) continue;
                    double G0 = ZERO;
                    for (int L = 1; L <= 7; ++L) G0 = G0 + gfm(I, J, K, L);
                    bal_ms = bal_ms + std::fabs(ONE - G0) * VOL_C(I, J, K);
                }
        bal_ms = bal_ms * 1.0 / vol_tot;
        // soot (Gslv3m.f90:225-284)
        if (!pr.react) return;
        const int L = 8;
        for (int I = 2; I <= MP; I += 2)
            for (int J = 2; J <= NP; J += 2)
                for (int K = 2; K <= LP; K += 2) a3(FZ, I, J, K) = a3(SMF, I, J, K);
        SOURCEM(11, MI1, MI3, NJ1, NJ3, LK1, LK3);
        SGM = pr.ssigma;
        GSLV3G0(MI1, MI3, NJ1, NJ3, LK1, LK3, 1);
        const double RFM = pr.rfm_soot, RFMC = ONE - pr.rfm_soot;
        for (int I = MI1; I <= MI3; I += 2)
            for (int J = NJ1; J <= NJ3; J += 2)
                for (int K = LK1; K <= LK3; K += 2) {
                    if (ibcell(I, J, K) >= 1) continue;
                    const double VOL = VOL_C(I, J, K);
                    a3(BS, I, J, K) = a3(BS, I, J, K) * VOL;
                    a3(AP, I, J, K) = a3(AP, I, J, K) - (a3(SFP, I, J, K) * VOL);
                    a3(AP, I, J, K) = a3(AP, I, J, K) / RFM;
                    a3(BS, I, J, K) = a3(BS, I, J, K) + RFMC * a3(FZ, I, J, K) * a3(AP, I, J, K);
                }
        resid_ms_pre[L] = calc_residual(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3);
        ADLBL3(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3, pr.ntimesm);
        resid_ms[L] = calc_residual(FZ, MI1, MI3, NJ1, NJ3, LK1, LK3);
        soot_tot = 0; smf_max = ZERO; smf_max_noclip = ZERO;
        for (int I = MI1; I <= MI3; I += 2)
            for (int J = NJ1; J <= NJ3; J += 2)
                for (int K = LK1; K <= LK3; K += 2) {
                    if (ibcell(I, J, K) >= 1) continue;
                    const double z = a3(FZ, I, J, K);
                    smf_max_noclip = std::max(smf_max_noclip, z);
                    double G0;
                    if (z > pr.soot_cap) G0 = pr.soot_cap;
                    else if (z > small20) G0 = z;
                    else G0 = ZERO;
                    smf_max = std::max(smf_max, G0);
                    a3(SMF, I, J, K) = RFM * G0 + RFMC * a3(SMF, I, J, K);
                    const double vol = DX[I] * DR[J] * DZ[K];
                    soot_tot = soot_tot + a3(SMF, I, J, K) * a3(DNST, I, J, K) * pr.dnst0 * vol;
                }
    }
    // SOURCEM (Sourcem.f90:8-122): NELM 1..7 the species, 11 soot (the
    // current soot model, ioldsoot = 0)
    void SOURCEM(int NELM, int MI1, int MI3, int NJ1, int NJ3, int LK1, int LK3) {
        if (NELM != 11) {
            for (int I = MI1; I <= MI3; I += 2)
                for (int J = NJ1; J <= NJ3; J += 2)
                    for (int K = LK1; K <= LK3; K += 2) {
                        a3(SFP, I, J, K) = ZERO;
                        a3(BS, I, J, K) = ZERO;
                        if (ibcell(I, J, K) > 0) continue;
                        const int ID2 = I / 2, JD2 = J / 2, KD2 = K / 2;
                        double G0;
                        if (NELM == 1) G0 = -rrms(ID2, JD2, KD2, 1);
                        else if (NELM == 2)
                            G0 = -rrms(ID2, JD2, KD2, 1) * 1.5 - rrms(ID2, JD2, KD2, 2) * 0.5 - rrms(ID2, JD2, KD2, 4);
                        else if (NELM == 3) G0 = rrms(ID2, JD2, KD2, 1) - rrms(ID2, JD2, KD2, 2);
                        else if (NELM == 4) G0 = rrms(ID2, JD2, KD2, 1) * TWO;
                        else if (NELM == 5) G0 = rrms(ID2, JD2, KD2, 2);
                        else if (NELM == 6) G0 = -rrms(ID2, JD2, KD2, 4);
                        else G0 = rrms(ID2, JD2, KD2, 4) * TWO;
                        a3(BS, I, J, K) = G0 * WMS[NELM - 1] / pr.gmfr;
                    }
            return;
        }
        const double snorm = pr.r0 / (pr.dnst0 * pr.ug0);
        const double E0_sf = pr.t0_sf < small20 ? ZERO : std::exp(-pr.esf_r / pr.t0_sf);
        const double E0_so = pr.t0_so < small20 ? ZERO : std::sqrt(pr.t0_so) * std::exp(-pr.eso_r / pr.t0_so);
        std::fill(BS.begin(), BS.end(), ZERO);
        std::fill(SFP.begin(), SFP.end(), ZERO);
        for (int i = MI1; i <= MI3; i += 2)
            for (int j = NJ1; j <= NJ3; j += 2)
                for (int k = LK1; k <= LK3; k += 2) {
                    const double Tcell = a3(T, i, j, k) * pr.t0;
                    if (ibcell(i, j, k) > 0 || !pr.react) continue;
                    if (Tcell > pr.t0_sf) {
                        a3(BS, i, j, k) = pr.aform * gfm(i, j, k, 1) * (std::exp(-pr.esf_r / Tcell) - E0_sf) * snorm;
                        if (itr_ms > 1)
                            a3(BS, i, j, k) = pr.rf_soot_form * a3(BS, i, j, k) + (ONE - pr.rf_soot_form) * a3(BS_SOOT_PREV, i, j, k);
                    }
                    if (Tcell > pr.t0_so) {
                        a3(SFP, i, j, k) = -pr.aoxid * gfm(i, j, k, 2) * (std::sqrt(Tcell) * std::exp(-pr.eso_r / Tcell) - E0_so) * snorm;
                        if (itr_ms > 1)
                            a3(SFP, i, j, k) = pr.rf_soot_oxid * a3(SFP, i, j, k) + (ONE - pr.rf_soot_oxid) * a3(SFP_SOOT_PREV, i, j, k);
                    }
                }
        BS_SOOT_PREV = BS;
        SFP_SOOT_PREV = SFP;
    }
    // MSFLOW (Msflow.f90:29-165); returns the iterations done
    int MSFLOW(int maxms, double* gfm_out, double& svf_r) {
        IGS0 = 0;
        int done = 0;
        for (int L1 = 1; L1 <= maxms; ++L1) {
            itr_ms = itr_ms + 1;
            ++done;
            GSLV3M();
            for (int L = 1; L <= 7; ++L)
                gfm_out[L - 1] = flxm(5, L, 2) + flxm(MP - 3, L, 1) + flym(5, L, 2) + flym(NP - 3, L, 1);
            double G1 = 0;
            svf_r = 0;
            for (int I = 2; I <= MP; I += 2)
                for (int J = 2; J <= NP; J += 2)
                    for (int K = 2; K <= LP; K += 2) {
                        if (ibcell(I, J, K) != 3) continue;
                        double G0 = AREA_C(I, J, K, 3);
                        if (G0 < small20) G0 = AREA_C(I, J, K, 2);
                        if (G0 < small20) G0 = AREA_C(I, J, K, 1);
                        G1 = G1 + G0;
                        svf_r = svf_r + a3(SMF, I, J, K) * a3(DNST, I, J, K) * pr.dnst0 / DNST_SOOT * G0;
                    }
            svf_r = svf_r / G1;
            imscon = 0;
            if (itr_ms > 10) {
                imscon = 1;
                for (int l = 1; l <= 8; ++l) if (resid_ms[l] > pr.bmcon) imscon = 0;
            }
            if (imscon == 1) break;
            EXTRM();
            INTPM();
        }
        return done;
    }

    void props(double G0) {   // Gflow.f90:302-382
        for (int I = 2; I <= MP; I += 2)
            for (int J = 2; J <= NP; J += 2)
                for (int K = 2; K <= LP; K += 2) {
                    if (ibcell(I, J, K) >= 1) continue;
                    CONC(I, J, K);
                    enth_to_T_at(I, J, K);
                    if (a3(T, I, J, K) > pr.t_mx) { a3(T, I, J, K) = pr.t_mx; T_to_enth_at(I, J, K); }
                    else if (a3(T, I, J, K) < pr.t_mn) { a3(T, I, J, K) = pr.t_mn; T_to_enth_at(I, J, K); }
                    a3(P, I, J, K) = a3(P, I, J, K) - G0;
                    BOUND(a3(P, I, J, K), 0, 1);
                    dnst_calc(I, J, K);
                    THER(I, J, K);
                }
    }
    void T_ave_calc() {   // Utility.f90:1485-1510
        double tave = 0, rho_vol_tot = 0;
        for (int k = 4; k <= LP - 2; k += 2)
            for (int j = 4; j <= NP - 2; j += 2)
                for (int i = 4; i <= MP - 2; i += 2) {
                    if (ibcell(i, j, k) != 0) continue;
                    double vol = VOL_C(i, j, k);
                    tave = tave + a3(T, i, j, k) * a3(DNST, i, j, k) * vol;
                    rho_vol_tot = rho_vol_tot + a3(DNST, i, j, k) * vol;
                }
        Tave = tave * pr.t0 / rho_vol_tot;
    }
    void rad_qe_only() {   // Rad_emis.f90:411-466 with RAD0 (Rad0.f90:112-157); gray bands or RAD_GAS
        std::vector<double> qe2(QE.size(), 0.0);
        for (auto& t : T) t = t * pr.t0;
        double SGN = pr.sig * pr.ri * pr.ri;
        std::vector<double> DEB0(NWL), DEB(NWL);
        for (int l = 0; l < NWL; ++l) DEB0[l] = pr.hck / pr.ri / WL[l];
        RadGas rg;
        rg.init(NWL, WL.data());
        for (int I = 2; I <= MP; I += 2)
            for (int J = 2; J <= NP; J += 2)
                for (int K = 2; K <= LP; K += 2) {
                    double T_RAD = a3(T, I, J, K);
                    if (!(ibcell(I, J, K) <= 0 && T_RAD >= 300.0)) continue;
                    if (pr.gas_model) rad_gas_inputs(rg, I, J, K, T_RAD);
                    double VOL = VOL_C(I, J, K);
                    double SA = ((DX[I] * DR[J]) + (DR[J] * DZ[K]) + (DX[I] * DZ[K])) * TWO;
                    if (SA <= small16) continue;
                    double OPL = 6.0 * VOL / SA;
                    if (OPL <= 1.0e-10) continue;
                    if (pr.gas_model) { rg.OPL = OPL; rg.RAD_GAS(); }
                    // DEBX (Rad_fun.f90:122-140)
                    double EB0 = 0;
                    for (int L = 1; L <= NWL - 1; ++L) {
                        double X1 = DEB0[L - 1] / T_RAD;
                        double EB1 = RIF3(X1);
                        DEB[L - 1] = EB1 - EB0;
                        if (DEB[L - 1] <= 1.0e-3) DEB[L - 1] = ZERO; else EB0 = EB1;
                    }
                    DEB[NWL - 1] = ONE - EB0;
                    double t2 = T_RAD * T_RAD;
                    double area_sgn_t4 = SA * SGN * (t2 * t2);
                    double sum = ZERO;
                    for (int l = 0; l < NWL; ++l) sum = sum + DEB[l] * EMF(pr.gas_model ? rg.AKL0[l + 1] : AKL0[l], OPL);
                    qe2[cix(I / 2, J / 2, K / 2)] = area_sgn_t4 * sum;
                }
        i1st_rad_qe_done = 1;
        for (auto& t : T) t = t / pr.t0;
        QE = qe2;
    }

    void gflow(int stop_after) {
        wall_functions();
        if (stop_after == GFO_STEP_WALLFN) return;
        eq_reset();
        GSLV3V_momasm();
        if (stop_after == GFO_STEP_MOMASM) return;
        GSLV3V_psolve();
        if (stop_after == GFO_STEP_PSOLVE) return;
        GSLV3V_momsolve();
        if (stop_after == GFO_STEP_MOMSOLVE) return;
        GSLV3V_pcorr();
        if (stop_after == GFO_STEP_PCORR) return;
        GSLV3V_velcorr();
        if (stop_after == GFO_STEP_VELCORR) return;
        GSLV3V_exits();
        if (stop_after == GFO_STEP_GSLV3V) return;
        double G0 = pref_g0();
        GSLV3G();
        if (stop_after == GFO_STEP_SCALARS) return;
        props(G0);
        T_ave_calc();
        if (stop_after == GFO_STEP_PROPS) return;
        EXTR();
        INTP();
    }
    void eq_reset() {}

    void fill_stats(gfm_iter_stats* s, int converged) {
        if (!s) return;
        std::memset(s, 0, sizeof *s);
        s->itr_gas = itr_gas; s->converged = converged;
        s->res_mass = res_mass; s->res_mass_max = res_mass_max;
        s->p_resid_pre = p_resid_pre; s->p_resid = p_resid; s->pcorr_resid = pcorr_resid;
        for (int i = 0; i < 3; ++i) { s->u_resid_pre[i] = u_resid_pre[i]; s->u_resid[i] = u_resid[i]; }
        for (int i = 0; i < 10; ++i) { s->gf_resid_pre[i] = gf_resid_pre[i]; s->gf_resid[i] = gf_resid[i]; }
        s->factor = FACTOR; s->gfin = GFIN; s->gfex = GFEX;
        s->q_react = q_react; s->q_exhaust = q_exhaust; s->q_conv_total = qconv_total;
        double q_in_tot = q_react + q_h_in, q_out_tot = q_exhaust;
        s->q_global_bal = std::fabs((q_in_tot - q_out_tot) / q_in_tot);
        s->tave = Tave; s->tmean_ex = Tmean_ex;
    }
};

// ---------------------------------------------------------------------------
// Volume radiation transfer, restated from
//   RAD_EMIS   Rad_emis.f90:144-189  wall markers with open neighbours, T*T0
//   RAD0       Rad0.f90:112-166      AKL = EMF(AKL0, OPL) (ID_RAD=10), totals
//   QRNF       Qrn.f90:58-229        emitter loop (emission/absorption part)
//   QREF       Qre.f90:31-515        per emitter: x, y and z fluxes
//   QRTX/Y/Z   Qrtx.f90:15-209, Qrty.f90:9-224, Qrtz.f90:15-234
//   QRN1       Qrn.f90:244-275       QA = sum over bands of QAL
// and the unmarking and T/T0 of Rad_emis.f90:364-377.  The wall exchange that
// QRNF runs afterwards (wall_q_amb, wallq, qrn2) is not part of this.
// ---------------------------------------------------------------------------

// atan(x) in degrees (the Fortran intrinsic ATAND).  Own implementation, the
// same operations as the GPU kernel's: |x| > 1 is reduced by
// atan(x) = pi/2 - atan(1/x), then a > tan(pi/12) by
// atan(a) = pi/6 + atan((a*sqrt(3) - 1)/(a + sqrt(3))) (Abramowitz & Stegun
// 4.4.34 with tan(pi/6) = 1/sqrt(3)), and the reduced argument t goes through
// the Maclaurin series atan(t) = sum_{n=0}^{14} (-1)^n t^(2n+1)/(2n+1)
// (A&S 4.4.42), Horner's rule in t^2 with fused multiply-adds.
double ATAND(double x) {
    const double PI = 3.14159265358979323846;
    const double SQRT3 = 1.73205080756887729353;
    const double TAN_PI_12 = 0.26794919243112270647;
    double a = std::fabs(x);
    const bool inv = a > 1.0;
    if (inv) a = 1.0 / a;
    const bool sh = a > TAN_PI_12;
    if (sh) a = (a * SQRT3 - 1.0) / (a + SQRT3);
    const double z = a * a;
    double p = 1.0 / 29.0;
    for (int n = 13; n >= 0; --n) p = std::fma(p, z, ((n & 1) ? -1.0 : 1.0) / (double)(2 * n + 1));
    double r = a * p;
    if (sh) r = PI / 6.0 + r;
    if (inv) r = PI / 2.0 - r;
    const double d = r * (180.0 / PI);
    return x < 0.0 ? -d : d;
}

struct RadVolume {
    Oracle& o;
    int MP, NP, LP, MZ, NZ, LZ, NWL;
    long NC;
    std::vector<int> IBR;            // IBCELL with the wall markers, one value per cell (even positions)
    vec AKL, QAL, QEL;               // (MZ,NZ,LZ,NWL)
    vec DEB, DEB0, QEL0, QEL1, Q11, Q12;
    double ANG0[4];
    vec ANG1, ANG2, ANG3;            // ANG1(MP,2), ANG2(NP,2), ANG3(LP,2), 1-based
    int DA, DB;                      // extents of the slab arrays of the current direction
    vec QTX1, QTX2, Q2M;
    std::vector<char> IQT1, IQTM, IQT2;
    double SGN, TG_MN;
    double qa_sum_to_melt = 0, qa_sum_to_exit = 0, qa_sum_to_inlet = 0, qa_sum_to_wall = 0, qa_sum_to_open = 0;
    double qe_sum_from_open = 0, tot_qe_h2o_co2 = 0, tot_qe_soot = 0;
    double qa_sum_bnd, qa_sum_vol, c_melt, c_exit, c_inlet, c_wall, c_open;
    int n_emit = 0;

    explicit RadVolume(Oracle& oo) : o(oo) {
        MP = o.MP; NP = o.NP; LP = o.LP; MZ = o.MZ; NZ = o.NZ; LZ = o.LZ; NWL = o.NWL;
        NC = (long)MZ * NZ * LZ;
        DEB.assign(NWL + 1, 0.0); DEB0.assign(NWL + 1, 0.0); QEL0.assign(NWL + 1, 0.0); QEL1.assign(NWL + 1, 0.0);
        Q11.assign(NWL + 1, 0.0); Q12.assign(NWL + 1, 0.0);
        ANG1.assign(2 * (MP + 2), 0.0); ANG2.assign(2 * (NP + 2), 0.0); ANG3.assign(2 * (LP + 2), 0.0);
    }
    long cell(int id2, int jd2, int kd2) const { return (long)(id2 - 1) + (long)MZ * ((long)(jd2 - 1) + (long)NZ * (kd2 - 1)); }
    int ibr(int i, int j, int k) const { return IBR[cell(i / 2, j / 2, k / 2)]; }
    double& akl(int id2, int jd2, int kd2, int l) { return AKL[cell(id2, jd2, kd2) + (long)(l - 1) * NC]; }
    double& qal(int id2, int jd2, int kd2, int l) { return QAL[cell(id2, jd2, kd2) + (long)(l - 1) * NC]; }
    double& qel(int id2, int jd2, int kd2, int l) { return QEL[cell(id2, jd2, kd2) + (long)(l - 1) * NC]; }
    double& ang1(int i, int c) { return ANG1[(c - 1) * (MP + 2) + i]; }
    double& ang2(int j, int c) { return ANG2[(c - 1) * (NP + 2) + j]; }
    double& ang3(int k, int c) { return ANG3[(c - 1) * (LP + 2) + k]; }
    double& qtx1(int a, int b, int l) { return QTX1[((long)(l - 1) * DB + (b - 1)) * DA + (a - 1)]; }
    double& qtx2(int a, int b, int l) { return QTX2[((long)(l - 1) * DB + (b - 1)) * DA + (a - 1)]; }
    double& q2m(int a, int b, int l) { return Q2M[((long)(l - 1) * DB + (b - 1)) * DA + (a - 1)]; }
    char& iqt1(int a, int b) { return IQT1[(long)(b - 1) * DA + (a - 1)]; }
    char& iqtm(int a, int b) { return IQTM[(long)(b - 1) * DA + (a - 1)]; }
    char& iqt2(int a, int b) { return IQT2[(long)(b - 1) * DA + (a - 1)]; }
    double X(int i) const { return o.X[i]; }
    double R(int j) const { return o.R[j]; }
    double Z(int k) const { return o.Z[k]; }
    static double T4(double t) { double t2 = t * t; return t2 * t2; }

    void alloc_slab(int da, int db) {   // ALLOCATE + zero/.TRUE. at the start of a direction
        DA = da; DB = db;
        QTX1.assign((long)DA * DB * NWL, 0.0); QTX2.assign((long)DA * DB * NWL, 0.0); Q2M.assign((long)DA * DB * NWL, 0.0);
        IQT1.assign((long)DA * DB, 1); IQTM.assign((long)DA * DB, 1); IQT2.assign((long)DA * DB, 1);
    }
    void DEBX(double TG0) {   // Rad_fun.f90:83-101
        double EB0 = 0;
        for (int L = 1; L <= NWL - 1; ++L) {
            double X1 = DEB0[L] / TG0;
            double EB1 = RIF3(X1);
            DEB[L] = EB1 - EB0;
            if (DEB[L] <= 1.0e-3) DEB[L] = ZERO; else EB0 = EB1;
        }
        DEB[NWL] = ONE - EB0;
    }
    // absorption of the power arriving at one slab cell (the loop bodies of
    // Qre.f90:185-219 / 336-369 / 486-522); a, b index the slab arrays
    void absorb(int I, int J, int K, int a, int b, bool end) {
        if (iqt2(a, b)) return;
        const int ID2 = I / 2, JD2 = J / 2, KD2 = K / 2;
        for (int L = 1; L <= NWL; ++L) {
            if (qtx2(a, b, L) < small16) continue;
            const int ib = ibr(I, J, K);
            if (ib >= 1 || end) {
                qal(ID2, JD2, KD2, L) = qal(ID2, JD2, KD2, L) + qtx2(a, b, L);
                qa_sum_bnd = qa_sum_bnd + qtx2(a, b, L);
                if (ib == 4) c_melt = c_melt + qtx2(a, b, L);
                else if (ib == 3) c_exit = c_exit + qtx2(a, b, L);
                else if (ib == 2) c_inlet = c_inlet + qtx2(a, b, L);
                else c_wall = c_wall + qtx2(a, b, L);
            } else {
                double QA0 = qtx2(a, b, L) * akl(ID2, JD2, KD2, L);
                qal(ID2, JD2, KD2, L) = qal(ID2, JD2, KD2, L) + QA0;
                qtx1(a, b, L) = qtx2(a, b, L) - QA0;
                iqt1(a, b) = 0;
                qa_sum_vol = qa_sum_vol + QA0;
                c_open = c_open + QA0;
            }
            qtx2(a, b, L) = 0;
            iqt2(a, b) = 1;
        }
    }

    // ---- QRTX (Qrtx.f90:15-209) ----------------------------------------------
    void QRTX(int I0, int J0, int K0, int I10, int I1) {
        int J2 = 0;   // the spread's DO variable, as the corner branch reads it (J1 == J0 never occurs in a box)
        int I2 = I1 + (I1 - I10) / 2;
        I2 = std::min(I2, MP);
        for (int JM = -1; JM <= 1; JM += 2) {
            const int JEND = JM < 0 ? 2 : NP;
            for (int JJ = J0 + JM; JM > 0 ? JJ <= JEND : JJ >= JEND; JJ += JM * 2) {
                double a2;
                double b = std::fabs(X(I2) - X(I0));
                if (b < small16) a2 = 90; else a2 = ATAND(std::fabs(R(JJ) - R(J0)) / b);
                if (a2 >= ANG0[2]) break;
                ang2(JJ, 2) = a2;
            }
        }
        for (int KM = -1; KM <= 1; KM += 2) {
            const int KEND = KM < 0 ? 2 : LP;
            for (int KK = K0 + KM; KM > 0 ? KK <= KEND : KK >= KEND; KK += KM * 2) {
                double a3;
                double b = std::fabs(X(I2) - X(I0));
                if (b < small16) a3 = 90; else a3 = ATAND(std::fabs(Z(KK) - Z(K0)) / b);
                if (a3 >= ANG0[3]) break;
                ang3(KK, 2) = a3;
            }
        }
        for (int K1 = 4; K1 <= LP - 2; K1 += 2) {
            if (K1 < K0 && ang3(K1 + 1, 2) >= ANG0[3]) continue;
            if (K1 > K0 && ang3(K1 - 1, 2) >= ANG0[3]) break;
            const int KD2 = K1 / 2;
            for (int JPM = -2; JPM <= 2; JPM += 4) {
                double A11 = 0, A12 = 0;
                const int JEND = JPM < 0 ? 2 : NP;
                for (int J1 = J0; JPM > 0 ? J1 <= JEND - JPM : J1 >= JEND - JPM; J1 += JPM) {
                    if (A11 >= ANG0[2]) break;
                    const int J12 = J1 + JPM / 2;
                    A12 = ang2(J12, 1);
                    const double DANG = A12 - A11;
                    if (DANG <= 1.0e-10) { A11 = A12; continue; }
                    double A21 = A11;
                    const int J1D2 = J1 / 2;
                    if (iqt1(J1D2, KD2)) { A11 = A12; continue; }
                    if (J1 == J0) {
                        for (int L = 1; L <= NWL; ++L) Q11[L] = qtx1(J1D2, KD2, L) * HALF;
                        if (JPM > 0) for (int L = 1; L <= NWL; ++L) qtx1(J1D2, KD2, L) = ZERO;
                    } else {
                        for (int L = 1; L <= NWL; ++L) { Q11[L] = qtx1(J1D2, KD2, L); qtx1(J1D2, KD2, L) = ZERO; }
                    }
                    if (J1 != J0 || JPM > 0) iqt1(J1D2, KD2) = 1;
                    for (int L = 1; L <= NWL; ++L) Q12[L] = Q11[L];
                    for (J2 = J1; JPM > 0 ? J2 <= JEND : J2 >= JEND; J2 += JPM) {
                        const int J2D2 = J2 / 2;
                        if (ibr(I1, J2, K1) < 1) {
                            const int J2M = J2 + JPM / 2;
                            const double A22 = ang2(J2M, 2);
                            if (A22 <= A21) continue;
                            if (A22 < A12) {
                                const double FIJ = (A22 - A21) / DANG;
                                for (int L = 1; L <= NWL; ++L) {
                                    if (Q11[L] < small16) continue;
                                    double Q21 = Q11[L] * FIJ;
                                    q2m(J2D2, KD2, L) = q2m(J2D2, KD2, L) + Q21;
                                    Q12[L] = Q12[L] - Q21;
                                }
                                iqtm(J2D2, KD2) = 0;
                                A21 = A22;
                                continue;
                            }
                        }
                        for (int L = 1; L <= NWL; ++L) q2m(J2D2, KD2, L) = q2m(J2D2, KD2, L) + Q12[L];
                        iqtm(J2D2, KD2) = 0;
                        break;
                    }
                    A11 = A12;
                }
            }
        }
        for (int J1 = 2; J1 <= NP; J1 += 2) {
            if (J1 < J0 && ang2(J1 + 1, 2) >= ANG0[2]) continue;
            if (J1 > J0 && ang2(J1 - 1, 2) >= ANG0[2]) break;
            const int JD2 = J1 / 2;
            for (int KM = -2; KM <= 2; KM += 4) {
                double A11 = 0, A12 = 0;
                const int KEND = KM < 0 ? 2 : LP;
                for (int K1 = K0; KM > 0 ? K1 <= KEND - KM : K1 >= KEND - KM; K1 += KM) {
                    if (A11 >= ANG0[3]) break;
                    const int K12 = K1 + KM / 2;
                    A12 = ang3(K12, 1);
                    const double DANG = A12 - A11;
                    if (DANG <= 1.0e-10) { A11 = A12; continue; }
                    double A21 = A11;
                    const int KD2 = K1 / 2;
                    if (iqtm(JD2, KD2)) { A11 = A12; continue; }
                    if (K1 == K0) {
                        for (int L = 1; L <= NWL; ++L) Q11[L] = q2m(JD2, KD2, L) * HALF;
                        if (KM > 0) for (int L = 1; L <= NWL; ++L) q2m(JD2, KD2, L) = ZERO;
                    } else {
                        for (int L = 1; L <= NWL; ++L) { Q11[L] = q2m(JD2, KD2, L); q2m(JD2, KD2, L) = ZERO; }
                    }
                    if (K1 != K0 || KM > 0) iqtm(JD2, KD2) = 1;
                    const int IBC1 = ibr(I1, J1, K1);
                    if (IBC1 == 101 || IBC1 == 111 || IBC1 == 4) {
                        for (int L = 1; L <= NWL; ++L) qtx2(JD2, KD2, L) = qtx2(JD2, KD2, L) + Q11[L];
                        iqt2(JD2, KD2) = 0;
                        A11 = A12;
                        continue;
                    }
                    for (int L = 1; L <= NWL; ++L) Q12[L] = Q11[L];
                    for (int K2 = K1; KM > 0 ? K2 <= KEND : K2 >= KEND; K2 += KM) {
                        const int K2M = K2 + KM / 2, K2D2 = K2 / 2;
                        const int IBC2 = ibr(I1, J1, K2);
                        bool to330 = IBC1 <= 0 && IBC2 >= 1;
                        if (!to330) {
                            if (IBC1 > 100 && IBC2 == 1) {
                                if (J1 < J0) J2 = J1 + 2; else if (J1 > J0) J2 = J1 - 2;
                                const int J2D2 = J2 / 2, K2D2M = K2D2 - KM / 2;
                                for (int L = 1; L <= NWL; ++L) {
                                    if (Q12[L] < small16) continue;
                                    double Q21 = Q12[L] * HALF;
                                    qtx2(J2D2, K2D2, L) = qtx2(J2D2, K2D2, L) + Q21;
                                    qtx2(JD2, K2D2M, L) = qtx2(JD2, K2D2M, L) + Q21;
                                }
                                iqt2(J2D2, K2D2) = 0;
                                iqt2(JD2, K2D2M) = 0;
                                break;
                            }
                            if (K2M > LP || K2M < 2) to330 = true;
                            else {
                                const double A22 = ang3(K2M, 2);
                                if ((A22 - A21) <= 1.0e-10) continue;
                                if (A22 < A12) {
                                    const double FIJ = (A22 - A21) / DANG;
                                    for (int L = 1; L <= NWL; ++L) {
                                        if (Q11[L] < small16) continue;
                                        double Q21 = Q11[L] * FIJ;
                                        qtx2(JD2, K2D2, L) = qtx2(JD2, K2D2, L) + Q21;
                                        Q12[L] = Q12[L] - Q21;
                                    }
                                    iqt2(JD2, K2D2) = 0;
                                    A21 = A22;
                                    continue;
                                }
                            }
                        }
                        for (int L = 1; L <= NWL; ++L) qtx2(JD2, K2D2, L) = qtx2(JD2, K2D2, L) + Q12[L];
                        iqt2(JD2, K2D2) = 0;
                        break;
                    }
                    A11 = A12;
                }
            }
        }
    }

    // ---- QRTY (Qrty.f90:9-224) -------------------------------------------------
    void QRTY(int I0, int J0, int K0, int J10, int J1) {
        int I2 = 0;   // the spread's DO variable, as the corner branch reads it (I1 == I0 never occurs in a box)
        int J2 = J1 + (J1 - J10) / 2;
        J2 = std::min(J2, NP);
        for (int IM = -1; IM <= 1; IM += 2) {
            const int IEND = IM < 0 ? 2 : MP;
            for (int II = I0 + IM; IM > 0 ? II <= IEND : II >= IEND; II += IM * 2) {
                double a1;
                double b = std::fabs(R(J2) - R(J0));
                if (b < small16) a1 = 90; else a1 = ATAND(std::fabs(X(II) - X(I0)) / b);
                if (a1 >= ANG0[1]) break;
                ang1(II, 2) = a1;
            }
        }
        for (int KM = -1; KM <= 1; KM += 2) {
            const int KEND = KM < 0 ? 2 : LP;
            for (int KK = K0 + KM; KM > 0 ? KK <= KEND : KK >= KEND; KK += KM * 2) {
                double a3;
                double b = std::fabs(R(J2) - R(J0));
                if (b < small16) a3 = 90; else a3 = ATAND(std::fabs(Z(KK) - Z(K0)) / b);
                if (a3 >= ANG0[3]) break;
                ang3(KK, 2) = a3;
            }
        }
        for (int K1 = 4; K1 <= LP - 2; K1 += 2) {
            if (K1 < K0 && ang3(K1 + 1, 2) >= ANG0[3]) continue;
            if (K1 > K0 && ang3(K1 - 1, 2) >= ANG0[3]) break;
            const int KD2 = K1 / 2;
            for (int IPM = -2; IPM <= 2; IPM += 4) {
                double A11 = 0, A12 = 0;
                const int IEND = IPM < 0 ? 2 : MP;
                for (int I1 = I0; IPM > 0 ? I1 <= IEND - IPM : I1 >= IEND - IPM; I1 += IPM) {
                    if (A11 >= ANG0[1]) break;
                    const int I12 = I1 + IPM / 2;
                    A12 = ang1(I12, 1);
                    const double DANG = A12 - A11;
                    if (DANG <= 1.0e-10) { A11 = A12; continue; }
                    double A21 = A11;
                    const int I1D2 = I1 / 2;
                    if (iqt1(I1D2, KD2)) { A11 = A12; continue; }
                    if (I1 == I0) {
                        for (int L = 1; L <= NWL; ++L) Q11[L] = qtx1(I1D2, KD2, L) * HALF;
                        if (IPM > 0) for (int L = 1; L <= NWL; ++L) qtx1(I1D2, KD2, L) = ZERO;
                    } else {
                        for (int L = 1; L <= NWL; ++L) { Q11[L] = qtx1(I1D2, KD2, L); qtx1(I1D2, KD2, L) = ZERO; }
                    }
                    if (I1 != I0 || IPM > 0) iqt1(I1D2, KD2) = 1;
                    for (int L = 1; L <= NWL; ++L) Q12[L] = Q11[L];
                    for (I2 = I1; IPM > 0 ? I2 <= IEND : I2 >= IEND; I2 += IPM) {
                        const int I2D2 = I2 / 2;
                        if (ibr(I2, J1, K1) < 1) {
                            const int I2M = I2 + IPM / 2;
                            const double A22 = ang1(I2M, 2);
                            if (A22 <= A21) continue;
                            if (A22 < A12) {
                                const double FIJ = (A22 - A21) / DANG;
                                for (int L = 1; L <= NWL; ++L) {
                                    if (Q11[L] < small16) continue;
                                    double Q21 = Q11[L] * FIJ;
                                    q2m(I2D2, KD2, L) = q2m(I2D2, KD2, L) + Q21;
                                    Q12[L] = Q12[L] - Q21;
                                }
                                iqtm(I2D2, KD2) = 0;
                                A21 = A22;
                                continue;
                            }
                        }
                        for (int L = 1; L <= NWL; ++L) q2m(I2D2, KD2, L) = q2m(I2D2, KD2, L) + Q12[L];
                        iqtm(I2D2, KD2) = 0;
                        break;
                    }
                    A11 = A12;
                }
            }
        }
        for (int I1 = 2; I1 <= MP; I1 += 2) {
            if (I1 < I0 && ang1(I1 + 1, 2) >= ANG0[1]) continue;
            if (I1 > I0 && ang1(I1 - 1, 2) >= ANG0[1]) break;
            const int ID2 = I1 / 2;
            for (int KM = -2; KM <= 2; KM += 4) {
                double A11 = 0, A12 = 0;
                const int KEND = KM < 0 ? 2 : LP;
                for (int K1 = K0; KM > 0 ? K1 <= KEND - KM : K1 >= KEND - KM; K1 += KM) {
                    if (A11 >= ANG0[3]) break;
                    const int K12 = K1 + KM / 2;
                    A12 = ang3(K12, 1);
                    const double DANG = A12 - A11;
                    if (DANG <= 1.0e-10) { A11 = A12; continue; }
                    double A21 = A11;
                    const int KD2 = K1 / 2;
                    if (iqtm(ID2, KD2)) { A11 = A12; continue; }
                    if (K1 == K0) {
                        for (int L = 1; L <= NWL; ++L) Q11[L] = q2m(ID2, KD2, L) * HALF;
                        if (KM > 0) for (int L = 1; L <= NWL; ++L) q2m(ID2, KD2, L) = ZERO;
                    } else {
                        for (int L = 1; L <= NWL; ++L) { Q11[L] = q2m(ID2, KD2, L); q2m(ID2, KD2, L) = ZERO; }
                    }
                    if (K1 != K0 || KM > 0) iqtm(ID2, KD2) = 1;
                    const int IBC1 = ibr(I1, J1, K1);
                    if (IBC1 == 201 || IBC1 == 211 || IBC1 == 4) {
                        for (int L = 1; L <= NWL; ++L) qtx2(ID2, KD2, L) = qtx2(ID2, KD2, L) + Q11[L];
                        iqt2(ID2, KD2) = 0;
                        A11 = A12;
                        continue;
                    }
                    for (int L = 1; L <= NWL; ++L) Q12[L] = Q11[L];
                    for (int K2 = K1; KM > 0 ? K2 <= KEND : K2 >= KEND; K2 += KM) {
                        const int K2M = K2 + KM / 2, K2D2 = K2 / 2;
                        const int IBC2 = ibr(I1, J1, K2);
                        bool to330 = IBC1 <= 0 && IBC2 >= 1;
                        if (!to330) {
                            if (IBC1 >= 100 && IBC2 == 1) {
                                if (I1 < I0) I2 = I1 + 2; else if (I1 > I0) I2 = I1 - 2;
                                const int I2D2 = I2 / 2, K2D2M = K2D2 - KM / 2;
                                for (int L = 1; L <= NWL; ++L) {
                                    if (Q12[L] < small16) continue;
                                    double Q21 = Q12[L] * HALF;
                                    qtx2(I2D2, K2D2, L) = qtx2(I2D2, K2D2, L) + Q21;
                                    qtx2(ID2, K2D2M, L) = qtx2(ID2, K2D2M, L) + Q21;
                                }
                                iqt2(I2D2, K2D2) = 0;
                                iqt2(ID2, K2D2M) = 0;
                                break;
                            }
                            if (K2M > LP || K2M < 2) to330 = true;
                            else {
                                const double A22 = ang3(K2M, 2);
                                if ((A22 - A21) <= 1.0e-10) continue;
                                if (A22 < A12) {
                                    const double FIJ = (A22 - A21) / DANG;
                                    for (int L = 1; L <= NWL; ++L) {
                                        if (Q11[L] < small16) continue;
                                        double Q21 = Q11[L] * FIJ;
                                        qtx2(ID2, K2D2, L) = qtx2(ID2, K2D2, L) + Q21;
                                        Q12[L] = Q12[L] - Q21;
                                    }
                                    iqt2(ID2, K2D2) = 0;
                                    A21 = A22;
                                    continue;
                                }
                            }
                        }
                        for (int L = 1; L <= NWL; ++L) qtx2(ID2, K2D2, L) = qtx2(ID2, K2D2, L) + Q12[L];
                        iqt2(ID2, K2D2) = 0;
                        break;
                    }
                    A11 = A12;
                }
            }
        }
    }

    // ---- QRTZ (Qrtz.f90:15-234) -------------------------------------------------
    void QRTZ(int I0, int J0, int K0, int K10, int K1) {
        int I2 = 0;   // the spread's DO variable, as the corner branch reads it (I1 == I0 never occurs in a box)
        int K2 = K1 + (K1 - K10) / 2;
        K2 = std::min(K2, LP);
        for (int IM = -1; IM <= 1; IM += 2) {
            const int IEND = IM < 0 ? 2 : MP;
            for (int II = I0 + IM; IM > 0 ? II <= IEND : II >= IEND; II += IM * 2) {
                double a1;
                double b = std::fabs(Z(K2) - Z(K0));
                if (b < small16) a1 = 90; else a1 = ATAND(std::fabs(X(II) - X(I0)) / b);
                if (a1 >= ANG0[1]) break;
                ang1(II, 2) = a1;
            }
        }
        for (int JM = -1; JM <= 1; JM += 2) {
            const int JEND = JM < 0 ? 2 : NP;
            for (int JJ = J0 + JM; JM > 0 ? JJ <= JEND : JJ >= JEND; JJ += JM * 2) {
                double a2;
                double b = std::fabs(Z(K2) - Z(K0));
                if (b < small16) a2 = 90; else a2 = ATAND(std::fabs(R(JJ) - R(J0)) / b);
                if (a2 >= ANG0[2]) break;
                ang2(JJ, 2) = a2;
            }
        }
        for (int J1 = 4; J1 <= NP - 2; J1 += 2) {
            if (J1 < J0 && ang2(J1 + 1, 2) >= ANG0[2]) continue;
            if (J1 > J0 && ang2(J1 - 1, 2) >= ANG0[2]) break;
            const int JD2 = J1 / 2;
            for (int IPM = -2; IPM <= 2; IPM += 4) {
                double A11 = 0, A12 = 0;
                const int IEND = IPM < 0 ? 2 : MP;
                for (int I1 = I0; IPM > 0 ? I1 <= IEND - IPM : I1 >= IEND - IPM; I1 += IPM) {
                    if (A11 >= ANG0[1]) break;
                    const int I12 = I1 + IPM / 2;
                    A12 = ang1(I12, 1);
                    const double DANG = A12 - A11;
                    if (DANG <= 1.0e-10) { A11 = A12; continue; }
                    double A21 = A11;
                    const int I1D2 = I1 / 2;
                    if (iqt1(I1D2, JD2)) { A11 = A12; continue; }
                    if (I1 == I0) {
                        for (int L = 1; L <= NWL; ++L) Q11[L] = qtx1(I1D2, JD2, L) * HALF;
                        if (IPM > 0) for (int L = 1; L <= NWL; ++L) qtx1(I1D2, JD2, L) = ZERO;
                    } else {
                        for (int L = 1; L <= NWL; ++L) { Q11[L] = qtx1(I1D2, JD2, L); qtx1(I1D2, JD2, L) = ZERO; }
                    }
                    if (I1 != I0 || IPM > 0) iqt1(I1D2, JD2) = 1;
                    for (int L = 1; L <= NWL; ++L) Q12[L] = Q11[L];
                    for (I2 = I1; IPM > 0 ? I2 <= IEND : I2 >= IEND; I2 += IPM) {
                        const int I2D2 = I2 / 2;
                        if (ibr(I2, J1, K1) < 1) {
                            const int I2M = I2 + IPM / 2;
                            const double A22 = ang1(I2M, 2);
                            if (A22 <= A21) continue;
                            if (A22 < A12) {
                                const double FIJ = (A22 - A21) / DANG;
                                for (int L = 1; L <= NWL; ++L) {
                                    if (Q11[L] < small16) continue;
                                    double Q21 = Q11[L] * FIJ;
                                    q2m(I2D2, JD2, L) = q2m(I2D2, JD2, L) + Q21;
                                    Q12[L] = Q12[L] - Q21;
                                }
                                iqtm(I2D2, JD2) = 0;
                                A21 = A22;
                                continue;
                            }
                        }
                        for (int L = 1; L <= NWL; ++L) q2m(I2D2, JD2, L) = q2m(I2D2, JD2, L) + Q12[L];
                        iqtm(I2D2, JD2) = 0;
                        break;
                    }
                    A11 = A12;
                }
            }
        }
        for (int I1 = 2; I1 <= MP; I1 += 2) {
            if (I1 < I0 && ang1(I1 + 1, 2) >= ANG0[1]) continue;
            if (I1 > I0 && ang1(I1 - 1, 2) >= ANG0[1]) break;
            const int ID2 = I1 / 2;
            for (int JM = -2; JM <= 2; JM += 4) {
                double A11 = 0, A12 = 0;
                const int JEND = JM < 0 ? 2 : NP;
                for (int J1 = J0; JM > 0 ? J1 <= JEND - JM : J1 >= JEND - JM; J1 += JM) {
                    if (A11 >= ANG0[2]) break;
                    const int J12 = J1 + JM / 2;
                    A12 = ang2(J12, 1);
                    const double DANG = A12 - A11;
                    if (DANG <= 1.0e-10) { A11 = A12; continue; }
                    double A21 = A11;
                    const int JD2 = J1 / 2;
                    if (iqtm(ID2, JD2)) { A11 = A12; continue; }
                    if (J1 == J0) {
                        for (int L = 1; L <= NWL; ++L) Q11[L] = q2m(ID2, JD2, L) * HALF;
                        if (JM > 0) for (int L = 1; L <= NWL; ++L) q2m(ID2, JD2, L) = ZERO;
                    } else {
                        for (int L = 1; L <= NWL; ++L) { Q11[L] = q2m(ID2, JD2, L); q2m(ID2, JD2, L) = ZERO; }
                    }
                    if (J1 != J0 || JM > 0) iqtm(ID2, JD2) = 1;
                    const int IBC1 = ibr(I1, J1, K1);
                    if (IBC1 == 301 || IBC1 == 311 || IBC1 == 4) {
                        for (int L = 1; L <= NWL; ++L) qtx2(ID2, JD2, L) = qtx2(ID2, JD2, L) + Q11[L];
                        iqt2(ID2, JD2) = 0;
                        A11 = A12;
                        continue;
                    }
                    for (int L = 1; L <= NWL; ++L) Q12[L] = Q11[L];
                    for (int J2 = J1; JM > 0 ? J2 <= JEND : J2 >= JEND; J2 += JM) {
                        const int J2M = J2 + JM / 2, J2D2 = J2 / 2;
                        const int IBC2 = ibr(I1, J2, K1);
                        bool to330 = IBC1 <= 0 && IBC2 >= 1;
                        if (!to330) {
                            if (IBC1 > 1 && IBC2 == 1) {
                                if (I1 < I0) I2 = I1 + 2; else if (I1 > I0) I2 = I1 - 2;
                                const int I2D2 = I2 / 2, J2D2M = J2D2 - JM / 2;
                                for (int L = 1; L <= NWL; ++L) {
                                    if (Q12[L] < small16) continue;
                                    double Q21 = Q12[L] * HALF;
                                    qtx2(I2D2, J2D2, L) = qtx2(I2D2, J2D2, L) + Q21;
                                    qtx2(ID2, J2D2M, L) = qtx2(ID2, J2D2M, L) + Q21;
                                }
                                iqt2(I2D2, J2D2) = 0;
                                iqt2(ID2, J2D2M) = 0;
                                break;
                            }
                            if (J2M > NP || J2M < 2) to330 = true;
                            else {
                                const double A22 = ang2(J2M, 2);
                                if ((A22 - A21) <= 1.0e-10) continue;
                                if (A22 < A12) {
                                    const double FIJ = (A22 - A21) / DANG;
                                    for (int L = 1; L <= NWL; ++L) {
                                        if (Q11[L] < small16) continue;
                                        double Q21 = Q11[L] * FIJ;
                                        qtx2(ID2, J2D2, L) = qtx2(ID2, J2D2, L) + Q21;
                                        Q12[L] = Q12[L] - Q21;
                                    }
                                    iqt2(ID2, J2D2) = 0;
                                    A21 = A22;
                                    continue;
                                }
                            }
                        }
                        for (int L = 1; L <= NWL; ++L) qtx2(ID2, J2D2, L) = qtx2(ID2, J2D2, L) + Q12[L];
                        iqt2(ID2, J2D2) = 0;
                        break;
                    }
                    A11 = A12;
                }
            }
        }
    }

    // ---- QREF (Qre.f90:31-515); ANG0 follows SANG1 for an open cell -----------
    void QREF(int I0, int J0, int K0) {
        qa_sum_bnd = qa_sum_vol = 0;
        c_melt = c_exit = c_inlet = c_wall = c_open = 0;
        const int I0D2 = I0 / 2, J0D2 = J0 / 2, K0D2 = K0 / 2;
        for (int L = 1; L <= NWL; ++L) qel(I0D2, J0D2, K0D2, L) = ZERO;
        if (ibr(I0, J0, K0) >= 1) return;
        const double G0 = SGN * T4(o.a3(o.T, I0, J0, K0));
        for (int L = 1; L <= NWL; ++L) QEL0[L] = DEB[L] * akl(I0D2, J0D2, K0D2, L) * G0;

        // x-flux
        for (int L = 1; L <= NWL; ++L) QEL1[L] = QEL0[L] * o.DR[J0] * o.DZ[K0];
        alloc_slab(NZ, LZ);
        for (int IPM = -2; IPM <= 2; IPM += 4) {
            for (int L = 1; L <= NWL; ++L) qtx1(J0D2, K0D2, L) = QEL1[L];
            iqt1(J0D2, K0D2) = 0;
            for (int L = 1; L <= NWL; ++L) qel(I0D2, J0D2, K0D2, L) = qel(I0D2, J0D2, K0D2, L) + QEL1[L];
            {
                const int i1 = I0 + IPM / 2, j1 = J0 + IPM / 2, k1 = K0 + IPM / 2;
                ANG0[1] = 0;
                double b = std::fabs(X(i1) - X(I0));
                if (b < small16) { ANG0[2] = 90; ANG0[3] = 90; }
                else { ANG0[2] = ATAND(std::fabs(R(j1) - R(J0)) / b); ANG0[3] = ATAND(std::fabs(Z(k1) - Z(K0)) / b); }
            }
            for (int j = 1; j <= NP; ++j) { ang2(j, 1) = ANG0[2]; ang2(j, 2) = ANG0[2]; }
            ang2(J0, 1) = ang2(J0, 2) = ZERO;
            for (int k = 1; k <= LP; ++k) { ang3(k, 1) = ANG0[3]; ang3(k, 2) = ANG0[3]; }
            ang3(K0, 1) = ang3(K0, 2) = ZERO;
            const int IEND = IPM < 0 ? 2 : MP;
            for (int I = I0 + IPM; IPM > 0 ? I <= IEND : I >= IEND; I += IPM) {
                QRTX(I0, J0, K0, I - IPM, I);
                for (int J = 2; J <= NP; J += 2)
                    for (int K = 2; K <= LP; K += 2) absorb(I, J, K, J / 2, K / 2, I == IEND);
                for (int j = 1; j <= NP; ++j) ang2(j, 1) = ang2(j, 2);
                for (int k = 1; k <= LP; ++k) ang3(k, 1) = ang3(k, 2);
            }
        }
        // y-flux
        for (int L = 1; L <= NWL; ++L) QEL1[L] = QEL0[L] * o.DX[I0] * o.DZ[K0];
        alloc_slab(MZ, LZ);
        for (int JPM = -2; JPM <= 2; JPM += 4) {
            for (int L = 1; L <= NWL; ++L) qtx1(I0D2, K0D2, L) = QEL1[L];
            iqt1(I0D2, K0D2) = 0;
            for (int L = 1; L <= NWL; ++L) qel(I0D2, J0D2, K0D2, L) = qel(I0D2, J0D2, K0D2, L) + QEL1[L];
            {
                const int i1 = I0 + JPM / 2, j1 = J0 + JPM / 2, k1 = K0 + JPM / 2;
                ANG0[2] = 0;
                double b = std::fabs(R(j1) - R(J0));
                if (b < small16) { ANG0[1] = 90; ANG0[3] = 90; }
                else { ANG0[1] = ATAND(std::fabs(X(i1) - X(I0)) / b); ANG0[3] = ATAND(std::fabs(Z(k1) - Z(K0)) / b); }
            }
            for (int i = 1; i <= MP; ++i) { ang1(i, 1) = ANG0[1]; ang1(i, 2) = ANG0[1]; }
            ang1(I0, 1) = ang1(I0, 2) = ZERO;
            for (int k = 1; k <= LP; ++k) { ang3(k, 1) = ANG0[3]; ang3(k, 2) = ANG0[3]; }
            ang3(K0, 1) = ang3(K0, 2) = ZERO;
            const int JEND = JPM < 0 ? 2 : NP;
            for (int J = J0 + JPM; JPM > 0 ? J <= JEND : J >= JEND; J += JPM) {
                QRTY(I0, J0, K0, J - JPM, J);
                for (int I = 2; I <= MP; I += 2)
                    for (int K = 2; K <= LP; K += 2) absorb(I, J, K, I / 2, K / 2, J == JEND);
                for (int i = 1; i <= MP; ++i) ang1(i, 1) = ang1(i, 2);
                for (int k = 1; k <= LP; ++k) ang3(k, 1) = ang3(k, 2);
            }
        }
        // z-flux
        for (int L = 1; L <= NWL; ++L) QEL1[L] = QEL0[L] * o.DX[I0] * o.DR[J0];
        alloc_slab(MZ, NZ);
        for (int KPM = -2; KPM <= 2; KPM += 4) {
            for (int L = 1; L <= NWL; ++L) qtx1(I0D2, J0D2, L) = QEL1[L];
            iqt1(I0D2, J0D2) = 0;
            for (int L = 1; L <= NWL; ++L) qel(I0D2, J0D2, K0D2, L) = qel(I0D2, J0D2, K0D2, L) + QEL1[L];
            {
                const int i1 = I0 + KPM / 2, j1 = J0 + KPM / 2, k1 = K0 + KPM / 2;
                ANG0[3] = 0;
                double b = std::fabs(Z(k1) - Z(K0));
                if (b < small16) { ANG0[1] = 90; ANG0[2] = 90; }
                else { ANG0[1] = ATAND(std::fabs(X(i1) - X(I0)) / b); ANG0[2] = ATAND(std::fabs(R(j1) - R(J0)) / b); }
            }
            for (int i = 1; i <= MP; ++i) { ang1(i, 1) = ANG0[1]; ang1(i, 2) = ANG0[1]; }
            ang1(I0, 1) = ang1(I0, 2) = ZERO;
            for (int j = 1; j <= NP; ++j) { ang2(j, 1) = ANG0[2]; ang2(j, 2) = ANG0[2]; }
            ang2(J0, 1) = ang2(J0, 2) = ZERO;
            const int KEND = KPM < 0 ? 2 : LP;
            for (int K = K0 + KPM; KPM > 0 ? K <= KEND : K >= KEND; K += KPM) {
                QRTZ(I0, J0, K0, K - KPM, K);
                for (int I = 2; I <= MP; I += 2)
                    for (int J = 2; J <= NP; J += 2) absorb(I, J, K, I / 2, J / 2, K == KEND);
                for (int i = 1; i <= MP; ++i) ang1(i, 1) = ang1(i, 2);
                for (int j = 1; j <= NP; ++j) ang2(j, 1) = ang2(j, 2);
            }
        }
        double qe = qel(I0D2, J0D2, K0D2, 1);
        for (int L = 2; L <= NWL; ++L) qe = qe + qel(I0D2, J0D2, K0D2, L);
        o.QE[o.cix(I0D2, J0D2, K0D2)] = qe;
        qe_sum_from_open = qe_sum_from_open + qe;
    }

    void run() {
        // wall markers (Rad_emis.f90:144-178) on a copy of IBCELL's cell values
        IBR.assign(NC, 0);
        for (int I = 2; I <= MP; I += 2)
            for (int J = 2; J <= NP; J += 2)
                for (int K = 2; K <= LP; K += 2) IBR[cell(I / 2, J / 2, K / 2)] = o.ibcell(I, J, K);
        for (int I = 2; I <= MP; I += 2)
            for (int J = 2; J <= NP; J += 2)
                for (int K = 2; K <= LP; K += 2) {
                    if (ibr(I, J, K) != 1) continue;
                    const int KM2 = std::max(K - 2, 2), KP2 = std::min(K + 2, LP);
                    const int JM2 = std::max(J - 2, 2), JP2 = std::min(J + 2, NP);
                    const int IM2 = std::max(I - 2, 2), IP2 = std::min(I + 2, MP);
                    int& m = IBR[cell(I / 2, J / 2, K / 2)];
                    if (ibr(I, J, KM2) <= 0) m = 301;
                    else if (ibr(I, J, KP2) <= 0) m = 311;
                    else if (ibr(I, JM2, K) <= 0) m = 201;
                    else if (ibr(I, JP2, K) <= 0) m = 211;
                    else if (ibr(IM2, J, K) <= 0) m = 101;
                    else if (ibr(IP2, J, K) <= 0) m = 111;
                }
        for (auto& t : o.T) t = t * o.pr.t0;
        if (o.wall_on) o.wall_start();
        // RAD0 (Rad0.f90:22-42, 112-166): RAD_GAS and SOOTA on the minor
        // species, or gray bands (AKLG = AKL0, AKLS = 0)
        SGN = o.pr.sig * o.pr.ri * o.pr.ri;
        for (int L = 1; L <= NWL; ++L) DEB0[L] = o.pr.hck / o.pr.ri / o.WL[L - 1];
        TG_MN = 300;
        AKL.assign(NC * NWL, 0.0);
        RadGas rg;
        rg.init(NWL, o.WL.data());
        for (int I = 2; I <= MP; I += 2)
            for (int J = 2; J <= NP; J += 2)
                for (int K = 2; K <= LP; K += 2) {
                    const double T_RAD = o.a3(o.T, I, J, K);
                    if (!(ibr(I, J, K) <= 0 && T_RAD >= TG_MN)) continue;   // walls: emissivities, used only by the wall exchange
                    if (o.pr.gas_model) o.rad_gas_inputs(rg, I, J, K, T_RAD);
                    const double VOL = o.VOL_C(I, J, K);
                    const double SA = ((o.DX[I] * o.DR[J]) + (o.DR[J] * o.DZ[K]) + (o.DX[I] * o.DZ[K])) * TWO;
                    if (SA <= small16) continue;
                    const double OPL = 6.0 * VOL / SA;
                    if (OPL <= 1.0e-10) continue;
                    if (o.pr.gas_model) { rg.OPL = OPL; rg.RAD_GAS(); }
                    DEBX(T_RAD);
                    const double area_sgn_t4 = SA * SGN * T4(T_RAD);
                    double sg = ZERO, ss = ZERO;
                    for (int L = 1; L <= NWL; ++L) {
                        const double a0 = o.pr.gas_model ? rg.AKL0[L] : o.AKL0[L - 1];
                        const double ag = o.pr.gas_model ? rg.AKLG[L] : o.AKL0[L - 1];
                        const double as = o.pr.gas_model ? rg.AKLS[L] : ZERO;
                        akl(I / 2, J / 2, K / 2, L) = EMF(a0, OPL);
                        sg = sg + DEB[L] * EMF(ag, OPL);
                        ss = ss + DEB[L] * EMF(as, OPL);
                    }
                    tot_qe_h2o_co2 = tot_qe_h2o_co2 + (area_sgn_t4 * sg);
                    tot_qe_soot = tot_qe_soot + (area_sgn_t4 * ss);
                }
        // QRNF (Qrn.f90:58-154)
        std::fill(o.QE.begin(), o.QE.end(), 0.0);
        std::fill(o.QA.begin(), o.QA.end(), 0.0);
        QEL.assign(NC * NWL, 0.0);
        QAL.assign(NC * NWL, 0.0);
        for (int I = 2; I <= MP; I += 2)
            for (int J = 2; J <= NP; J += 2)
                for (int K = 2; K <= LP; K += 2) {
                    if (ibr(I, J, K) >= 1) continue;
                    if (o.a3(o.T, I, J, K) <= TG_MN) continue;
                    DEBX(o.a3(o.T, I, J, K));
                    QREF(I, J, K);
                    ++n_emit;
                    qa_sum_to_melt = qa_sum_to_melt + c_melt;
                    qa_sum_to_exit = qa_sum_to_exit + c_exit;
                    qa_sum_to_inlet = qa_sum_to_inlet + c_inlet;
                    qa_sum_to_wall = qa_sum_to_wall + c_wall;
                    qa_sum_to_open = qa_sum_to_open + c_open;
                }
        // QRN1 (Qrn.f90:250-259): QA of every cell
        for (int I = 2; I <= MP; I += 2)
            for (int J = 2; J <= NP; J += 2)
                for (int K = 2; K <= LP; K += 2) {
                    double G0 = 0;
                    for (int L = 1; L <= NWL; ++L) G0 = G0 + qal(I / 2, J / 2, K / 2, L);
                    o.QA[o.cix(I / 2, J / 2, K / 2)] = G0;
                }
        // the wall exchange of QRNF (Qrn.f90:209-211); qrn2 rebuilds QA as above
        if (o.wall_on) {
            o.wall_q_amb();
            o.wallq();
        }
        for (auto& t : o.T) t = t / o.pr.t0;
        o.i1st_rad_qe_done = 1;
        if (o.wall_on) o.i1st_rad_done = 1;
    }
};

void copy_in(vec& dst, const double* src, long n) { dst.assign(src, src + n); }
vec one_based(const double* src, int n) {
    vec v(n + 3, 0.0);
    for (int i = 0; i < n; ++i) v[i + 1] = src[i];
    return v;
}

}  // namespace

extern "C" {

void* gfo_create(const gfm_grid* g, const gfm_params* p, const gfm_fields* f) {
    if (!g || !p || !f) return nullptr;
    Oracle* o = new Oracle();
    o->MP = g->mp; o->NP = g->np; o->LP = g->lp;
    o->MPM1 = o->MP - 1; o->MPM2 = o->MP - 2; o->NPM1 = o->NP - 1; o->NPM2 = o->NP - 2; o->LPM1 = o->LP - 1; o->LPM2 = o->LP - 2;
    o->MZ = o->MP / 2; o->NZ = o->NP / 2; o->LZ = o->LP / 2;
    o->N = (long)o->MP * o->NP * o->LP;
    // NP,LP >= 6 branch of GRID3 (Grid3.f90:142-156, 202-216)
    o->NJY1 = 4; o->NJY2 = o->NPM2; o->LKZ1 = 4; o->LKZ2 = o->LPM2;
    o->NJY1V[1] = 4; o->NJY2V[1] = o->NPM2; o->NJY1V[2] = 5; o->NJY2V[2] = o->NP - 3; o->NJY1V[3] = 4; o->NJY2V[3] = o->NPM2;
    o->LKZ1V[1] = 4; o->LKZ2V[1] = o->LPM2; o->LKZ1V[2] = 4; o->LKZ2V[2] = o->LPM2; o->LKZ1V[3] = 5; o->LKZ2V[3] = o->LP - 3;
    o->NCELLS = g->ncells; o->I_REF = g->i_ref; o->J_REF = g->j_ref; o->K_REF = g->k_ref; o->P_REF = g->p_ref;
    o->X = one_based(g->x, o->MP); o->DX = one_based(g->dx, o->MP);
    o->R = one_based(g->r, o->NP); o->DR = one_based(g->dr, o->NP); o->RS = one_based(g->rs, o->NP);
    o->Z = one_based(g->z, o->LP); o->DZ = one_based(g->dz, o->LP);
    o->IBC.assign(g->ibcell, g->ibcell + o->N);
    for (int b = 1; b <= 2; ++b) {
        o->BV_F[b] = g->bv_f[b - 1];
        for (int ixd = 1; ixd <= 3; ++ixd) o->BA_F[ixd][b] = g->ba_f[3 * (b - 1) + ixd - 1];
    }
    for (int i = 0; i < g->b_cnt; ++i) {
        o->b_typ.push_back(g->b_typ[i]); o->b_i.push_back(g->b_i[i]); o->b_j.push_back(g->b_j[i]); o->b_k.push_back(g->b_k[i]);
        o->b_orient.push_back(g->b_orient[i]); o->b_direct.push_back(g->b_direct[i]); o->b_T.push_back(g->b_t[i]);
    }
    o->q_conv.assign(g->b_cnt, 0.0);
    o->NR0 = g->nr0;
    copy_in(o->RTIM, g->rtim, g->nr0); copy_in(o->DELRT, g->delrt, g->nr0); copy_in(o->HRT, g->hrt, g->nr0);
    copy_in(o->DELR, g->delr, g->nr0); copy_in(o->TIMED, g->timed, g->nr0); copy_in(o->HRD, g->hrd, g->nr0);
    o->NWL = g->nwl; copy_in(o->WL, g->wl, g->nwl); copy_in(o->AKL0, g->akl0, g->nwl);
    o->pr = *p;
    for (int i = 0; i < 21; ++i) { o->RFC[i] = ONE - p->rf[i]; o->RFLC[i] = ONE - p->rfl[i]; }
    const long N = o->N;
    copy_in(o->P, f->p, N); copy_in(o->T, f->t, N); copy_in(o->DNST, f->dnst, N); copy_in(o->THETA, f->theta, N);
    copy_in(o->TMU, f->tmu, N); copy_in(o->GAMA, f->gama, N); copy_in(o->CRATE, f->crate, N); copy_in(o->HRATE, f->hrate, N);
    copy_in(o->bs_hprev, f->bs_hprev, N);
    copy_in(o->UG, f->ug, 3 * N); copy_in(o->GF, f->gf, 9 * N);
    long NCA = (long)o->MZ * o->NZ * o->LZ;
    copy_in(o->QA, f->qa, NCA); copy_in(o->QE, f->qe, NCA);
    o->GTE.assign(N, 0.0); o->FZ.assign(N, 0.0); o->BS.assign(N, 0.0); o->SFP.assign(N, 0.0); o->AP.assign(N, 0.0);
    o->AS.assign(6 * N, 0.0);
    o->itr_gas = f->itr_gas; o->do_rad_qe_only_cnt = f->do_rad_qe_only_cnt; o->i1st_rad_qe_done = f->i1st_rad_qe_done;
    o->FACTOR = f->factor; o->FADJ = f->fadj; o->GFIN0 = f->gfin0; o->q_h_in = f->q_h_in;
    o->GFIN = 0; o->GFEX = 0; o->SGM = ONE; o->NELG = 0;
    o->res_mass = o->res_mass_max = 0;
    o->p_resid_pre = o->p_resid = o->pcorr_resid = 0;
    for (int i = 0; i < 3; ++i) o->u_resid_pre[i] = o->u_resid[i] = 0;
    for (int i = 0; i < 10; ++i) o->gf_resid_pre[i] = o->gf_resid[i] = 0;
    o->q_react = o->q_exhaust = o->qconv_total = o->q_rad_vol_tot = o->Tmean_ex = o->Tave = 0;
    o->h_resid_pre = 0;
    return o;
}

void gfo_destroy(void* o) { delete static_cast<Oracle*>(o); }

int gfo_initsv(void* vo) {
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o) return GFM_E_ARG;
    o->INTPV();
    o->EXTR();
    o->INTP();
    return GFM_OK;
}

int gfo_gflow_steps(void* vo, int stop_after) {
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o) return GFM_E_ARG;
    o->itr_gas = o->itr_gas + 1;
    o->gflow(stop_after);
    return GFM_OK;
}

int gfo_gflow(void* vo, int n_iter, gfm_iter_stats* out, int* n_done) {
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o || n_iter < 0) return GFM_E_ARG;
    int done = 0, conv = 0;
    for (int it = 0; it < n_iter; ++it) {
        o->itr_gas = o->itr_gas + 1;
        o->gflow(GFO_STEP_ALL);
        ++done;
        if (o->res_mass < o->pr.bgcon) { conv = 1; break; }
        if (o->pr.rad_emission) {   // Sphase.f90:204-231 (emission only)
            o->do_rad_qe_only_cnt = o->do_rad_qe_only_cnt + 1;
            if (o->do_rad_qe_only_cnt >= o->pr.rad_qe_frequency && o->itr_gas > 50) {
                if (o->pr.gas_model && o->i1st_rad_qe_done == 0) {
                    // the first emission update runs INITSVM and MSFLOW(300) before it
                    double out[7], svf;
                    o->INITSVM(o->pr.irstypm != 0 && o->minor_from_host);
                    o->MSFLOW(300, out, svf);
                }
                if (o->pr.gas_model && !o->minor_on) return GFM_E_ARG;
                o->rad_qe_only();
                o->do_rad_qe_only_cnt = 0;
            }
        }
    }
    o->fill_stats(out, conv);
    if (n_done) *n_done = done;
    return GFM_OK;
}

int gfo_download(void* vo, gfm_fields* f) {
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o || !f) return GFM_E_ARG;
    const long N = o->N;
    auto cp = [](double* dst, const vec& src) { if (dst) std::memcpy(dst, src.data(), src.size() * sizeof(double)); };
    cp(f->p, o->P); cp(f->t, o->T); cp(f->dnst, o->DNST); cp(f->theta, o->THETA); cp(f->tmu, o->TMU);
    cp(f->gama, o->GAMA); cp(f->crate, o->CRATE); cp(f->hrate, o->HRATE); cp(f->bs_hprev, o->bs_hprev);
    cp(f->ug, o->UG); cp(f->gf, o->GF); cp(f->qa, o->QA); cp(f->qe, o->QE);
    (void)N;
    f->itr_gas = o->itr_gas; f->do_rad_qe_only_cnt = o->do_rad_qe_only_cnt; f->i1st_rad_qe_done = o->i1st_rad_qe_done;
    f->factor = o->FACTOR; f->fadj = o->FADJ; f->gfin0 = o->GFIN0; f->q_h_in = o->q_h_in;
    return GFM_OK;
}

long gfo_get_array(void* vo, const char* name, double* out, long cap) {
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o || !name || !out) return GFM_E_ARG;
    const vec* src = nullptr;
    long off = 0, n = o->N;
    std::string s(name);
    // per-patch arrays of the wall exchange
    const vec* patch_arr = s == "b_t" ? &o->b_T : s == "radiosity" ? &o->radiosity : s == "q_amb" ? &o->q_amb
                         : s == "q_conv" ? &o->q_conv : s == "qc" ? &o->qc : s == "qeb" ? &o->qeb : s == "emis" ? &o->emis
                         : s == "b_face_area" ? &o->b_face_area : s == "patch_area" ? &o->patch_area : nullptr;
    if (s == "qrs") {   // QRS at each melt patch's (b_i, b_j), 0 for the others
        const long nb = (long)o->b_typ.size();
        if (cap < nb) return GFM_E_ARG;
        for (long i = 0; i < nb; ++i)
            out[i] = o->b_typ[i] == 4 && !o->qrs.empty() ? o->qrs[(size_t)(o->b_i[i] - 1) + (size_t)o->MP * (o->b_j[i] - 1)] : 0.0;
        return nb;
    }
    if (patch_arr) {
        const long nb = (long)patch_arr->size();
        if (cap < nb) return GFM_E_ARG;
        std::memcpy(out, patch_arr->data(), nb * sizeof(double));
        return nb;
    }
    if (s == "ap") src = &o->AP; else if (s == "bs") src = &o->BS; else if (s == "sfp") src = &o->SFP;
    else if (s == "fz") src = &o->FZ; else if (s == "gte") src = &o->GTE; else if (s == "bs_hprev") src = &o->bs_hprev;
    else if (s.size() == 4 && s[0] == 'a' && s[1] == 's') {
        int l = s[2] - '0', m = s[3] - '0';
        if (l < 1 || l > 3 || m < 1 || m > 2) return GFM_E_ARG;
        src = &o->AS; off = (long)((l - 1) * 2 + (m - 1)) * o->N;
    } else return GFM_E_ARG;
    if (cap < n) return GFM_E_ARG;
    std::memcpy(out, src->data() + off, n * sizeof(double));
    return n;
}

static void load_system(Oracle* o, const double* ap, const double* const as[6], const double* bs) {
    o->AP.assign(ap, ap + o->N);
    o->BS.assign(bs, bs + o->N);
    for (int q = 0; q < 6; ++q) std::memcpy(o->AS.data() + (long)q * o->N, as[q], o->N * sizeof(double));
}

int gfo_adlbl3(void* vo, double* xt, const double* ap, const double* const as[6], const double* bs,
               int ib, int ie, int jb, int je, int kb, int ke, int nim) {
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o || !xt || !ap || !as || !bs) return GFM_E_ARG;
    load_system(o, ap, as, bs);
    vec X(xt, xt + o->N);
    o->ADLBL3(X, ib, ie, jb, je, kb, ke, nim);
    std::memcpy(xt, X.data(), o->N * sizeof(double));
    return GFM_OK;
}

double gfo_calc_residual(void* vo, const double* xt, const double* ap, const double* const as[6], const double* bs,
                         int ib, int ie, int jb, int je, int kb, int ke) {
    Oracle* o = static_cast<Oracle*>(vo);
    load_system(o, ap, as, bs);
    vec X(xt, xt + o->N);
    return o->calc_residual(X, ib, ie, jb, je, kb, ke);
}

double gfo_da(double d, double f) { return DA(d, f); }
double gfo_tgamf(double b) { return TGAMF(b); }
double gfo_emf(double xkl, double xl0) { return EMF(xkl, xl0); }
double gfo_atand(double x) { return ATAND(x); }

int gfo_rad_transfer(void* vo, gfm_rad_totals* out) {
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o || o->NWL < 1) return GFM_E_ARG;
    if (o->pr.gas_model && !o->minor_on) return GFM_E_ARG;
    RadVolume rv(*o);
    rv.run();
    if (out) {
        std::memset(out, 0, sizeof *out);
        out->qe_sum_from_open = rv.qe_sum_from_open;
        out->qa_sum_to_open = rv.qa_sum_to_open;
        out->qa_sum_to_wall = rv.qa_sum_to_wall;
        out->qa_sum_to_inlet = rv.qa_sum_to_inlet;
        out->qa_sum_to_exit = rv.qa_sum_to_exit;
        out->qa_sum_to_melt = rv.qa_sum_to_melt;
        out->tot_qe_h2o_co2 = rv.tot_qe_h2o_co2;
        out->tot_qe_soot = rv.tot_qe_soot;
        out->n_emitters = rv.n_emit;
    }
    return GFM_OK;
}
int gfo_wall_patch_list(void* vo, int* out, int cap) {
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o) return GFM_E_ARG;
    std::vector<int> pl;
    o->wall_patch_list(pl);
    const int n = (int)pl.size() / 6;
    if (out) {
        if (cap < n) return GFM_E_ARG;
        std::memcpy(out, pl.data(), pl.size() * sizeof(int));
    }
    return n;
}
int gfo_wall_setup(void* vo, const gfm_wall_spec* spec) {
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o || !spec) return GFM_E_ARG;
    if (spec->nex < 0 || spec->nex > GFM_MAX_EXHAUSTS) return GFM_E_ARG;
    // the patch list the case carries must be the one MAPB gives
    std::vector<int> pl;
    o->wall_patch_list(pl);
    if (pl.size() != 6 * o->b_typ.size()) return GFM_E_ARG;
    for (size_t n = 0; n < o->b_typ.size(); ++n) {
        const int v[6] = {o->b_typ[n], o->b_i[n], o->b_j[n], o->b_k[n], o->b_orient[n], o->b_direct[n]};
        for (int q = 0; q < 6; ++q) if (pl[6 * n + q] != v[q]) return GFM_E_ARG;
    }
    for (size_t n = 0; n < o->b_typ.size(); ++n)
        if (o->b_typ[n] == 3) {
            // every exit patch needs an exhaust entry (exh_type(b_exh) is read)
            o->wall_setup(*spec);
            for (size_t q = 0; q < o->b_typ.size(); ++q) if (o->b_typ[q] == 3 && o->b_exh[q] == 0) { o->wall_on = false; return GFM_E_ARG; }
            return GFM_OK;
        }
    o->wall_setup(*spec);
    return GFM_OK;
}
int gfo_wall_totals(void* vo, gfm_wall_totals* t) {
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o || !t || !o->wall_on) return GFM_E_ARG;
    std::memset(t, 0, sizeof *t);
    t->b_cnt = (int)o->b_typ.size();
    t->sweeps = o->iterw;
    t->outer = o->wall_outer;
    t->avg_wall_T = o->avg_wall_T; t->q_melt = o->q_melt; t->q_wall_loss = o->q_wall_loss;
    t->q_incident_total = o->q_incident_total; t->q_incident_wall = o->q_incident_wall;
    t->q_incident_inlet = o->q_incident_inlet; t->q_incident_exit = o->q_incident_exit;
    t->q_incident_melt = o->q_incident_melt; t->qconv_total = o->qconv_total;
    t->q_rad_inlet = o->q_rad_inlet; t->q_rad_outlet = o->q_rad_outlet;
    t->qm_flame = o->qm_flame; t->qm_bnds = o->qm_bnds; t->qm_conv = o->qm_conv;
    t->rel_rad_chg_mean = o->last_rel_rad_chg_mean;
    return GFM_OK;
}
int gfo_rad_emission(void* vo) {
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o || o->NWL < 1) return GFM_E_ARG;
    if (o->pr.gas_model && !o->minor_on) return GFM_E_ARG;
    o->rad_qe_only();
    return GFM_OK;
}

int gfo_minor_set(void* vo, const gfm_minor* m) {
    if (!vo || !m || !m->gfm || !m->smf || !m->bs_soot_prev || !m->sfp_soot_prev || !m->rrms) return GFM_E_ARG;
    Oracle* o = static_cast<Oracle*>(vo);
    const long NCA = (long)o->MZ * o->NZ * o->LZ;
    copy_in(o->GFMS, m->gfm, 7 * o->N);
    copy_in(o->SMF, m->smf, o->N);
    copy_in(o->BS_SOOT_PREV, m->bs_soot_prev, o->N);
    copy_in(o->SFP_SOOT_PREV, m->sfp_soot_prev, o->N);
    copy_in(o->RRMS, m->rrms, 5 * NCA);
    o->itr_ms = m->itr_ms;
    o->imscon = m->imscon;
    if (!o->minor_on) for (int l = 0; l <= 8; ++l) { o->resid_ms[l] = 1.0e-16; o->resid_ms_pre[l] = 1.0e-16; }
    o->minor_on = 1;
    o->minor_from_host = 1;
    return GFM_OK;
}
int gfo_initsvm(void* vo, int restart) {
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o || (restart && !o->minor_on)) return GFM_E_ARG;
    o->INITSVM(restart);
    return GFM_OK;
}
int gfo_msflow(void* vo, int maxms, gfm_msflow_stats* out) {
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o || maxms < 0 || !o->minor_on) return GFM_E_ARG;
    double g[7] = {0}, svf = 0;
    const int done = o->MSFLOW(maxms, g, svf);
    if (out) {
        std::memset(out, 0, sizeof *out);
        out->itr_ms = o->itr_ms;
        out->iterations = done;
        out->converged = o->imscon;
        for (int l = 0; l < 8; ++l) { out->resid_ms_pre[l] = o->resid_ms_pre[l + 1]; out->resid_ms[l] = o->resid_ms[l + 1]; }
        out->bal_ms = o->bal_ms;
        out->soot_tot = o->soot_tot;
        out->smf_max = o->smf_max;
        out->smf_max_noclip = o->smf_max_noclip;
        for (int l = 0; l < 7; ++l) out->gfm_out[l] = g[l];
        out->svf_r = svf;
    }
    return GFM_OK;
}
int gfo_minor_get(void* vo, gfm_minor* m) {
    if (!vo || !m || !m->gfm || !m->smf || !m->bs_soot_prev || !m->sfp_soot_prev || !m->rrms) return GFM_E_ARG;
    Oracle* o = static_cast<Oracle*>(vo);
    if (!o->minor_on) return GFM_E_ARG;
    std::copy(o->GFMS.begin(), o->GFMS.end(), m->gfm);
    std::copy(o->SMF.begin(), o->SMF.end(), m->smf);
    std::copy(o->BS_SOOT_PREV.begin(), o->BS_SOOT_PREV.end(), m->bs_soot_prev);
    std::copy(o->SFP_SOOT_PREV.begin(), o->SFP_SOOT_PREV.end(), m->sfp_soot_prev);
    std::copy(o->RRMS.begin(), o->RRMS.end(), m->rrms);
    m->itr_ms = o->itr_ms;
    m->imscon = o->imscon;
    return GFM_OK;
}

double gfo_rif3(double x) { return RIF3(x); }
double gfo_zy1(const double* x, const double* y, double x1, int n) { return ZY1(x, y, x1, n); }
double gfo_t_to_enth(const double* y, double t_norm) {
    double c[9]; std::memcpy(c, y, sizeof c);
    return T_to_enth(Y9{c, 1}, t_norm);
}
double gfo_enth_to_t(const double* y, double h_norm, double t_guess_norm) {
    double c[9]; std::memcpy(c, y, sizeof c);
    c[IH - 1] = h_norm;
    return enth_to_T(Y9{c, 1}, t_guess_norm);
}
void gfo_conc(double* y) { conc(Y9{y, 1}); }

}  // extern "C"

// ---------------------------------------------------------------------------
// Start-up of the synthetic furnace, restated for the oracle so that its runs
// (the reference arm of the benchmark among them) need nothing from the
// product library: GRID3's coordinate lines and cell map with the
// 27-neighbour propagation (Grid3.f90:31-280), the SETUP constants
// (Setup.f90:542-731), SBC's inlet states with the SBC1/SBC3 face values and
// the outlet composition (Sbc.f90:57-388, 491-576), gen_initial_guess
// (Initsv.f90:97-162), the wall patches of the convective sink
// (Qwall.f90:395-513) and the kinetics table (Setup.f90:858-888).  The
// furnace itself (a box, inlets on x=0 snapped to whole cells with the
// velocity rescaled to keep the mass flow, a flue on x=lx, seeded jitter and
// noise) is the benchmark's synthetic stand-in for a case directory; its
// conventions are the generator's and are the same here.
// ---------------------------------------------------------------------------
namespace {

struct OCase {
    int mp = 0, np = 0, lp = 0;
    vec x, dx, r, dr, rs, z, dz;
    std::vector<int16_t> ib;
    std::vector<int16_t> b_typ, b_i, b_j, b_k, b_orient, b_direct;
    vec b_t, rtim, delrt, hrt, delr, timed, hrd, wl, akl0;
    vec p, t, dnst, theta, tmu, gama, crate, hrate, bs_hprev, ug, gf, qa, qe, t_surf_prev;
    long at(int i, int j, int k) const { return (i - 1) + (long)mp * ((j - 1) + (long)np * (k - 1)); }
    long n() const { return (long)mp * np * lp; }
};

uint64_t oc_mix64(uint64_t x) {   // splitmix64 finaliser: the generator's per-cell noise
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
double oc_noise(uint64_t seed, uint64_t idx, uint64_t comp) {   // uniform on [-1, 1)
    uint64_t h = oc_mix64(seed ^ oc_mix64(idx * 16 + comp));
    return ((double)(h >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
}

// GRID3 coordinate line (Grid3.f90:79-109) of a uniform grid file: X(1..3) =
// 0, then DEL added I2-I1 times up to X(N-1) = length, X(N) = X(N-1),
// DX(I) = X(I+1) - X(I-1) inside, 0 at both ends.
void oc_line(int n, double len, vec& x, vec& dx) {
    x.assign(n, 0.0);
    dx.assign(n, 0.0);
    const int i1 = 3, i2 = n - 1;
    const double del = (len - x[i1 - 1]) / (i2 - i1);
    for (int i = i1 + 1; i <= i2; ++i) x[i - 1] = x[i - 2] + del;
    x[n - 1] = x[n - 2];
    for (int i = 2; i <= n - 1; ++i) dx[i - 1] = x[i] - x[i - 2];
}

// the generator's opening on a line of ncell cells of width h: a run of whole
// cells, count = round((b-a)/h) at least 1, centred on the opening
void oc_snap(double a, double b, double h, int ncell, int& first, int& count) {
    count = (int)std::lround((b - a) / h);
    if (count < 1) count = 1;
    if (count > ncell) count = ncell;
    first = (int)std::lround(0.5 * (a + b) / h - 0.5 * count) + 1;
    if (first < 1) first = 1;
    if (first + count - 1 > ncell) first = ncell - count + 1;
}

struct OInlet { int j1, j2, k1, k2; double u, t_k, yf, yox, yn2, yco2, yh2o; };

}  // namespace

extern "C" {

int gfo_case_build(const gfm_case_spec* sp, const char* kinetic_path, gfm_case* out) {
    if (!sp || !kinetic_path || !out) return GFM_E_ARG;
    std::memset(out, 0, sizeof *out);
    if (sp->nx < 4 || sp->ny < 4 || sp->nz < 4 || sp->n_inlets < 1 || sp->n_inlets > 8 || sp->nwl < 1 || sp->nwl > 16)
        return GFM_E_ARG;
    OCase* c = new OCase;
    OCase& s = *c;
    const int mp = 2 * sp->nx + 4, np = 2 * sp->ny + 4, lp = 2 * sp->nz + 4;
    s.mp = mp; s.np = np; s.lp = lp;
    const long N = s.n();
    oc_line(mp, sp->lx, s.x, s.dx);
    oc_line(np, sp->ly, s.r, s.dr);
    oc_line(lp, sp->lz, s.z, s.dz);
    s.rs.assign(np, 1.0);   // cartesian (Grid3.f90:166)
    auto IB = [&](int i, int j, int k) -> int16_t& { return s.ib[s.at(i, j, k)]; };

    // cell map: walls (IBCELL 1) on the six faces of the box, inlets (2) on
    // x=0, the flue (3) on x=lx, open cells (0) inside
    s.ib.assign(N, 0);
    for (int k = 2; k <= lp; k += 2)
        for (int j = 2; j <= np; j += 2)
            for (int i = 2; i <= mp; i += 2)
                if (i == 2 || i == mp || j == 2 || j == np || k == 2 || k == lp) IB(i, j, k) = 1;
    const double hy = sp->ly / sp->ny, hz = sp->lz / sp->nz;
    std::vector<OInlet> inl(sp->n_inlets);
    for (int n = 0; n < sp->n_inlets; ++n) {
        const gfm_inlet_spec& is = sp->inlets[n];
        int fy, cy, fz, cz;
        oc_snap(is.y0, is.y1, hy, sp->ny, fy, cy);
        oc_snap(is.z0, is.z1, hz, sp->nz, fz, cz);
        OInlet& b = inl[n];
        b.j1 = 2 * fy + 2; b.j2 = 2 * (fy + cy - 1) + 2;
        b.k1 = 2 * fz + 2; b.k2 = 2 * (fz + cz - 1) + 2;
        const double jit = sp->inlet_jitter > 0 ? 1.0 + sp->inlet_jitter * oc_noise(sp->seed, 1000003ull + n, 7) : 1.0;
        b.u = is.u_ms * ((is.y1 - is.y0) * (is.z1 - is.z0)) / (cy * hy * cz * hz) * jit;
        b.t_k = is.t_k; b.yf = is.yf; b.yox = is.yo2; b.yn2 = is.yn2; b.yco2 = is.yco2; b.yh2o = is.yh2o;
        for (int k = b.k1; k <= b.k2; k += 2)
            for (int j = b.j1; j <= b.j2; j += 2) IB(2, j, k) = 2;
    }
    {
        int fy, cy, fz, cz;
        oc_snap(sp->exit_y0, sp->exit_y1, hy, sp->ny, fy, cy);
        oc_snap(sp->exit_z0, sp->exit_z1, hz, sp->nz, fz, cz);
        for (int k = 2 * fz + 2; k <= 2 * (fz + cz - 1) + 2; k += 2)
            for (int j = 2 * fy + 2; j <= 2 * (fy + cy - 1) + 2; j += 2) IB(mp, j, k) = 3;
    }
    // NCELLS and the propagation of each closed cell's code onto its faces,
    // edges and corners that are not walls (Grid3.f90:259-275)
    int ncells = 0;
    for (int i = 2; i <= mp; i += 2)
        for (int j = 2; j <= np; j += 2)
            for (int k = 2; k <= lp; k += 2) {
                const int ibc1 = IB(i, j, k);
                if (ibc1 <= 0) { ++ncells; continue; }
                for (int i1 = i - 1; i1 <= i + 1; ++i1)
                    for (int j1 = j - 1; j1 <= j + 1; ++j1)
                        for (int k1 = k - 1; k1 <= k + 1; ++k1) {
                            if (i1 > mp || j1 > np || k1 > lp) continue;
                            if (IB(i1, j1, k1) != 1) IB(i1, j1, k1) = (int16_t)ibc1;
                        }
            }

    // SETUP (Setup.f90:542-731); GMFR is the inlets' total mass flow, as the
    // case-writing front end puts it in the &INPUT group
    const double pg0 = sp->pg0 > 0 ? sp->pg0 : 1.01325e5;
    const double RU = 8.3143e+3;
    double gmfr = 0.0;
    for (int n = 0; n < sp->n_inlets; ++n) {
        const gfm_inlet_spec& is = sp->inlets[n];
        const double w_in = ONE / (is.yf / WF + is.yco2 / WCO2 + is.yh2o / WH2O + is.yo2 / WO2 + is.yn2 / WN2);
        const double rho = pg0 * w_in / (RU * is.t_k);
        const int cy = (inl[n].j2 - inl[n].j1) / 2 + 1, cz = (inl[n].k2 - inl[n].k1) / 2 + 1;
        gmfr += rho * std::fabs(inl[n].u) * (cy * hy) * (cz * hz);
    }
    gfm_params& P = out->params;
    const double t0 = T0C, h_0 = H0C, area0 = 1.0, r0 = 1.0;
    const double wt0 = 1.0 / (0.5 / 16.0426 + 0.0 / 44.0098 + 0.0 / 18.0152 + 0.49 / 31.9988 + 0.01 / 28.0134);
    const double dnst0 = pg0 * wt0 / RU / t0;
    const double ug0 = gmfr / dnst0 / area0;
    const double gmu_ref = 2.6e-5 * std::pow(5.33e+2 / 2.98e+2, 0.0);
    const double tk0 = 5.0e-2 * (ug0 * ug0), epsi0 = 1.0 * (tk0 * tk0);
    const double reyg = 2.0 * dnst0 * ug0 * r0 / gmu_ref;
    P.t0 = t0; P.h_0 = h_0; P.dnst0 = dnst0; P.ug0 = ug0; P.gmfr = gmfr; P.pg0 = pg0; P.r0 = r0;
    P.reyg = reyg; P.reyg2 = reyg / 2.0;
    P.epsr = tk0 / (ug0 * ug0);
    P.taur = epsi0 * r0 / (tk0 * ug0);
    P.eun = pg0 / (dnst0 * (ug0 * ug0));
    P.qr0 = h_0 * dnst0 * ug0 / r0;
    P.q0 = (sp->q0_jkg > 0 ? sp->q0_jkg : 2.42e6) / h_0;
    P.tk0 = tk0;
    P.gra[0] = 0.0 / ug0 / ug0 * r0; P.gra[1] = 0.0 / ug0 / ug0 * r0; P.gra[2] = -9.80621 / ug0 / ug0 * r0;
    P.amu = 0.0; P.trdg = 298.15 / 5.0e+2; P.wt0 = wt0; P.stoich = 2.0 * 31.9988 / 16.0426;
    P.cmu = 9.0e-2; P.ct1 = 1.44; P.ct2 = 1.92;
    P.p_mx = 0.2; P.p_mn = -0.6; P.t_mx = 3.0e+3 / t0; P.t_mn = 2.0e+2 / 5.0e+2;
    P.u_mx = 1.0e+3 / ug0; P.u_mn = -P.u_mx; P.f_mx = 1.5; P.f_mn = 0.8;
    for (int i = 0; i < 21; ++i) { P.rf[i] = 0.7; P.rfl[i] = 0.6; }
    P.rf[0] = P.rf[1] = P.rf[2] = sp->rf_uvw;
    P.rf[17] = 0.6; P.rf[20] = 0.6;
    P.rfl[0] = sp->rfl_species; P.rfl[1] = sp->rfl_species; P.rfl[2] = sp->rfl_h; P.rfl[3] = sp->rfl_k;
    P.rfl[4] = sp->rfl_eps; P.rfl[5] = sp->rfl_species; P.rfl[6] = sp->rfl_species;
    const double sig0[12] = {0.7, 0.7, 0.7, 1.0, 1.0, 0.7, 0.7, 0.7, 0.7, 0.7, 0.7, 0.7};
    for (int i = 0; i < 12; ++i) P.sigma[i] = sig0[i];
    P.sigma[3] = sp->sigma_k; P.sigma[4] = sp->sigma_eps;
    for (int i = 0; i < 20; ++i) P.ntimesg[i] = i < 12 ? sp->ntimesg[i] : 2;
    P.rf_hsource = sp->rf_hsource;
    P.react = sp->react; P.turb = 1;
    P.wall_sink = sp->wall_sink; P.h_g = sp->h_g;
    P.rad_emission = sp->rad_emission; P.rad_qe_frequency = 10;
    P.sig = 5.668e-8; P.ri = 1.0; P.hck = 1.439e-2;
    P.bgcon = sp->bgcon; P.maxgi = sp->maxgi; P.adi_mode = sp->adi_mode; P.precision = sp->precision;
    // minor species defaults (Var_mod.f90:215, 474-492; relaxfactorc.txt)
    P.gas_model = 0; P.maxms = 300; P.ntimesm = 4; P.irstypm = 0; P.bmcon = 1.0e-7; P.ssigma = 0.7;
    P.rfm = 0.5; P.rfm_soot = 0.2; P.rf_soot_form = 0.3; P.rf_soot_oxid = 0.3;
    P.soot_cap = 4.0e-3; P.t0_sf = 0.0; P.t0_so = 0.0; P.aform = 400.0; P.aoxid = 26.0;
    P.esf_r = 5.0e7 / 8.3143e+3; P.eso_r = 5.0e7 / 8.3143e+3;

    // fields at allocation (Setup.f90:747-779)
    s.p.assign(N, 0.0); s.t.assign(N, 1.0); s.dnst.assign(N, 1.0); s.theta.assign(N, 1.0);
    s.tmu.assign(N, 0.0); s.gama.assign(N, 0.0); s.crate.assign(N, 0.0); s.hrate.assign(N, 0.0);
    s.bs_hprev.assign(N, 0.0); s.ug.assign(3 * N, 0.0); s.gf.assign(9 * N, 0.0);
    const long ncell_arr = (long)(mp / 2) * (np / 2) * (lp / 2);
    s.qa.assign(ncell_arr, 0.0); s.qe.assign(ncell_arr, 0.0);
    s.t_surf_prev.assign((size_t)(mp / 2) * (np / 2), 0.0);
    auto Y = [&](long a) { return Y9{&s.gf[a], N}; };
    auto GF = [&](long a, int l) -> double& { return s.gf[a + (long)(l - 1) * N]; };
    auto dnst_at = [&](long a) {   // dnst_calc (Prop.f90:187-198)
        conc(Y(a));
        const double temp = (ONE + s.p[a]) / s.t[a] * wmix(Y(a)) / P.wt0;
        s.dnst[a] = fmax2(temp, small20);
    };
    auto ther_at = [&](long a) {   // THER (Prop.f90:130-154)
        GF(a, IEPS) = fmax2(GF(a, IEPS), 1.0e-12);
        s.tmu[a] = P.cmu * P.reyg * P.epsr / (TWO * P.taur) * (GF(a, IK) * GF(a, IK)) / GF(a, IEPS) * s.dnst[a];
        s.gama[a] = TWO / P.reyg * (s.tmu[a] + std::pow(s.t[a] / P.trdg, P.amu));
    };
    auto tke_at = [&](long a) {    // TKE (Prop.f90:162-176)
        const double g = s.ug[a] * s.ug[a] + s.ug[a + N] * s.ug[a + N] + s.ug[a + 2 * N] * s.ug[a + 2 * N];
        GF(a, IK) = fmax2(g, 1.0e-6);
        GF(a, IEPS) = GF(a, IK) * GF(a, IK);
    };
    auto t2h_at = [&](long a) { GF(a, IH) = T_to_enth(Y(a), s.t[a]); };

    // SBC (Sbc.f90:57-269): inlet cells of each block, IU = 1 (x faces)
    const double p_ref = 0.0 / pg0;
    double fr_f = 0, fr_ox = 0, fr_n2 = 0, q_h_in = 0;
    std::vector<char> done(N, 0);
    for (const OInlet& b : inl) {
        const double T_0 = b.t_k / t0, U_0 = b.u / ug0;
        for (int j = b.j1; j <= b.j2; j += 2)
            for (int k = b.k1; k <= b.k2; k += 2) {
                const long a = s.at(2, j, k);
                if (IB(2, j, k) != 2 || done[a]) continue;
                done[a] = 1;
                s.p[a] = p_ref;
                s.t[a] = T_0;
                GF(a, IYF) = b.yf; GF(a, IYCO2) = b.yco2; GF(a, IYH2O) = b.yh2o; GF(a, IYO2) = b.yox; GF(a, IYN2) = b.yn2;
                dnst_at(a);
                s.ug[a] = U_0; s.ug[a + N] = 0.0; s.ug[a + 2 * N] = 0.0;
                tke_at(a);
                ther_at(a);
                t2h_at(a);
                double g0 = s.theta[a] * s.dnst[a] * dnst0;
                const double area = s.dr[j - 1] * s.rs[j - 1] * s.dz[k - 1] * area0;   // AREA_C(.,.,.,1)
                g0 = g0 * std::fabs(U_0) * ug0 * area;
                fr_f += g0 * GF(a, IYF);
                fr_ox += g0 * GF(a, IYO2);
                fr_n2 += g0 * GF(a, IYN2);
                q_h_in += GF(a, IH) * h_0 * g0;
            }
        // SBC1 (Sbc.f90:391-486): the faces between a block's inlet cells
        auto sbc1 = [&](long A, long B, long C, double f1) {
            const double f2 = 1.0 - f1;
            s.p[C] = f1 * s.p[A] + f2 * s.p[B];
            s.t[C] = f1 * s.t[A] + f2 * s.t[B];
            for (int l = 0; l < 9; ++l) {
                if (l < 3) s.ug[C + l * N] = f1 * s.ug[A + l * N] + f2 * s.ug[B + l * N];
                s.gf[C + l * N] = f1 * s.gf[A + l * N] + f2 * s.gf[B + l * N];
            }
            dnst_at(C);
            s.theta[C] = f1 * s.theta[A] + f2 * s.theta[B];
            s.tmu[C] = f1 * s.tmu[A] + f2 * s.tmu[B];
            s.gama[C] = f1 * s.gama[A] + f2 * s.gama[B];
        };
        // SBC3 (Sbc.f90:491-522): copy onto the inlet's neighbouring face planes
        auto sbc3 = [&](long A, long B) {
            for (int l = 0; l < 3; ++l) s.ug[B + l * N] = s.ug[A + l * N];
            s.p[B] = s.p[A]; s.t[B] = s.t[A];
            for (int l = 0; l < 9; ++l) s.gf[B + l * N] = s.gf[A + l * N];
            s.dnst[B] = s.dnst[A]; s.theta[B] = s.theta[A]; s.tmu[B] = s.tmu[A]; s.gama[B] = s.gama[A];
        };
        const int i = 2;   // IU = 1 block on the x=0 wall (Sbc.f90:179-206)
        if (b.k2 > b.k1)
            for (int k = b.k1 + 1; k <= b.k2 - 1; k += 2)
                for (int j = b.j1; j <= b.j2; j += 2)
                    sbc1(s.at(i, j, k + 1), s.at(i, j, k - 1), s.at(i, j, k), (s.z[k - 1] - s.z[k - 2]) / s.dz[k - 1]);
        if (b.j2 > b.j1)
            for (int j = b.j1 + 1; j <= b.j2 - 1; j += 2)
                for (int k = b.k1; k <= b.k2; ++k)
                    sbc1(s.at(i, j + 1, k), s.at(i, j - 1, k), s.at(i, j, k), (s.r[j - 1] - s.r[j - 2]) / s.dr[j - 1]);
        for (int j = b.j1; j <= b.j2; ++j)
            for (int k = b.k1; k <= b.k2; ++k) {
                if (i < mp && IB(i + 1, j, k) == 2) sbc3(s.at(i, j, k), s.at(i + 1, j, k));
                if (i > 2 && IB(i - 1, j, k) == 2) sbc3(s.at(i, j, k), s.at(i - 1, j, k));
            }
    }
    const double gfin = fr_f + fr_ox + fr_n2;
    if (!(gfin > 0.0)) { delete c; std::memset(out, 0, sizeof *out); return GFM_E_ARG; }
    // est_out_mass_frac (Sbc.f90:566-576)
    const double yn2_out = fr_n2 / gfin;
    const double yh2o_out = (2 * fr_f * WH2O / WF) / gfin;
    const double yco2_out = (fr_f * WCO2 / WF) / gfin;
    const double yo2_out = (fr_ox - 2 * fr_f * WO2 / WF) / gfin;

    // gen_initial_guess (Initsv.f90:97-162), with the generator's seeded
    // perturbation of T and the species in the open cells
    gfm_fields& F = out->fields;
    F.factor = 1.0; F.fadj = 0.0;
    const double T_init = sp->t_init_k / t0, amp = sp->noise_amp;
    for (int i = 2; i <= mp; i += 2)
        for (int j = 2; j <= np; j += 2)
            for (int k = 2; k <= lp; k += 2) {
                const int ibc = IB(i, j, k);
                if (ibc == 2) continue;
                const long a = s.at(i, j, k);
                double nz5[5] = {0, 0, 0, 0, 0};
                if (ibc == 0 && amp != 0.0)
                    for (int q = 0; q < 5; ++q) nz5[q] = amp * oc_noise(sp->seed, (uint64_t)a, (uint64_t)q);
                GF(a, IYF) = 0;
                GF(a, IYO2) = yo2_out * (1.0 + nz5[1]);
                GF(a, IYCO2) = yco2_out * (1.0 + nz5[2]);
                GF(a, IYH2O) = yh2o_out * (1.0 + nz5[3]);
                GF(a, IYN2) = yn2_out * (1.0 + nz5[4]);
                if (ibc == 1) {
                    s.t[a] = T_init;
                    t2h_at(a);
                    continue;
                }
                s.ug[a] = 0; s.ug[a + N] = 0; s.ug[a + 2 * N] = 0;
                s.theta[a] = 1.0;
                if (ibc != 4) s.t[a] = T_init * (1.0 + nz5[0]);
                t2h_at(a);
                tke_at(a);
                dnst_at(a);
                ther_at(a);
            }

    // wall patches (Qwall.f90:395-513): faces of closed cells next to an
    // open one, x then y then z faces, b_T the fixed wall temperature
    auto add_patch = [&](int typ, int ori, int dir, int i, int j, int k) {
        s.b_typ.push_back((int16_t)typ); s.b_orient.push_back((int16_t)ori); s.b_direct.push_back((int16_t)dir);
        s.b_i.push_back((int16_t)i); s.b_j.push_back((int16_t)j); s.b_k.push_back((int16_t)k);
        s.b_t.push_back(sp->t_wall_k);
    };
    for (int k = 2; k <= lp; k += 2)
        for (int j = 2; j <= np; j += 2)
            for (int i = 3; i <= mp - 1; i += 2) {
                const int m = IB(i, j, k);
                if (m < 1 || (IB(i - 1, j, k) > 0 && IB(i + 1, j, k) > 0)) continue;
                add_patch(m, 1, IB(i + 1, j, k) == 0 ? 0 : 1, i, j, k);
            }
    for (int k = 2; k <= lp; k += 2)
        for (int j = 3; j <= np - 1; j += 2)
            for (int i = 2; i <= mp; i += 2) {
                const int m = IB(i, j, k);
                if (m < 1 || (IB(i, j - 1, k) > 0 && IB(i, j + 1, k) > 0)) continue;
                add_patch(m, 2, IB(i, j + 1, k) == 0 ? 0 : 1, i, j, k);
            }
    for (int k = 3; k <= lp - 1; k += 2)
        for (int j = 2; j <= np; j += 2)
            for (int i = 2; i <= mp; i += 2) {
                const int m = IB(i, j, k);
                if (m < 1 || (IB(i, j, k - 1) > 0 && IB(i, j, k + 1) > 0)) continue;
                add_patch(m, 3, IB(i, j, k + 1) == 0 ? 0 : 1, i, j, k);
            }

    // kinetics table (Setup.f90:858-888): two blocks of NR0 rows after a
    // header line each; times scaled by 0.7, heat by CHRD/H_0/WF
    const int nr0 = 100;
    {
        FILE* fp = std::fopen(kinetic_path, "r");
        if (!fp) { delete c; std::memset(out, 0, sizeof *out); return GFM_E_IO; }
        char line[512];
        bool ok = std::fgets(line, sizeof line, fp) != nullptr;
        const double chrd = 0.166;
        s.rtim.resize(nr0); s.delrt.resize(nr0); s.hrt.resize(nr0);
        s.delr.resize(nr0); s.timed.resize(nr0); s.hrd.resize(nr0);
        for (int i = 0; ok && i < nr0; ++i) {
            ok = std::fgets(line, sizeof line, fp) && std::sscanf(line, "%lf %lf %lf", &s.rtim[i], &s.delrt[i], &s.hrt[i]) == 3;
            s.rtim[i] = s.rtim[i] * 0.7;
            s.hrt[i] = chrd * s.hrt[i] / h_0 / WF;
        }
        ok = ok && std::fgets(line, sizeof line, fp) != nullptr;
        for (int i = 0; ok && i < nr0; ++i) {
            ok = std::fgets(line, sizeof line, fp) && std::sscanf(line, "%lf %lf %lf", &s.delr[i], &s.timed[i], &s.hrd[i]) == 3;
            s.timed[i] = s.timed[i] * 0.7;
            s.hrd[i] = chrd * s.hrd[i] / h_0 / WF;
        }
        std::fclose(fp);
        if (!ok) { delete c; std::memset(out, 0, sizeof *out); return GFM_E_IO; }
    }
    for (int l = 0; l < sp->nwl; ++l) { s.wl.push_back(sp->wl_um[l] * 1.0e-6); s.akl0.push_back(sp->kappa[l]); }

    gfm_grid& G = out->grid;
    G.mp = mp; G.np = np; G.lp = lp;
    G.x = s.x.data(); G.dx = s.dx.data(); G.r = s.r.data(); G.dr = s.dr.data(); G.rs = s.rs.data();
    G.z = s.z.data(); G.dz = s.dz.data(); G.ibcell = s.ib.data(); G.ncells = ncells;
    G.i_ref = 2; G.j_ref = inl[0].j1; G.k_ref = inl[0].k1; G.p_ref = p_ref;
    G.b_cnt = (int)s.b_typ.size();
    G.b_typ = s.b_typ.data(); G.b_i = s.b_i.data(); G.b_j = s.b_j.data(); G.b_k = s.b_k.data();
    G.b_orient = s.b_orient.data(); G.b_direct = s.b_direct.data(); G.b_t = s.b_t.data();
    G.nr0 = nr0;
    G.rtim = s.rtim.data(); G.delrt = s.delrt.data(); G.hrt = s.hrt.data();
    G.delr = s.delr.data(); G.timed = s.timed.data(); G.hrd = s.hrd.data();
    G.nwl = sp->nwl; G.wl = s.wl.data(); G.akl0 = s.akl0.data();
    for (int q = 0; q < 2; ++q) G.bv_f[q] = 1.0;   // GRID3 defaults (Grid3.f90:252-254)
    for (int q = 0; q < 6; ++q) G.ba_f[q] = 1.0;
    F.p = s.p.data(); F.t = s.t.data(); F.dnst = s.dnst.data(); F.theta = s.theta.data();
    F.tmu = s.tmu.data(); F.gama = s.gama.data(); F.crate = s.crate.data(); F.hrate = s.hrate.data();
    F.bs_hprev = s.bs_hprev.data(); F.ug = s.ug.data(); F.gf = s.gf.data(); F.qa = s.qa.data(); F.qe = s.qe.data();
    F.gfin0 = gfin / gmfr; F.q_h_in = q_h_in;
    out->tail.mz = mp / 2; out->tail.nz = np / 2; out->tail.t_surf_prev = s.t_surf_prev.data();
    out->tail.interval_rad = 100;
    out->priv = c;
    return GFM_OK;
}

void gfo_case_free(gfm_case* c) {
    if (!c) return;
    delete static_cast<OCase*>(c->priv);
    std::memset(c, 0, sizeof *c);
}

}  // extern "C"
