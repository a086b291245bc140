// physics.h -- per-cell property functions of the GFM combustion-space solver,
// usable from host code (case construction) and from device kernels.
//
// Each function restates one reference routine; floating-point operations are
// kept in the reference's evaluation order so FP64 results track the Fortran.
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define GFM_HD __host__ __device__ __forceinline__
#else
#define GFM_HD inline
#endif

namespace gfm {

// ---- module constants (combustion/Code/Var_mod.f90) ------------------------
constexpr double kSmall20 = 1.0e-20;
constexpr double kSmall16 = 1.0e-16;
constexpr double kBig = 1.0e+20;
constexpr double kRu = 8.3143e+3;        // Var_mod.f90:22
constexpr double kWf = 16.0426;          // Var_mod.f90:142-147
constexpr double kWo2 = 31.9988;
constexpr double kWco2 = 44.0098;
constexpr double kWh2o = 18.0152;
constexpr double kWn2 = 28.0134;
constexpr double kCp0 = 1.0057e+3;       // Var_mod.f90:154
constexpr double kT0 = 5.0e+2;           // Var_mod.f90:179
constexpr double kTl0 = 298.15;
constexpr double kTl00 = 5.33e+2;
constexpr double kCmu = 9.0e-2;          // Var_mod.f90:203
constexpr double kCt1 = 1.44, kCt2 = 1.92;
constexpr double kCtea = 5.0e-2, kCtda = 1.0;
constexpr double kSig = 5.668e-8;        // Var_mod.f90:133
constexpr double kHck = 1.439e-2;
constexpr double kT0r = 1.0e2, kP0r = 1.01325e5;
constexpr double kTolEnth = 1.0e-11;     // Var_mod.f90:398
constexpr int kNmaxEnth = 10;            // Var_mod.f90:397
// gas-side viscosity / conductivity cubic fits (Var_mod.f90:168-176)
constexpr double kGmu3 = 2.0e-15, kGmu2 = -1.1e-11, kGmu1 = 4.5e-8, kGmu0 = 7.0e-6;

// GF component indices, 0-based (IYF=1, IYO2=2, IH=3, IK=4, IEPS=5, IYCO2=6,
// IYN2=7, IYH2O=9 in Var_mod.f90:116-123)
constexpr int kYF = 0, kYO2 = 1, kH = 2, kK = 3, kEps = 4, kYCO2 = 5, kYN2 = 6, kYH2O = 8;

// NIST Shomate coefficient sets (Setup.f90:103-141): species order CH4, O2,
// CO2, N2, H2O; [species][0=lo,1=hi].  These are physical data that have to be
// identical to the reference's for parity.
template <typename R>
struct NistT {
    R a[5][2], b[5][2], c[5][2], d[5][2], e[5][2], f[5][2], h[5][2];
    R cut[5];
    int gidx[5];
};
using Nist = NistT<double>;
// Host copy of the table; device code receives a pointer to a __constant__
// copy (see kernels), so every function below takes the table explicitly.
inline const Nist& nist_host() {
    static const Nist t = {
        {{-0.703029, 85.81217}, {29.659, 29.659}, {24.99735, 58.16639}, {26.092, 26.092}, {30.092, 41.96426}},
        {{108.4773, 11.26467}, {6.137261, 6.137261}, {55.18696, 2.720074}, {8.218801, 8.218801}, {6.832514, 8.622053}},
        {{-42.52157, -2.114146}, {-1.186521, -1.186521}, {-33.69137, -0.492289}, {-1.976141, -1.976141}, {6.793435, -1.49978}},
        {{5.862788, 0.13819}, {0.09578, 0.09578}, {7.948387, 0.038844}, {0.159274, 0.159274}, {-2.53448, 0.098119}},
        {{0.678565, -26.42221}, {-0.219663, -0.219663}, {-0.136638, -6.447293}, {0.044434, 0.044434}, {0.082139, -11.15764}},
        {{-76.84376, -153.5327}, {-9.861391, -9.861391}, {-403.6075, -425.9186}, {-7.98923, -7.98923}, {-250.881, -272.1797}},
        {{-74.8731, -74.8731}, {0.0, 0.0}, {-393.5224, -393.5224}, {0.0, 0.0}, {-241.8264, -241.8264}},
        {1300.0, 6000.0, 1200.0, 6000.0, 1700.0},       // cutT, Var_mod.f90:417-422
        {kYF, kYO2, kYCO2, kYN2, kYH2O}};               // gf_chem_index, Setup.f90:85-89
    return t;
}
// The table rounded to the arithmetic type of a kernel.
template <typename R>
inline NistT<R> nist_cast(const Nist& n) {
    NistT<R> t;
    for (int s = 0; s < 5; ++s) {
        for (int k = 0; k < 2; ++k) {
            t.a[s][k] = R(n.a[s][k]); t.b[s][k] = R(n.b[s][k]); t.c[s][k] = R(n.c[s][k]); t.d[s][k] = R(n.d[s][k]);
            t.e[s][k] = R(n.e[s][k]); t.f[s][k] = R(n.f[s][k]); t.h[s][k] = R(n.h[s][k]);
        }
        t.cut[s] = R(n.cut[s]);
        t.gidx[s] = n.gidx[s];
    }
    return t;
}

// Species closure CONC (Prop.f90:28-59).  y points at the 9 GF components of a
// position, stride `s` between components.
template <typename R>
GFM_HD void conc(R* y, long s) {
    R g0 = y[kYF * s] + y[kYO2 * s] + y[kYCO2 * s] + y[kYN2 * s];
    if (g0 > R(1)) {
        g0 = g0 + y[kYH2O * s];
        y[kYF * s] = y[kYF * s] / g0;
        y[kYO2 * s] = y[kYO2 * s] / g0;
        y[kYCO2 * s] = y[kYCO2 * s] / g0;
        y[kYN2 * s] = y[kYN2 * s] / g0;
        y[kYH2O * s] = y[kYH2O * s] / g0;
    } else {
        y[kYH2O * s] = R(1) - g0;
    }
}

// Mixture molecular weight in the order of dnst_calc / enth_to_T
// (Prop.f90:192-194, 375-376).
template <typename R>
GFM_HD R wmix(const R* y, long s) {
    return R(1) / (y[kYF * s] / R(kWf) + y[kYCO2 * s] / R(kWco2) + y[kYH2O * s] / R(kWh2o) +
                   y[kYO2 * s] / R(kWo2) + y[kYN2 * s] / R(kWn2));
}

// dnst_calc (Prop.f90:187-198): calls CONC first, then ideal-gas density.
template <typename R>
GFM_HD R dnst_calc(R* y, long s, R p, R t, R wt0) {
    conc(y, s);
    R wt = wmix(y, s);
    R temp = (R(1) + p) / t * wt / wt0;
    return temp > R(kSmall20) ? temp : R(kSmall20);
}

// Shomate mixture coefficients with the reference's f_mix/h_mix accumulation
// (f_mix = d_mix + Y*F and h_mix = e_mix + Y*H inside the species loop,
// Prop.f90:398-418).
template <typename R>
struct ShomateMix { R a, b, c, d, e, f, h; int lohi[5]; };

template <typename R>
GFM_HD void shomate_mix(const NistT<R>& N, const R* y, long s, R real_T, ShomateMix<R>& m) {
    m.a = m.b = m.c = m.d = m.e = m.f = m.h = R(0);
    for (int n = 0; n < 5; ++n) {
        int set = (real_T < N.cut[n]) ? 0 : 1;
        R yy = y[N.gidx[n] * s];
        m.a = m.a + yy * N.a[n][set];
        m.b = m.b + yy * N.b[n][set];
        m.c = m.c + yy * N.c[n][set];
        m.d = m.d + yy * N.d[n][set];
        m.e = m.e + yy * N.e[n][set];
        m.f = m.d + yy * N.f[n][set];
        m.h = m.e + yy * N.h[n][set];
        m.lohi[n] = set;
    }
}

// Newton stopping test on |dT| (T in kK).  FP64 uses the reference's 1e-11
// (Var_mod.f90:398); FP32 stops at 1e-6 kK, where the next quadratic step is
// already below the FP32 resolution of T.
template <typename R> struct EnthTol { static constexpr double v = kTolEnth; };
template <> struct EnthTol<float> { static constexpr double v = 1.0e-6; };

// T_to_enth (Prop.f90:525-565): returns normalised enthalpy.
template <typename R>
GFM_HD R t_to_enth(const NistT<R>& N, const R* y, long s, R T, R t0, R h0) {
    R w_mix = wmix(y, s);
    R real_T = T * t0;
    ShomateMix<R> m;
    shomate_mix(N, y, s, real_T, m);
    R tn = real_T / R(1000);
    R ef = tn * (m.a + tn * ((m.b / R(2)) + tn * ((m.c / R(3)) + tn * (m.d / R(4))))) - (m.e / tn) + m.f - m.h;
    return ef * R(1.0e6) / (w_mix * h0);
}

// enth_to_T (Prop.f90:369-505): Newton on the Shomate integral with the
// reference's in-loop coefficient-set switches for CH4, CO2 and H2O.
// Returns the normalised temperature.
template <typename R>
GFM_HD R enth_to_t(const NistT<R>& N, const R* y, long s, R h_norm, R T, R t0, R h0) {
    R w_mix = wmix(y, s);
    R h_s = h_norm * h0;
    R h_molar = h_s * w_mix / R(1.0e6);
    R real_T = T * t0;
    ShomateMix<R> m;
    shomate_mix(N, y, s, real_T, m);
    R T_old = real_T / R(1000);
    R T_new = T_old;   // the reference keeps the module value of an earlier call here
    for (int it = 0; it < kNmaxEnth; ++it) {
        R gp = m.a + T_old * (m.b + T_old * (m.c + T_old * m.d)) + m.e / (T_old * T_old);
        if (gp == R(0)) break;
        R g0 = T_old * (m.a + T_old * ((m.b / R(2)) + T_old * ((m.c / R(3)) + T_old * (m.d / R(4))))) -
               (m.e / T_old) + m.f - m.h;
        R dT = (g0 - h_molar) / gp;
        T_new = T_old - dT;
        if (fabs(dT) < R(EnthTol<R>::v)) break;
        T_old = T_new;
        for (int nn = 0; nn < 5; nn += 2) {      // CH4, CO2, H2O (O2, N2 have one set)
            R yy = y[N.gidx[nn] * s];
            if (T_new * R(1000) < N.cut[nn] && m.lohi[nn] != 0) {
                m.a = m.a - yy * N.a[nn][1]; m.b = m.b - yy * N.b[nn][1]; m.c = m.c - yy * N.c[nn][1];
                m.d = m.d - yy * N.d[nn][1]; m.e = m.e - yy * N.e[nn][1];
                m.f = m.d - yy * N.f[nn][1]; m.h = m.e - yy * N.h[nn][1];
                m.lohi[nn] = 0;
                m.a = m.a + yy * N.a[nn][0]; m.b = m.b + yy * N.b[nn][0]; m.c = m.c + yy * N.c[nn][0];
                m.d = m.d + yy * N.d[nn][0]; m.e = m.e + yy * N.e[nn][0];
                m.f = m.d + yy * N.f[nn][0]; m.h = m.e + yy * N.h[nn][0];
            }
            if (T_new * R(1000) >= N.cut[nn] && m.lohi[nn] != 1) {
                m.a = m.a - yy * N.a[nn][0]; m.b = m.b - yy * N.b[nn][0]; m.c = m.c - yy * N.c[nn][0];
                m.d = m.d - yy * N.d[nn][0]; m.e = m.e - yy * N.e[nn][0];
                m.f = m.d - yy * N.f[nn][0]; m.h = m.e - yy * N.h[nn][0];
                m.lohi[nn] = 1;
                m.a = m.a + yy * N.a[nn][1]; m.b = m.b + yy * N.b[nn][1]; m.c = m.c + yy * N.c[nn][1];
                m.d = m.d + yy * N.d[nn][1]; m.e = m.e + yy * N.e[nn][1];
                m.f = m.d + yy * N.f[nn][1]; m.h = m.e + yy * N.h[nn][1];
            }
        }
    }
    return T_new * R(1000) / t0;
}

// Elementary functions in the arithmetic of the path: the float versions in
// the mixed path (no promotion to FP64, whose pipe is narrow on GB300), the
// double versions exactly as in the FP64 path.
GFM_HD float r_exp(float x) { return expf(x); }
GFM_HD double r_exp(double x) { return exp(x); }
GFM_HD float r_log(float x) { return logf(x); }
GFM_HD double r_log(double x) { return log(x); }
GFM_HD float r_pow(float a, float b) { return powf(a, b); }
GFM_HD double r_pow(double a, double b) { return pow(a, b); }
GFM_HD float r_sqrt(float x) { return sqrtf(x); }
GFM_HD double r_sqrt(double x) { return sqrt(x); }

// Exponential-scheme weight DA(D,F) (Prop.f90:97-117).
template <typename R>
GFM_HD R da(R d, R f) {
    if (d <= R(1.0e-25)) return R(0);
    R fa = f < R(0) ? -f : f;
    R pe = fa / d;
    if (pe <= R(1.0e-2)) {
        const R sixth = R(1.0) / R(6.0);
        return d / (R(1) + pe * (R(0.5) + pe * (sixth + pe / R(24.0))));
    } else if (pe <= R(2.0e+1)) {
        return fa / (r_exp(pe) - R(1));
    }
    return R(0);
}

// Log-law wall factor TGAMF (Gflow.f90:417-426).
template <typename R>
GFM_HD R tgamf(R b) {
    if (b < R(11.5)) return R(1);
    R g0 = b / (r_log(R(9) * b) * R(2.5));
    return g0 > R(1) ? g0 : R(1);
}

// Gray-band emissivity EMF (Rad_fun.f90:97-115).
GFM_HD double emf(double xkl, double xl0) {
    const double x1 = 1.0e-3;
    const double g1 = (1.0 - exp(-x1)) / x1;
    double x0 = xkl * xl0;
    return x0 <= x1 ? x0 * g1 : 1.0 - exp(-x0);
}

// Chang-Rhee series RIF(3,0,X) used by DEBX (Rad_fun.f90:45-91 with M=3,
// A=0; Y(I+1)=PER(3,I) = 1,3,6,6).  Integer powers are products, as the
// Fortran X**(M-I) and (A+N)**(I+1) are.  DEBX never passes X=0 (X=DEB0/T>0);
// that branch returns 1 (the full-spectrum fraction).
GFM_HD double rif3(double x) {
    const double pi = 3.141592653589793;
    if (x > 1.0e16) return 0.0;
    if (x == 0.0) return 1.0;
    double r = 0.0;
    for (int n = 1; n <= 1000; ++n) {
        double an = (double)n;
        double an2 = an * an, an3 = an2 * an, an4 = an3 * an;
        double g0 = 0.0;
        g0 = g0 + 1.0 * (x * x * x) / an;
        g0 = g0 + 3.0 * (x * x) / an2;
        g0 = g0 + 6.0 * x / an3;
        g0 = g0 + 6.0 * 1.0 / an4;
        g0 = g0 * exp(-an * x);
        r = r + g0;
        if (fabs(g0) <= 1.0e-16) break;
    }
    r = r * 1.5e1 / (pi * pi * pi * pi);
    return r > 1.0 ? 1.0 : r;
}

// Linear table lookup ZY1 (Source.f90:814-831).
GFM_HD double zy1(const double* x, const double* y, double x1, int n) {
    if (x1 < x[0]) return y[0] * x1 / x[0];
    for (int i = 1; i < n; ++i) {
        if (x1 < x[i]) {
            double ratio = (x1 - x[i - 1]) / (x[i] - x[i - 1]);
            return y[i - 1] + (y[i] - y[i - 1]) * ratio;
        }
    }
    return y[n - 1];
}

}  // namespace gfm
