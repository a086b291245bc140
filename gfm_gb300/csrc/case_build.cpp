// case_build.cpp -- host construction of a case in the reference's data
// layout: the work the Fortran host does before the first GFLOW (GRID3,
// SETUP, SBC, INITSV; combustion/Code/A0main.f90:158-190).
//
// gfm_case_build makes the synthetic furnace that stands in for the
// reference's gd####c.dat / sbc####c.dat input files: a rectangular box, walls
// on all six sides, inlets on the x=0 wall, one flue opening on the x=lx wall.
// finish_case is the part shared with the case-file reader (case_files.cpp).
#include "case_store.h"
#include "physics.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

namespace gfm {
namespace host {

using gfm::Nist;

void prop_dnst(CaseStore& s, const gfm_params& P, long a) {
    s.dnst[a] = gfm::dnst_calc<double>(&s.gf[a], s.n(), s.p[a], s.t[a], P.wt0);
}

void prop_ther(CaseStore& s, const gfm_params& P, long a) {
    const long N = s.n();
    double* y = &s.gf[a];
    if (y[gfm::kEps * N] < 1.0e-12) y[gfm::kEps * N] = 1.0e-12;
    double g0 = P.cmu * P.reyg * P.epsr / (2.0 * P.taur) * (y[gfm::kK * N] * y[gfm::kK * N]) / y[gfm::kEps * N] * s.dnst[a];
    s.tmu[a] = g0;
    s.gama[a] = 2.0 / P.reyg * (s.tmu[a] + std::pow(s.t[a] / P.trdg, P.amu));
}

void prop_tke(CaseStore& s, long a) {
    const long N = s.n();
    double g = s.ug[a] * s.ug[a] + s.ug[a + N] * s.ug[a + N] + s.ug[a + 2 * N] * s.ug[a + 2 * N];
    s.gf[a + gfm::kK * N] = g > 1.0e-6 ? g : 1.0e-6;
    s.gf[a + gfm::kEps * N] = s.gf[a + gfm::kK * N] * s.gf[a + gfm::kK * N];
}

void prop_t2h(CaseStore& s, const gfm_params& P, long a) {
    s.gf[a + gfm::kH * s.n()] = gfm::t_to_enth(gfm::nist_host(), &s.gf[a], s.n(), s.t[a], P.t0, P.h_0);
}

namespace {

// splitmix64: deterministic per-cell noise for the perturbed initial state
uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
double unit_noise(uint64_t seed, uint64_t idx, uint64_t comp) {
    uint64_t h = splitmix64(seed ^ splitmix64(idx * 16 + comp));
    return ((double)(h >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;  // [-1,1)
}

// AREA_C (Grid3.f90:411-471) on the host arrays (1-based indices): 0 on a
// wall, times BA_F on a half-blocked cell, and on a cell with IBCELL >= 2
// times BA_F of a half-blocked neighbour two positions away along ix
double area_c(const CaseStore& s, int i, int j, int k, int ix) {
    auto IB = [&](int a, int b, int c) { return (int)s.ibcell[s.at(a, b, c)]; };
    const int ib = IB(i, j, k);
    if (ib == 1) return 0.0;
    double a = ix == 1 ? s.dr[j - 1] * s.rs[j - 1] * s.dz[k - 1]
                       : ix == 2 ? s.dx[i - 1] * s.dz[k - 1] : s.dx[i - 1] * s.dr[j - 1] * s.rs[j - 1];
    if (ib == 0) return a;
    if (ib <= -1) return a * s.ba_f[3 * (-ib - 1) + ix - 1];
    int nb = 0;
    if (ix == 1) {
        if (i <= s.mp - 2 && IB(i + 2, j, k) <= -1) nb = IB(i + 2, j, k);
        else if (i >= 4 && IB(i - 2, j, k) <= -1) nb = IB(i - 2, j, k);
    } else if (ix == 2) {
        if (j <= s.np - 2 && IB(i, j + 2, k) <= -1) nb = IB(i, j + 2, k);
        else if (j >= 4 && IB(i, j - 2, k) <= -1) nb = IB(i, j - 2, k);
    } else {
        if (k <= s.lp - 2 && IB(i, j, k + 2) <= -1) nb = IB(i, j, k + 2);
        else if (k >= 4 && IB(i, j, k - 2) <= -1) nb = IB(i, j, k - 2);
    }
    return nb <= -1 ? a * s.ba_f[3 * (-nb - 1) + ix - 1] : a;
}

// GRID3 coordinate line (Grid3.f90:79-109): X(1..i1)=x0, then linear to
// X(n-1)=x1 by repeated addition of DEL, X(n)=X(n-1), DX(I)=X(I+1)-X(I-1).
void coord_line(int n, double len, std::vector<double>& x, std::vector<double>& dx) {
    x.assign(n, 0.0);
    dx.assign(n, 0.0);
    const int i1 = 3, i2 = n - 1;
    for (int i = 1; i <= i1; ++i) x[i - 1] = 0.0;
    double del = (len - x[i1 - 1]) / (i2 - i1);
    for (int i = i1 + 1; i <= i2; ++i) x[i - 1] = x[i - 2] + del;
    for (int i = 1; i <= n - 1; ++i) x[i - 1] = x[i - 1] / 1.0;   // /R0, R0=1
    x[n - 1] = x[n - 2];
    dx[0] = 0.0;
    for (int i = 2; i <= n - 1; ++i) dx[i - 1] = x[i] - x[i - 2];
    dx[n - 1] = 0.0;
}

// snap an opening [a,b] on a uniform line of `ncell` cells of width h to a
// run of whole cells; returns 1-based first cell and count
void snap(double a, double b, double h, int ncell, int& first, int& count) {
    count = (int)std::lround((b - a) / h);
    if (count < 1) count = 1;
    if (count > ncell) count = ncell;
    double c = 0.5 * (a + b) / h;
    first = (int)std::lround(c - 0.5 * count) + 1;
    if (first < 1) first = 1;
    if (first + count - 1 > ncell) first = ncell - count + 1;
}

bool read_kinetics(const char* path, int nr0, CaseStore& s, double h_0) {
    FILE* fp = std::fopen(path, "r");
    if (!fp) return false;
    char line[512];
    auto next = [&](double* a, double* b, double* c) -> bool {
        while (std::fgets(line, sizeof line, fp)) {
            if (std::sscanf(line, "%lf %lf %lf", a, b, c) == 3) return true;
            return false;   // header line
        }
        return false;
    };
    s.rtim.resize(nr0); s.delrt.resize(nr0); s.hrt.resize(nr0);
    s.delr.resize(nr0); s.timed.resize(nr0); s.hrd.resize(nr0);
    const double chrd = 0.166;
    if (!std::fgets(line, sizeof line, fp)) { std::fclose(fp); return false; }   // header
    for (int i = 0; i < nr0; ++i) {
        if (!next(&s.rtim[i], &s.delrt[i], &s.hrt[i])) { std::fclose(fp); return false; }
        s.rtim[i] = s.rtim[i] * 0.7;                       // Setup.f90:874
        s.hrt[i] = chrd * s.hrt[i] / h_0 / gfm::kWf;       // Setup.f90:876
    }
    if (!std::fgets(line, sizeof line, fp)) { std::fclose(fp); return false; }   // header
    for (int i = 0; i < nr0; ++i) {
        if (!next(&s.delr[i], &s.timed[i], &s.hrd[i])) { std::fclose(fp); return false; }
        s.timed[i] = s.timed[i] * 0.7;                     // Setup.f90:884
        s.hrd[i] = chrd * s.hrd[i] / h_0 / gfm::kWf;       // Setup.f90:886
    }
    std::fclose(fp);
    return true;
}

// melt_surf_T (Initsv.f90:394-547): the melt-surface cells of the z=2 slab
// take the it####t.dat temperatures, relaxed against T_surf_prev with the
// mean surface temperature preserved; the relaxation factor shrinks by 0.8
// while the relaxed maximum exceeds the mean by 250 K or more.
void melt_surf_t(CaseStore& s, const CaseInputs& in, const gfm_params& P, double area_melt_surf, bool restart) {
    const int mz = s.mp / 2, nz = s.np / 2;
    auto TG = [&](std::vector<double>& v, int i, int j) -> double& { return v[(i - 1) + (long)mz * (j - 1)]; };
    std::vector<double> tgs(in.tgs);
    if (!restart) s.t_surf_prev.assign((size_t)mz * nz, in.surf_t);
    const std::vector<double> tgs_bak(tgs);
    double rf = in.rf_tsurf, rfc = 1.0 - rf;
    const double area0 = 1.0;
    for (;;) {
        double relaxed = 0.0, tmax = 0.0;
        for (int j = 4; j <= s.np - 2; j += 2)
            for (int i = 4; i <= s.mp - 2; i += 2) {
                if (s.ibcell[s.at(i, j, 2)] != 4) continue;
                double& g = TG(tgs, i / 2, j / 2);
                if (in.itn > 0) {
                    g = rf * g + rfc * TG(s.t_surf_prev, i / 2, j / 2);
                    if (g > P.t_mx * P.t0) g = P.t_mx * P.t0;
                    relaxed = relaxed + g * s.dx[i - 1] * s.dr[j - 1] * area0;
                    tmax = std::fmax(tmax, g);
                }
                s.t[s.at(i, j, 2)] = g / P.t0;
            }
        if (in.itn <= 0) break;
        relaxed = relaxed / area_melt_surf;
        double check = 0.0;
        tmax = 0.0;
        for (int j = 4; j <= s.np - 2; j += 2)
            for (int i = 4; i <= s.mp - 2; i += 2) {
                if (s.ibcell[s.at(i, j, 2)] != 4) continue;
                double& g = TG(tgs, i / 2, j / 2);
                g = g * in.surf_t / relaxed;
                check = check + g * s.dx[i - 1] * s.dr[j - 1] * area0;
                tmax = std::fmax(tmax, g);
                s.t[s.at(i, j, 2)] = g / P.t0;
            }
        relaxed = check / area_melt_surf;
        if ((tmax - relaxed) < 250.0 || rf < 0.1) break;
        rf = rf * 0.8;
        rfc = 1 - rf;
        tgs = tgs_bak;
    }
    s.t_surf_prev = tgs;
}

}  // namespace

int finish_case(CaseStore* S, const CaseInputs& in, const char* kinetic_path, gfm_case* out,
                gfm_case_summary* sum) {
    CaseStore& s = *S;
    const int mp = s.mp, np = s.np, lp = s.lp;
    const long N = s.n();
    auto IB = [&](int i, int j, int k) -> int16_t& { return s.ibcell[s.at(i, j, k)]; };
    auto fail = [&](int rc) { delete S; std::memset(out, 0, sizeof *out); return rc; };

    // NCELLS and the 27-neighbour face/edge propagation (Grid3.f90:259-275),
    // loop order I, J, K as in the Fortran
    int ncells = 0;
    for (int i = 2; i <= mp; i += 2)
        for (int j = 2; j <= np; j += 2)
            for (int k = 2; k <= lp; k += 2) {
                int ibc1 = IB(i, j, k);
                if (ibc1 <= 0) { ++ncells; continue; }
                for (int i1 = i - 1; i1 <= i + 1; ++i1)
                    for (int j1 = j - 1; j1 <= j + 1; ++j1)
                        for (int k1 = k - 1; k1 <= k + 1; ++k1) {
                            if (i1 > mp || j1 > np || k1 > lp) continue;
                            if (IB(i1, j1, k1) != 1) IB(i1, j1, k1) = (int16_t)ibc1;
                        }
            }
    // melt-surface area (Grid3.f90:288-293)
    const double area0 = 1.0;
    double area_melt_surf = 0.0;
    int n_melt = 0;
    for (int i = 2; i <= mp; i += 2)
        for (int j = 2; j <= np; j += 2)
            if (IB(i, j, 2) == 4) { area_melt_surf = area_melt_surf + s.dx[i - 1] * s.dr[j - 1] * area0; ++n_melt; }
    if (n_melt > 0 && !in.have_it) return fail(GFM_E_ARG);   // melt_surf_T needs it####t.dat

    // ---- SETUP constants (Setup.f90:27-217, 542-731) -------------------------
    gfm_params& P = out->params;
    std::memset(&P, 0, sizeof P);
    const double t0 = gfm::kT0;
    const double h_0 = 1.0057e+3 * (5.0e+2 - 298.15);                       // Var_mod.f90:184
    const double wt0 = 1.0 / (0.5 / 16.0426 + 0.0 / 44.0098 + 0.0 / 18.0152 + 0.49 / 31.9988 + 0.01 / 28.0134);
    const double pg0 = in.pg0;
    const double gmfr = in.gmfr;
    const double r0 = 1.0;
    const double dnst0 = pg0 * wt0 / gfm::kRu / t0;
    const double ug0 = gmfr / dnst0 / area0;
    const double gmu_ref = in.gmu_ref * std::pow(gfm::kTl00 / 2.98e+2, 0.0);   // Setup.f90:660, AMU=0
    const double tk0 = gfm::kCtea * (ug0 * ug0);
    const double epsi0 = gfm::kCtda * (tk0 * tk0);
    const double reyg = 2.0 * dnst0 * ug0 * r0 / gmu_ref;
    P.t0 = t0; P.h_0 = h_0; P.dnst0 = dnst0; P.ug0 = ug0; P.gmfr = gmfr; P.pg0 = pg0; P.r0 = r0;
    P.reyg = reyg; P.reyg2 = reyg / 2.0;
    P.epsr = tk0 / (ug0 * ug0);
    P.taur = epsi0 * r0 / (tk0 * ug0);
    P.eun = pg0 / (dnst0 * (ug0 * ug0));
    P.qr0 = h_0 * dnst0 * ug0 / r0;
    P.q0 = in.q0_jkg / h_0;
    P.tk0 = tk0;
    P.gra[0] = 0.0 / ug0 / ug0 * r0; P.gra[1] = 0.0 / ug0 / ug0 * r0; P.gra[2] = -9.80621 / ug0 / ug0 * r0;
    P.amu = 0.0;
    P.trdg = 298.15 / 5.0e+2;
    P.wt0 = wt0;
    P.stoich = 2.0 * 31.9988 / 16.0426;
    P.cmu = gfm::kCmu; P.ct1 = gfm::kCt1; P.ct2 = gfm::kCt2;
    P.p_mx = 0.2; P.p_mn = -0.6;
    P.t_mx = 3.0e+3 / t0; P.t_mn = 2.0e+2 / 5.0e+2;
    P.u_mx = 1.0e+3 / ug0; P.u_mn = -P.u_mx;
    P.f_mx = 1.5; P.f_mn = 0.8;
    for (int i = 0; i < 21; ++i) { P.rf[i] = in.rf[i]; P.rfl[i] = in.rfl[i]; }
    for (int i = 0; i < 12; ++i) P.sigma[i] = in.sigma[i];
    for (int i = 0; i < 20; ++i) P.ntimesg[i] = in.ntimesg[i];
    P.rf_hsource = in.rf_hsource;
    P.react = in.react; P.turb = 1;
    P.wall_sink = in.wall_sink; P.h_g = in.h_g;
    P.rad_emission = in.rad_emission; P.rad_qe_frequency = 10;
    P.sig = gfm::kSig; P.ri = in.ri; P.hck = gfm::kHck;
    P.bgcon = in.bgcon; P.maxgi = in.maxgi;
    P.adi_mode = in.adi_mode; P.precision = in.precision;
    P.gas_model = in.gas_model; P.maxms = in.maxms; P.ntimesm = in.ntimesm; P.irstypm = in.irstypm;
    P.bmcon = in.bmcon; P.ssigma = in.ssigma; P.rfm = in.rfm; P.rfm_soot = in.rfm_soot;
    P.rf_soot_form = in.rf_soot_form; P.rf_soot_oxid = in.rf_soot_oxid;
    P.soot_cap = in.soot_cap; P.t0_sf = in.t0_sf; P.t0_so = in.t0_so;
    P.aform = in.aform; P.aoxid = in.aoxid;
    P.esf_r = in.esf / gfm::kRu; P.eso_r = in.eso / gfm::kRu;   // Setup.f90:416-417

    // ---- fields at allocation (Setup.f90:747-779) -----------------------------
    s.p.assign(N, 0.0); s.t.assign(N, 1.0); s.dnst.assign(N, 1.0); s.theta.assign(N, 1.0);
    s.tmu.assign(N, 0.0); s.gama.assign(N, 0.0); s.crate.assign(N, 0.0); s.hrate.assign(N, 0.0);
    s.bs_hprev.assign(N, 0.0);
    s.ug.assign(3 * N, 0.0); s.gf.assign(9 * N, 0.0);
    const int mz = mp / 2, nz = np / 2;
    const long ncell_arr = (long)mz * nz * (lp / 2);
    s.qa.assign(ncell_arr, 0.0); s.qe.assign(ncell_arr, 0.0);
    s.t_surf_prev.assign((size_t)mz * nz, 0.0);
    auto GF = [&](int i, int j, int k, int l) -> double& { return s.gf[s.at(i, j, k) + (long)l * N]; };
    auto UG = [&](int i, int j, int k, int l) -> double& { return s.ug[s.at(i, j, k) + (long)l * N]; };

    // ---- SBC: inlet states and inlet faces (Sbc.f90:57-269, 365-386) ---------
    if (in.i_ref < 2 || in.i_ref > mp || in.j_ref < 2 || in.j_ref > np || in.k_ref < 2 || in.k_ref > lp ||
        IB(in.i_ref, in.j_ref, in.k_ref) != 2)
        return fail(GFM_E_ARG);   // the pressure reference must be an inlet cell (Sbc.f90:58-63)
    const double p_ref = in.p_ref_pa / pg0;
    double fr_f = 0, fr_ox = 0, fr_n2 = 0, q_h_in = 0;
    std::vector<char> done(N, 0);   // plays the role of the temporary IBCELL=20 mark
    for (const InletBlock& b : in.inlets) {
        if (b.iu < 1 || b.iu > 3 || b.i1 < 2 || b.j1 < 2 || b.k1 < 2 || b.i2 > mp || b.j2 > np || b.k2 > lp)
            return fail(GFM_E_ARG);
        const double T_0 = b.t_k / t0, U_0 = b.u / ug0, V_0 = b.v / ug0, W_0 = b.w / ug0;
        for (int i = b.i1; i <= b.i2; i += 2)
            for (int j = b.j1; j <= b.j2; j += 2)
                for (int k = b.k1; k <= b.k2; k += 2) {
                    long a = s.at(i, j, k);
                    if (IB(i, j, k) != 2 || done[a]) continue;
                    done[a] = 1;
                    s.p[a] = p_ref;
                    s.t[a] = T_0;
                    GF(i, j, k, gfm::kYF) = b.yf; GF(i, j, k, gfm::kYCO2) = b.yco2;
                    GF(i, j, k, gfm::kYH2O) = b.yh2o; GF(i, j, k, gfm::kYO2) = b.yox;
                    GF(i, j, k, gfm::kYN2) = b.yn2;
                    prop_dnst(s, P, a);
                    UG(i, j, k, 0) = U_0; UG(i, j, k, 1) = V_0; UG(i, j, k, 2) = W_0;
                    prop_tke(s, a);
                    prop_ther(s, P, a);
                    prop_t2h(s, P, a);
                    double g0 = s.theta[a] * s.dnst[a] * dnst0;
                    // AREA_C(I,J,K,IU)*AREA0 of the inlet cell (Sbc.f90:138)
                    const double un = b.iu == 2 ? V_0 : b.iu == 3 ? W_0 : U_0;
                    g0 = g0 * std::fabs(un) * ug0 * (area_c(s, i, j, k, b.iu) * area0);
                    fr_f += g0 * GF(i, j, k, gfm::kYF);
                    fr_ox += g0 * GF(i, j, k, gfm::kYO2);
                    fr_n2 += g0 * GF(i, j, k, gfm::kYN2);
                    q_h_in += GF(i, j, k, gfm::kH) * h_0 * g0;
                }
        // SBC1: interpolate the faces between the block's inlet cells
        auto sbc1 = [&](int ia, int ja, int ka, int ib, int jb, int kb, int i, int j, int k, double f1) {
            double f2 = 1.0 - f1;
            long A = s.at(ia, ja, ka), B = s.at(ib, jb, kb), C = s.at(i, j, k);
            s.p[C] = f1 * s.p[A] + f2 * s.p[B];
            s.t[C] = f1 * s.t[A] + f2 * s.t[B];
            for (int l = 0; l < 9; ++l) {
                if (l < 3) s.ug[C + l * N] = f1 * s.ug[A + l * N] + f2 * s.ug[B + l * N];
                s.gf[C + l * N] = f1 * s.gf[A + l * N] + f2 * s.gf[B + l * N];
            }
            prop_dnst(s, P, C);
            s.theta[C] = f1 * s.theta[A] + f2 * s.theta[B];
            s.tmu[C] = f1 * s.tmu[A] + f2 * s.tmu[B];
            s.gama[C] = f1 * s.gama[A] + f2 * s.gama[B];
        };
        // SBC3 (Sbc.f90:491-522): copy onto the inlet face planes
        auto sbc3 = [&](int ia, int ja, int ka, int ib, int jb, int kb) {
            long A = s.at(ia, ja, ka), B = s.at(ib, jb, kb);
            for (int l = 0; l < 3; ++l) s.ug[B + l * N] = s.ug[A + l * N];
            s.p[B] = s.p[A]; s.t[B] = s.t[A];
            for (int l = 0; l < 9; ++l) s.gf[B + l * N] = s.gf[A + l * N];
            s.dnst[B] = s.dnst[A]; s.theta[B] = s.theta[A]; s.tmu[B] = s.tmu[A]; s.gama[B] = s.gama[A];
        };
        if (b.iu == 1) {   // Sbc.f90:179-206
            const int i = b.i1;
            if (b.k2 > b.k1)
                for (int k = b.k1 + 1; k <= b.k2 - 1; k += 2)
                    for (int j = b.j1; j <= b.j2; j += 2)
                        sbc1(i, j, k + 1, i, j, k - 1, i, j, k, (s.z[k - 1] - s.z[k - 2]) / s.dz[k - 1]);
            if (b.j2 > b.j1)
                for (int j = b.j1 + 1; j <= b.j2 - 1; j += 2)
                    for (int k = b.k1; k <= b.k2; ++k)
                        sbc1(i, j + 1, k, i, j - 1, k, i, j, k, (s.r[j - 1] - s.r[j - 2]) / s.dr[j - 1]);
            for (int j = b.j1; j <= b.j2; ++j)
                for (int k = b.k1; k <= b.k2; ++k) {
                    if (i < mp && IB(i + 1, j, k) == 2) sbc3(i, j, k, i + 1, j, k);
                    if (i > 2 && IB(i - 1, j, k) == 2) sbc3(i, j, k, i - 1, j, k);
                }
        } else if (b.iu == 2) {   // Sbc.f90:208-235
            const int j = b.j1;
            if (b.k2 > b.k1)
                for (int k = b.k1 + 1; k <= b.k2 - 1; k += 2)
                    for (int i = b.i1; i <= b.i2; i += 2)
                        sbc1(i, j, k + 1, i, j, k - 1, i, j, k, (s.z[k - 1] - s.z[k - 2]) / s.dz[k - 1]);
            if (b.i2 > b.i1)
                for (int i = b.i1 + 1; i <= b.i2 - 1; i += 2)
                    for (int k = b.k1; k <= b.k2; ++k)
                        sbc1(i + 1, j, k, i - 1, j, k, i, j, k, (s.x[i - 1] - s.x[i - 2]) / s.dx[i - 1]);
            for (int i = b.i1; i <= b.i2; ++i)
                for (int k = b.k1; k <= b.k2; ++k) {
                    if (j < np && IB(i, j + 1, k) == 2) sbc3(i, j, k, i, j + 1, k);
                    if (j > 2 && IB(i, j - 1, k) == 2) sbc3(i, j, k, i, j - 1, k);
                }
        } else {   // Sbc.f90:237-264
            const int k = b.k1;
            if (b.j2 > b.j1)
                for (int j = b.j1 + 1; j <= b.j2 - 1; j += 2)
                    for (int i = b.i1; i <= b.i2; i += 2)
                        sbc1(i, j + 1, k, i, j - 1, k, i, j, k, (s.r[j - 1] - s.r[j - 2]) / s.dr[j - 1]);
            if (b.i2 > b.i1)
                for (int i = b.i1 + 1; i <= b.i2 - 1; i += 2)
                    for (int j = b.j1; j <= b.j2; ++j)
                        sbc1(i + 1, j, k, i - 1, j, k, i, j, k, (s.x[i - 1] - s.x[i - 2]) / s.dx[i - 1]);
            for (int i = b.i1; i <= b.i2; ++i)
                for (int j = b.j1; j <= b.j2; ++j) {
                    if (k < lp && IB(i, j, k + 1) == 2) sbc3(i, j, k, i, j, k + 1);
                    if (k > 2 && IB(i, j, k - 1) == 2) sbc3(i, j, k, i, j, k - 1);
                }
        }
    }
    const double gfin = fr_f + fr_ox + fr_n2;
    if (!(gfin > 0.0)) return fail(GFM_E_ARG);
    const double gfin0 = gfin / gmfr;
    // est_out_mass_frac (Sbc.f90:566-576)
    const double yn2_out = fr_n2 / gfin;
    const double yh2o_out = (2 * fr_f * gfm::kWh2o / gfm::kWf) / gfin;
    const double yco2_out = (fr_f * gfm::kWco2 / gfm::kWf) / gfin;
    const double yo2_out = (fr_ox - 2 * fr_f * gfm::kWo2 / gfm::kWf) / gfin;

    // ---- INITSV: fresh start or restart (Initsv.f90:31-62) --------------------
    gfm_fields& F = out->fields;
    std::memset(&F, 0, sizeof F);
    F.factor = 1.0; F.fadj = 0.0;
    gfm_restart_tail& tail = out->tail;
    std::memset(&tail, 0, sizeof tail);
    tail.mz = mz; tail.nz = nz;
    tail.interval_rad = in.interval_rad;
    tail.itr_gend = in.initial_gitr;
    int maxgi = in.maxgi;
    const bool restart = in.rg_path != nullptr;
    if (restart) {
        int rc = read_restart(in.rg_path, s, P, F, tail, maxgi);
        if (rc == GFM_OK && in.rr_path) rc = read_rad_restart(in.rr_path, s, P);
        if (rc != GFM_OK) return fail(rc);
        P.maxgi = maxgi;
        if (in.have_it) melt_surf_t(s, in, P, area_melt_surf, true);
    } else {
        if (in.have_it) melt_surf_t(s, in, P, area_melt_surf, false);
        // gen_initial_guess with a seeded perturbation (Initsv.f90:97-162)
        const double T_init = in.t_init_k / t0;
        const double amp = in.noise_amp;
        for (int i = 2; i <= mp; i += 2)
            for (int j = 2; j <= np; j += 2)
                for (int k = 2; k <= lp; k += 2) {
                    int ibc = IB(i, j, k);
                    if (ibc == 2) continue;
                    long a = s.at(i, j, k);
                    double nz5[5] = {0, 0, 0, 0, 0};
                    if (ibc == 0 && amp != 0.0)
                        for (int c = 0; c < 5; ++c) nz5[c] = amp * unit_noise(in.seed, (uint64_t)a, (uint64_t)c);
                    GF(i, j, k, gfm::kYF) = 0;
                    GF(i, j, k, gfm::kYO2) = yo2_out * (1.0 + nz5[1]);
                    GF(i, j, k, gfm::kYCO2) = yco2_out * (1.0 + nz5[2]);
                    GF(i, j, k, gfm::kYH2O) = yh2o_out * (1.0 + nz5[3]);
                    GF(i, j, k, gfm::kYN2) = yn2_out * (1.0 + nz5[4]);
                    if (ibc == 1) {
                        s.t[a] = T_init;
                        prop_t2h(s, P, a);
                        continue;
                    }
                    UG(i, j, k, 0) = 0; UG(i, j, k, 1) = 0; UG(i, j, k, 2) = 0;
                    s.theta[a] = 1.0;
                    if (ibc != 4) s.t[a] = T_init * (1.0 + nz5[0]);
                    prop_t2h(s, P, a);
                    prop_tke(s, a);
                    prop_dnst(s, P, a);
                    prop_ther(s, P, a);
                }
    }

    // ---- boundary patches (prepare_for_wall_radiation_calculation,
    // Qwall.f90:54-520).  The cell map is copied to MAPB and each exit's
    // tunnel through the wall is closed: the exit moves to the tunnel's inner
    // end and the rest of the tunnel becomes wall (steps 1-2, Qwall.f90:72-
    // 346).  Patches are the faces with MAPB >= 1 next to an open position
    // (steps 3-5, Qwall.f90:395-513).  b_T is the fixed wall temperature for
    // wall patches and the melt-cell temperature for melt-surface patches
    // (Rad_emis.f90:196-210); the wall sink reads no other patch temperature.
    std::vector<int16_t> mapb(s.ibcell);
    auto MB = [&](int i, int j, int k) -> int16_t& { return mapb[s.at(i, j, k)]; };
    auto fill = [&](int ia, int ib, int ja, int jb, int ka, int kb, int16_t v) {
        for (int i = ia; i <= ib; ++i)
            for (int j = ja; j <= jb; ++j)
                for (int k = ka; k <= kb; ++k) MB(i, j, k) = v;
    };
    // extent of an exit from one corner: the last position of the run of 3s
    // along one axis (the reference leaves the end unset when the run reaches
    // the grid's edge; it then ends there)
    auto run_end = [&](int i, int j, int k, int di, int dj, int dk, int lim) {
        int a = i, b = j, c = k;
        for (;;) {
            const int n = (di ? a : dj ? b : c) + 2;
            if (n > lim) return n - 2;
            if (MB(a + 2 * di, b + 2 * dj, c + 2 * dk) != 3) return n - 2;
            a += 2 * di; b += 2 * dj; c += 2 * dk;
        }
    };
    for (int face = 0; face < 5; ++face) {
        // back (i=2), front (i=MP), sides (j=2, j=NP) and top (k=LP) walls
        const int ax = face < 2 ? 0 : face < 4 ? 1 : 2;
        const bool lo = face == 0 || face == 2;
        const int fixed = ax == 0 ? (lo ? 2 : mp) : ax == 1 ? (lo ? 2 : np) : lp;
        const int na = ax == 0 ? np : mp, nb = ax == 2 ? np : lp;   // the two other axes
        for (int u = 2; u <= na; u += 2)
            for (int v = 2; v <= nb; v += 2) {
                int i, j, k;
                if (ax == 0) { i = fixed; j = u; k = v; } else if (ax == 1) { i = u; j = fixed; k = v; } else { i = u; j = v; k = fixed; }
                if (MB(i, j, k) != 3) continue;
                // the exit's rectangle in the wall plane
                int a0, a1, b0, b1;
                if (ax == 0) { a0 = j; a1 = run_end(i, j, k, 0, 1, 0, np); b0 = k; b1 = run_end(i, j, k, 0, 0, 1, lp); }
                else if (ax == 1) { a0 = i; a1 = run_end(i, j, k, 1, 0, 0, mp); b0 = k; b1 = run_end(i, j, k, 0, 0, 1, lp); }
                else { a0 = i; a1 = run_end(i, j, k, 1, 0, 0, mp); b0 = j; b1 = run_end(i, j, k, 0, 1, 0, np); }
                // the interior end: the first layer in from the wall where a
                // position diagonally outside a corner of the rectangle is open
                const int n = ax == 0 ? mp : ax == 1 ? np : lp;
                auto open_at = [&](int w) {
                    // positions past the grid's edge count as closed
                    auto at = [&](int p, int q) -> int {
                        int i = w, j = p, k = q;
                        if (ax == 1) { i = p; j = w; k = q; } else if (ax == 2) { i = p; j = q; k = w; }
                        if (i < 1 || i > mp || j < 1 || j > np || k < 1 || k > lp) return 1;
                        return MB(i, j, k);
                    };
                    return at(a0 - 2, b0 - 2) == 0 || at(a1 + 2, b1 + 2) == 0 || at(a0 - 2, b1 + 2) == 0 ||
                           at(a1 + 2, b0 - 2) == 0;
                };
                int wnew = -1;
                if (lo) {
                    for (int w = 4; w <= n; w += 2) if (open_at(w)) { wnew = w - 2; break; }
                } else {
                    for (int w = n - 2; w >= 2; w -= 2) if (open_at(w)) { wnew = w + 2; break; }
                }
                if (wnew < 0) continue;   // no inner end: the map stays as read
                // exit at the inner end (two positions), wall in the rest of the tunnel
                int e0 = lo ? wnew : wnew - 1, e1 = lo ? wnew + 1 : wnew;
                int w0 = lo ? 2 : wnew + 1, w1 = lo ? wnew - 1 : n;
                if (ax == 0) { fill(e0, e1, a0, a1, b0, b1, 3); fill(w0, w1, a0, a1, b0, b1, 1); }
                else if (ax == 1) { fill(a0, a1, e0, e1, b0, b1, 3); fill(a0, a1, w0, w1, b0, b1, 1); }
                else { fill(a0, a1, b0, b1, e0, e1, 3); fill(a0, a1, b0, b1, w0, w1, 1); }
            }
    }
    auto add_patch = [&](int typ, int ori, int dir, int i, int j, int k) {
        s.b_typ.push_back((int16_t)typ); s.b_orient.push_back((int16_t)ori); s.b_direct.push_back((int16_t)dir);
        s.b_i.push_back((int16_t)i); s.b_j.push_back((int16_t)j); s.b_k.push_back((int16_t)k);
        double bt = in.t_wall_k;
        if (typ == 4) {   // the closed side of the patch holds the melt cell
            int ic = i, jc = j, kc = k;
            int sgn = dir == 0 ? -1 : 1;
            if (ori == 1) ic += sgn; else if (ori == 2) jc += sgn; else kc += sgn;
            bt = s.t[s.at(ic, jc, kc)] * t0;
        }
        s.b_t.push_back(bt);
    };
    for (int k = 2; k <= lp; k += 2)
        for (int j = 2; j <= np; j += 2)
            for (int i = 3; i <= mp - 1; i += 2) {
                int m = MB(i, j, k);
                if (m < 1) continue;
                if (MB(i - 1, j, k) > 0 && MB(i + 1, j, k) > 0) continue;
                add_patch(m, 1, MB(i + 1, j, k) == 0 ? 0 : 1, i, j, k);
            }
    for (int k = 2; k <= lp; k += 2)
        for (int j = 3; j <= np - 1; j += 2)
            for (int i = 2; i <= mp; i += 2) {
                int m = MB(i, j, k);
                if (m < 1) continue;
                if (MB(i, j - 1, k) > 0 && MB(i, j + 1, k) > 0) continue;
                add_patch(m, 2, MB(i, j + 1, k) == 0 ? 0 : 1, i, j, k);
            }
    for (int k = 3; k <= lp - 1; k += 2)
        for (int j = 2; j <= np; j += 2)
            for (int i = 2; i <= mp; i += 2) {
                int m = MB(i, j, k);
                if (m < 1) continue;
                if (MB(i, j, k - 1) > 0 && MB(i, j, k + 1) > 0) continue;
                add_patch(m, 3, MB(i, j, k + 1) == 0 ? 0 : 1, i, j, k);
            }

    // ---- kinetics table and radiation bands -----------------------------------
    if (!kinetic_path || !read_kinetics(kinetic_path, in.nr0, s, h_0)) return fail(GFM_E_IO);
    const int nwl = (int)in.wl_m.size();
    if (nwl < 1 || nwl > 16 || (int)in.kappa.size() != nwl) return fail(GFM_E_ARG);
    s.wl = in.wl_m;
    s.akl0 = in.kappa;

    // ---- fill the public structs -----------------------------------------------
    gfm_grid& G = out->grid;
    G.mp = mp; G.np = np; G.lp = lp;
    G.x = s.x.data(); G.dx = s.dx.data(); G.r = s.r.data(); G.dr = s.dr.data(); G.rs = s.rs.data();
    G.z = s.z.data(); G.dz = s.dz.data();
    G.ibcell = s.ibcell.data();
    G.ncells = ncells;
    G.i_ref = in.i_ref; G.j_ref = in.j_ref; G.k_ref = in.k_ref;
    G.p_ref = p_ref;
    G.b_cnt = (int)s.b_typ.size();
    G.b_typ = s.b_typ.data(); G.b_i = s.b_i.data(); G.b_j = s.b_j.data(); G.b_k = s.b_k.data();
    G.b_orient = s.b_orient.data(); G.b_direct = s.b_direct.data(); G.b_t = s.b_t.data();
    G.nr0 = in.nr0;
    G.rtim = s.rtim.data(); G.delrt = s.delrt.data(); G.hrt = s.hrt.data();
    G.delr = s.delr.data(); G.timed = s.timed.data(); G.hrd = s.hrd.data();
    G.nwl = nwl; G.wl = s.wl.data(); G.akl0 = s.akl0.data();
    for (int q = 0; q < 2; ++q) G.bv_f[q] = s.bv_f[q];
    for (int q = 0; q < 6; ++q) G.ba_f[q] = s.ba_f[q];
    out->wall = in.wall;

    F.p = s.p.data(); F.t = s.t.data(); F.dnst = s.dnst.data(); F.theta = s.theta.data();
    F.tmu = s.tmu.data(); F.gama = s.gama.data(); F.crate = s.crate.data(); F.hrate = s.hrate.data();
    F.bs_hprev = s.bs_hprev.data(); F.ug = s.ug.data(); F.gf = s.gf.data();
    F.qa = s.qa.data(); F.qe = s.qe.data();
    F.gfin0 = gfin0; F.q_h_in = q_h_in;
    tail.t_surf_prev = s.t_surf_prev.data();
    out->priv = S;

    if (sum) {
        sum->ncells = ncells;
        sum->area_melt_surf = area_melt_surf;
        sum->fr_f = fr_f; sum->fr_ox = fr_ox; sum->fr_n2 = fr_n2;
        sum->heat_in_fuel = fr_f * P.q0 * h_0;
        sum->q_h_in = q_h_in;
        sum->gmfr = gmfr; sum->gfin0 = gfin0;
        sum->interval_rad = tail.interval_rad;
        sum->n_inlet_blocks = (int)in.inlets.size();
        sum->n_melt_cells = n_melt;
        sum->restarted = restart ? 1 : 0;
        sum->itr_gas = F.itr_gas;
    }
    return GFM_OK;
}

}  // namespace host
}  // namespace gfm

using gfm::host::CaseInputs;
using gfm::host::CaseStore;
using gfm::host::InletBlock;

namespace gfm {
namespace host {

// The synthetic furnace of a gfm_case_spec as the inputs a case directory
// would give: grid, cell map (before the propagation) and CaseInputs.
int synth_inputs(const gfm_case_spec* sp, CaseStore& s, CaseInputs& in) {
    if (sp->nx < 4 || sp->ny < 4 || sp->nz < 4 || sp->nx > 4096 || sp->ny > 4096 || sp->nz > 4096)
        return GFM_E_ARG;
    if (sp->n_inlets < 1 || sp->n_inlets > 8 || sp->nwl < 1 || sp->nwl > 16) return GFM_E_ARG;
    if (!(sp->lx > 0 && sp->ly > 0 && sp->lz > 0)) return GFM_E_ARG;

    const int mp = 2 * sp->nx + 4, np = 2 * sp->ny + 4, lp = 2 * sp->nz + 4;
    s.mp = mp; s.np = np; s.lp = lp;
    const long N = s.n();

    // ---- GRID3 coordinates (Grid3.f90:76-226) -------------------------------
    coord_line(mp, sp->lx, s.x, s.dx);
    coord_line(np, sp->ly, s.r, s.dr);
    coord_line(lp, sp->lz, s.z, s.dz);
    s.rs.assign(np, 1.0);                        // cartesian: RS=1 (Grid3.f90:166)

    // ---- cell map: walls, inlets on x=0, exit on x=lx -----------------------
    s.ibcell.assign(N, 0);
    auto IB = [&](int i, int j, int k) -> int16_t& { return s.ibcell[s.at(i, j, k)]; };
    for (int k = 2; k <= lp; k += 2)
        for (int j = 2; j <= np; j += 2)
            for (int i = 2; i <= mp; i += 2)
                if (i == 2 || i == mp || j == 2 || j == np || k == 2 || k == lp) IB(i, j, k) = 1;
    const double hy = sp->ly / sp->ny, hz = sp->lz / sp->nz;
    in.inlets.resize(sp->n_inlets);
    for (int n = 0; n < sp->n_inlets; ++n) {
        const gfm_inlet_spec& is = sp->inlets[n];
        InletBlock& b = in.inlets[n];
        int fy, cy, fz, cz;
        snap(is.y0, is.y1, hy, sp->ny, fy, cy);
        snap(is.z0, is.z1, hz, sp->nz, fz, cz);
        b.i1 = b.i2 = 2; b.iu = 1;
        b.j1 = 2 * fy + 2; b.j2 = 2 * (fy + cy - 1) + 2;
        b.k1 = 2 * fz + 2; b.k2 = 2 * (fz + cz - 1) + 2;
        double a_nom = (is.y1 - is.y0) * (is.z1 - is.z0);
        double a_snap = cy * hy * cz * hz;
        double jit = 1.0;
        if (sp->inlet_jitter > 0) jit = 1.0 + sp->inlet_jitter * unit_noise(sp->seed, 1000003ull + n, 7);
        b.u = is.u_ms * a_nom / a_snap * jit;
        b.v = b.w = 0.0;
        b.t_k = is.t_k; b.yf = is.yf; b.yox = is.yo2; b.yn2 = is.yn2; b.yco2 = is.yco2; b.yh2o = is.yh2o; b.yck = 0.0;
        for (int k = b.k1; k <= b.k2; k += 2)
            for (int j = b.j1; j <= b.j2; j += 2) IB(2, j, k) = 2;
    }
    {
        int fy, cy, fz, cz;
        snap(sp->exit_y0, sp->exit_y1, hy, sp->ny, fy, cy);
        snap(sp->exit_z0, sp->exit_z1, hz, sp->nz, fz, cz);
        for (int k = 2 * fz + 2; k <= 2 * (fz + cz - 1) + 2; k += 2)
            for (int j = 2 * fy + 2; j <= 2 * (fy + cy - 1) + 2; j += 2) IB(mp, j, k) = 3;
        // the flue's exhaust entry: x-normal patches facing -x, at a fixed
        // 1473 K (the flue temperature of the shipped TC21 case 0041)
        gfm_wall_spec& w = in.wall;
        w.nex = 1;
        w.exh_i1[0] = mp; w.exh_j1[0] = 2 * fy + 2; w.exh_k1[0] = 2 * fz + 2;
        w.exh_i2[0] = mp; w.exh_j2[0] = 2 * (fy + cy - 1) + 2; w.exh_k2[0] = 2 * (fz + cz - 1) + 2;
        w.exh_orient[0] = 1; w.exh_direct[0] = 1; w.exh_type[0] = 1;
        w.exh_frac[0] = 0.9; w.exh_fixed[0] = 1473.0;
        w.eps_c = 0.9;   // crown emissivity of the synthetic furnace
        w.have_crown = 0;
    }

    // ---- SETUP inputs --------------------------------------------------------
    const double pg0 = sp->pg0 > 0 ? sp->pg0 : 1.01325e5;
    // GMFR = total inlet mass flow from the inlet states (the GUI writes it)
    double gmfr = 0.0;
    for (int n = 0; n < sp->n_inlets; ++n) {
        const gfm_inlet_spec& is = sp->inlets[n];
        const InletBlock& b = in.inlets[n];
        double w_in = 1.0 / (is.yf / gfm::kWf + is.yco2 / gfm::kWco2 + is.yh2o / gfm::kWh2o +
                             is.yo2 / gfm::kWo2 + is.yn2 / gfm::kWn2);
        double rho = pg0 * w_in / (gfm::kRu * is.t_k);
        int cy = (b.j2 - b.j1) / 2 + 1, cz = (b.k2 - b.k1) / 2 + 1;
        gmfr += rho * std::fabs(b.u) * (cy * hy) * (cz * hz);
    }
    in.gmfr = gmfr;
    in.pg0 = pg0;
    in.q0_jkg = sp->q0_jkg > 0 ? sp->q0_jkg : 2.42e6;
    in.t_init_k = sp->t_init_k;
    in.bgcon = sp->bgcon; in.maxgi = sp->maxgi; in.react = sp->react;
    for (int i = 0; i < 21; ++i) { in.rf[i] = 0.7; in.rfl[i] = 0.6; }
    in.rf[0] = in.rf[1] = in.rf[2] = sp->rf_uvw;
    in.rf[17] = 0.6; in.rf[20] = 0.6;
    in.rfl[0] = sp->rfl_species; in.rfl[1] = sp->rfl_species; in.rfl[2] = sp->rfl_h;
    in.rfl[3] = sp->rfl_k; in.rfl[4] = sp->rfl_eps; in.rfl[5] = sp->rfl_species; in.rfl[6] = sp->rfl_species;
    const double sig0[12] = {0.7, 0.7, 0.7, 1.0, 1.0, 0.7, 0.7, 0.7, 0.7, 0.7, 0.7, 0.7};
    for (int i = 0; i < 12; ++i) in.sigma[i] = sig0[i];
    in.sigma[3] = sp->sigma_k; in.sigma[4] = sp->sigma_eps;
    for (int i = 0; i < 20; ++i) in.ntimesg[i] = 2;
    for (int i = 0; i < 12; ++i) in.ntimesg[i] = sp->ntimesg[i];
    in.rf_hsource = sp->rf_hsource;
    in.i_ref = 2; in.j_ref = in.inlets[0].j1; in.k_ref = in.inlets[0].k1;
    in.p_ref_pa = 0.0;
    in.wl_m.resize(sp->nwl); in.kappa.resize(sp->nwl);
    for (int l = 0; l < sp->nwl; ++l) { in.wl_m[l] = sp->wl_um[l] * 1.0e-6; in.kappa[l] = sp->kappa[l]; }
    in.ri = 1.0; in.h_g = sp->h_g;
    in.t_wall_k = sp->t_wall_k;
    in.wall_sink = sp->wall_sink; in.rad_emission = sp->rad_emission;
    in.adi_mode = sp->adi_mode; in.precision = sp->precision;
    in.noise_amp = sp->noise_amp; in.seed = sp->seed;
    in.nr0 = 100;
    in.interval_rad = 100; in.initial_gitr = 0;
    return GFM_OK;
}

}  // namespace host
}  // namespace gfm

extern "C" int gfm_case_build(const gfm_case_spec* sp, const char* kinetic_path, gfm_case* out) {
    using namespace gfm::host;
    if (!sp || !out || !kinetic_path) return GFM_E_ARG;
    std::memset(out, 0, sizeof *out);
    CaseStore* S = new (std::nothrow) CaseStore;
    if (!S) return GFM_E_NOMEM;
    CaseInputs in;
    int rc = synth_inputs(sp, *S, in);
    if (rc != GFM_OK) { delete S; return rc; }
    return finish_case(S, in, kinetic_path, out, nullptr);
}

extern "C" void gfm_case_free(gfm_case* c) {
    if (!c) return;
    delete static_cast<CaseStore*>(c->priv);
    std::memset(c, 0, sizeof *c);
}
