// case_store.h -- host-side case construction shared by the synthetic furnace
// builder (case_build.cpp) and the reader of the reference's case files
// (case_files.cpp).  Both fill a CaseStore with the grid and cell map and a
// CaseInputs with what the reference reads from &INPUT, relaxfactorc.txt and
// the SBC file; finish_case then does the rest of the start-up the Fortran
// host does before the first GFLOW (A0main.f90:158-190).
#pragma once
#include "../../include/gfm_gb300.h"

#include <cstdint>
#include <vector>

namespace gfm {
namespace host {

struct CaseStore {
    int mp = 0, np = 0, lp = 0;
    std::vector<double> x, dx, r, dr, rs, z, dz;
    std::vector<int16_t> ibcell;
    std::vector<int16_t> b_typ, b_i, b_j, b_k, b_orient, b_direct;
    std::vector<double> b_t;
    std::vector<double> rtim, delrt, hrt, delr, timed, hrd;
    std::vector<double> wl, akl0;
    std::vector<double> p, t, dnst, theta, tmu, gama, crate, hrate, bs_hprev, ug, gf, qa, qe;
    std::vector<double> t_surf_prev;   // T_surf_prev(MZ,NZ) (K)
    // half-block factors of &GRD (Grid3.f90:12-13, 252-255): BV_F(IBC) and
    // BA_F(IX,IBC) at ba_f[3*(IBC-1) + IX-1]
    double bv_f[2] = {1.0, 1.0};
    double ba_f[6] = {1.0, 1.0, 1.0, 1.0, 1.0, 1.0};
    long at(int i, int j, int k) const { return (i - 1) + (long)mp * ((j - 1) + (long)np * (k - 1)); }
    long n() const { return (long)mp * np * lp; }
};

// One inlet block of the SBC file (Sbc.f90:64-76): a box of doubled indices,
// the face direction IU and the inlet state in SI units.
struct InletBlock {
    int i1, j1, k1, i2, j2, k2, iu;
    double t_k, yf, yox, yn2, yco2, yh2o, yck, u, v, w;
};

struct CaseInputs {
    // SETUP: &INPUT values and the constants derived from them
    double gmfr = 1.0, pg0 = 1.01325e5, q0_jkg = 2.42e6, t_init_k = 300.0, bgcon = 1.0e-8, gmu_ref = 2.6e-5;
    int maxgi = 2000, react = 1;
    int nr0 = 100;
    // relaxation factors and sweeps (Setup.f90:443-509), 0-based copies of
    // rf(1:21), rfl(1:21), ntimesg(1:20)
    double rf[21], rfl[21];
    int ntimesg[20];
    double rf_hsource = 0.3, rf_tsurf = 0.2;
    double sigma[12];
    // SBC: pressure reference and inlet blocks
    int i_ref = 0, j_ref = 0, k_ref = 0;
    double p_ref_pa = 0.0;
    std::vector<InletBlock> inlets;
    // bands: upper edges (m) and gray absorption coefficients (1/m)
    std::vector<double> wl_m, kappa;
    double ri = 1.0, h_g = 10.0;
    // configuration-level choices
    double t_wall_k = 1700.0;
    int wall_sink = 0, rad_emission = 0, adi_mode = 0, precision = 0;
    double noise_amp = 0.0;          // uniform +-noise on the fresh-start T and species
    uint64_t seed = 0;
    // melt-surface temperatures (it####t.dat): Tgs(MZ,NZ) in K
    bool have_it = false;
    int itn = 0;
    double surf_t = 0.0;
    std::vector<double> tgs;
    // restart file, NULL for a fresh start; radiation restart, NULL for none
    const char* rg_path = nullptr;
    const char* rr_path = nullptr;
    int interval_rad = 100, initial_gitr = 100;
    // minor species and soot (Var_mod.f90:215, 465-492; Setup.f90:161-185),
    // relaxfactorc.txt's minor-species lines (Setup.f90:476-511)
    int ms = 0, irstypm = 0, maxms = 300, ntimesm = 4;
    double bmcon = 1.0e-7, ssigma = 0.7, rfm = 0.5, rfm_soot = 0.2;
    double rf_soot_form = 0.3, rf_soot_oxid = 0.3, soot_cap = 4.0e-3, t0_sf = 0.0, t0_so = 0.0;
    double aform = 400.0, aoxid = 26.0, esf = 5.0e7, eso = 5.0e7;
    int gas_model = 0;
    // wall radiation inputs: &RADIN and the exhaust table of the SBC file
    gfm_wall_spec wall = wall_defaults();
    static gfm_wall_spec wall_defaults() {   // Sbc.f90:317-331, T_mnK (Var_mod.f90:45)
        gfm_wall_spec w{};
        w.eps_w = 0.8; w.eps_c = 0.8; w.eps_m = 0.95;
        w.have_crown = 0; w.height_to_ceiling = 0.0;
        w.maxri1 = 100; w.maxri2 = 1000; w.minri2 = 4;
        w.t_a = 350.0; w.h_a = 5.0; w.w_k = 2.0; w.w_d = 0.31;
        w.t_mnk = 200.0;
        return w;
    }
};

// The synthetic furnace of a gfm_case_spec as the inputs a case directory
// would give: grid, cell map (before the propagation) and CaseInputs.
int synth_inputs(const gfm_case_spec* sp, CaseStore& s, CaseInputs& in);

// Builds the rest of the case from the grid and cell map in *S (IBCELL
// before the 27-neighbour propagation) and the inputs; takes ownership of S
// (freed on error).  Returns a GFM status.
int finish_case(CaseStore* S, const CaseInputs& in, const char* kinetic_path, gfm_case* out,
                gfm_case_summary* sum);

// read_restart_data (Initsv.f90:225-316) onto the post-SBC state in s.
// Returns a GFM status; on success fills the restart tail values.
int read_restart(const char* path, CaseStore& s, const gfm_params& P, gfm_fields& F, gfm_restart_tail& tail,
                 int& maxgi);
// rad_emis_rr (Rad_emis.f90:17-110) after it: QE and QA, and the wall
// temperatures of the last exchange into T and H at the closed wall cells.
int read_rad_restart(const char* path, CaseStore& s, const gfm_params& P);

// Property helpers in the reference's order (Prop.f90), on the store's arrays.
void prop_dnst(CaseStore& s, const gfm_params& P, long a);   // dnst_calc (Prop.f90:187-198)
void prop_ther(CaseStore& s, const gfm_params& P, long a);   // THER (Prop.f90:130-154)
void prop_tke(CaseStore& s, long a);                         // TKE (Prop.f90:162-176)
void prop_t2h(CaseStore& s, const gfm_params& P, long a);   // T_to_enth (Prop.f90:520-560)

}  // namespace host
}  // namespace gfm
