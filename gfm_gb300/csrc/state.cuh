// state.cuh -- device state of one solver handle and the launcher interface
// between the host orchestration (solver.cu) and the kernel translation units.
#pragma once
#include "device.cuh"

namespace gfm {

constexpr int kFtVals = 11;   // P, TMU, GAMA, GF(1..7), T

// Boundary-cell record for EXTR (Extr.f90:31-250): indices and weights are
// fixed by IBCELL and the grid, so they are computed once on the host.
struct ExtrRec {
    int I, J, K, I1, J1, K1, I2, J2, K2, IX;
    int kind;            // 2 inlet, 3 exit, 1 wall
    int I3, J3, K3;      // exit: face receiving the SBC4 copy
    double F1, F2;
};
// Exit-face record for EXTRV (Extr.f90:358-567)
struct ExtrvRec {
    int I, J, K, IU;
    int mode;            // 0: flux branch with neighbour offset m; 1: copy from (Is,Js,Ks)
    int m;               // -1 / +1
    int Is, Js, Ks;
};
// Wall patch of the fixed-temperature sink (Qwall.f90:395-513)
struct Patch {
    int inc, jnc, knc;   // open cell centre next to the patch
    double ds_q;         // distance used in calc_q_conv_wall
    double ds_src;       // cell width used in the source (Source.f90:488-502)
    double area, bT;
};

// Device scalars (double), indices into Ctx::scal
enum Scal {
    S_RES_MASS = 0, S_RES_MASS_MAX, S_GFEX, S_GFIN0, S_GFIN, S_FACTOR, S_FADJ, S_G0, S_TMEAN_EX,
    S_Q_REACT, S_Q_EXHAUST, S_QCONV, S_TAVE, S_P_RESID_PRE, S_P_RESID, S_PCORR_RESID,
    S_U_RESID_PRE, S_U_RESID = S_U_RESID_PRE + 3, S_GF_RESID_PRE = S_U_RESID + 3, S_GF_RESID = S_GF_RESID_PRE + 10,
    S_TAREA_MEAN = S_GF_RESID + 10, S_AREA_EX, S_ITR_GAS, S_TAVE_DEN, S_RAD_ACTIVE,
    S_LP_SCALE, S_LP_USED, S_LP_RATIO, S_LP_ALPHA, S_LP_TSCALE,
    S_RAD_DONE,   // i1st_rad_done: a wall exchange has run, EXTR keeps wall h and T (Extr.f90:194-197)
    // MSFLOW: resid_ms_pre and resid_ms of the seven species and soot, bal_MS,
    // soot mass, largest soot mass fraction clipped and not
    S_MS_RPRE, S_MS_RES = S_MS_RPRE + 8, S_MS_BAL = S_MS_RES + 8, S_MS_SOOT, S_MS_SMFMAX, S_MS_SMFMAXNC,
    S_NUM
};

template <typename R>
struct Ctx {
    GeoT<R> g;
    Prm p;
    R *P, *T, *DNST, *THETA, *TMU, *GAMA, *CRATE, *HRATE, *GTE, *BSH;
    R *UG[3];
    R *GF[9];
    R *FZ;
    R *APm, *ASm[6], *BSm, *SFPm;          // momentum, face classes
    R *APc, *ASc[6], *BSp, *BSq;           // pressure / p', centre class
    R *DPc, *BSr;                          // p' refinement: correction and its right-hand side (mixed)
    R *APs[7], *BSs[7], *FZs[7], *SFPs[7]; // scalar equations L=1..7 at index L-1
    R *ASs[3][6];                          // coefficient sets shared by equal sigma
    int as_set[7];
    R *QA, *QE;                            // radiation rates (W) at cell centres
    const double *rtim, *delrt, *delr, *timed;
    int nr0;
    const ExtrRec *extr_io, *extr_wall, *extr_ft;
    int n_extr_io, n_extr_wall, n_extr_ft;
    const int* ft_col_start;               // fall-through wall cells grouped by (I,J) column
    int n_ft_cols;
    R* ft_buf;                             // source values of the fall-through cells (kFtVals each)
    const ExtrvRec* extrv;
    int n_extrv[3];                        // records per direction, stored back to back
    const Patch* patch;
    const int* cell_patch_start;           // CSR: patches adjacent to each listed open cell
    const int* cell_patch_list;
    const int* patch_cells;                // open cell centres with patches (packed I|J<<12|K<<24 not used: ijk triplets)
    int n_patch, n_patch_cells;
    R* qconv;                              // q_conv per patch (W/m2)
    const int8_t* intp_mode;               // INTP carried-F1 code per position
    double* scal;                          // S_NUM device scalars
    double* partials;                      // kRedSlots x kRedBlocks
    int nwl;
    double wl[16], akl0[16];
    int i_ref, j_ref, k_ref;
    double p_ref;
    int itr_gas;                           // host copy for launches that branch on it
    int rad_active;                        // i1st_rad_qe_done > 0: QA-QE enters the h source
    const NistT<R>* nist;                  // device copy of the Shomate table in the type R
};

// Equation system for the line solver: class given by (ib,jb,kb) parities.
template <typename R>
struct Sys {
    R* xt;
    const R* ap;
    const R* as[6];
    const R* bs;
    int ib, ie, jb, je, kb, ke, nim;
};

// Four values of one line row, loaded as one vector.
template <typename R>
struct __align__(4 * sizeof(R)) Quad { R x, y, z, w; };

// Per-equation scratch of the line solver.
//  march order: XT2, XT3, PT of y- and z-lines, indexed like the fields (pidx);
//  red-black order: colour-split arrays (2*CBH elements each, see adi.cu): the
//  unknown XS, the pass results X2/X3, the scaled x-neighbour right-hand sides
//  of the y- and z-lines, and the factored rows of both line directions.
template <typename R>
struct AdiScratch {
    R *xt2, *xt3, *pty, *ptz;
    R *xs, *x2, *x3, *sby, *sbz, *x2b, *x3b;
    Quad<R> *ya, *yb, *za, *zb;
};

// ---- wall radiosity exchange (wall.cu) -----------------------------------------
constexpr int kWallBlocks = 128;   // blocks of the per-patch kernels (fixed: their partial sums add in block order)
constexpr int kWallSlots = 16;
enum WallSlot {
    W_INC_TOTAL = 0, W_INC_WALL, W_INC_INLET, W_INC_EXIT, W_INC_MELT, W_REL, W_Q_MELT, W_Q_LOSS,
    W_T_AREA, W_Q_RAD_IN, W_Q_RAD_OUT, W_QM_FLAME, W_QM_BNDS, W_QM_CONV, W_QCONV
};
struct WallArgs {
    int nb;                        // boundary patches
    float* vf32;                   // nb x nb normalised view factors, row = near patch (mixed precision)
    double* vf64;                  //   the same in FP64 (FP64 path)
    const int *typ, *bi, *bj, *bk, *ori, *dir;
    const int *o_bc;               // split index of each patch's closed cell centre
    const int *o_b;                // split index of the patch position
    const int *sink;               // index in the wall-sink patch list, -1 for inlets and exits
    const double *px, *py, *pz;    // X(b_i), R(b_j), Z(b_k)
    const double *emis, *area, *face_area, *bT_exit;   // bT_exit: exits' temperature at the first exchange
    double *bT, *J, *Jn, *qc, *qeb, *qconv, *qamb, *rad, *rel;
    double* vfsum;                 // row sums of the view factors before normalisation
    double* part;                  // kWallSlots x kWallBlocks partial sums
    double sig, radi_min, t0, u_a0, t_a, t_mnk;
};

int launch_wall_vf(const WallArgs& a, cudaStream_t st);
template <typename R> void launch_wall_start(const WallArgs& a, const R* T, int first, cudaStream_t st);
template <typename R> void launch_wall_init(const WallArgs& a, const R* QA, R* QE, cudaStream_t st);
void launch_wall_to_sink(const WallArgs& a, Patch* sink_patches, cudaStream_t st);
template <typename R> void launch_wall_from_sink(const WallArgs& a, const R* qconv_sink, cudaStream_t st);
void launch_wall_sweep(const WallArgs& a, cudaStream_t st);
void launch_wall_rad(const WallArgs& a, int mask, cudaStream_t st);
void launch_wall_temps(const WallArgs& a, cudaStream_t st);
void launch_wall_qamb(const WallArgs& a, cudaStream_t st);
template <typename R> void launch_wall_post(const WallArgs& a, R* T, cudaStream_t st);
void launch_wall_exits(const WallArgs& a, const int* frac_exit, const double* frac, double avg_wall_T, cudaStream_t st);

// ---- volume radiation transfer (rad.cu) ---------------------------------------
constexpr int kRadMaxBands = 16;
struct RadArgs {
    GeoT<double> g;              // coordinates (1-based), parity-split IBCELL, pidx
    int MP, NP, LP, MZ, NZ, LZ, NWL;
    int akl_blocks;              // blocks of k_rad_akl and k_rad_qe (2 totals per block each)
    // per march direction (x, y, z): slab arrays in shared memory (else in
    // scratch/fscratch), dynamic shared memory, CTAs, first QAL copy
    int slab_in_smem[3];
    int slab_global;             // put the slab arrays in global scratch even where they fit (tests)
    size_t smem[3];
    int grid[3];
    int part_base[4];            // part_base[3]: QAL copies in all
    double t0, sgn;              // T0; SIG*RI*RI
    double akl0[kRadMaxBands];   // band absorption coefficients (1/m)
    double deb0[kRadMaxBands];   // HCK/RI/WL
    int16_t* ibr;                // IBCELL with the wall markers, per cell (MZ,NZ,LZ)
    double *akl, *tcell;         // AKL (cell + l*ncell), T*T0 per cell
    double* qel0;                // QEL0 of the emitters (cell + l*ncell)
    double *qal_part;            // one QAL copy per trace block
    double *qe, *qa;             // QE, QA per cell (MZ,NZ,LZ)
    double *tot_part, *akl_part, *qe_part;   // block totals (8 per trace CTA, 2 per akl / qe block)
    double* scratch[3];          // slab arrays when they do not fit in shared memory
    unsigned char* fscratch[3];
    int* err;                    // bit 0: geometry outside the supported set
    // band model (gas.cu): AKLG and AKLS per cell and band (cell + l*ncell);
    // null for the gray bands akl0
    const double *gas_aklg, *gas_akls;
    // per direction and CTA: the corner-split additions of the interior
    // columns of one slab, split_capc entries per column (rad.cu)
    int split_capc[3];
    int* split_cnt[3];           // [cta][column]
    int* split_meta[3];          // [cta][column][entry][row, target column, band mask]
    double* split_q[3];          // [cta][column][entry][band]
};
// ---- minor species and soot (ms=1): MSFLOW's state -----------------------------
template <typename R>
struct MinorDev {
    R* gfm[7];                   // GFM(.,L), parity split
    R *smf, *bsp, *sfpp;         // soot mass fraction, bs_soot_prev, sfp_soot_prev, parity split
    R* rrms;                     // RRMS(MZ,NZ,LZ,5), cell layout (I fastest)
};

// ---- gas and soot band model (gas.cu) ------------------------------------------
struct GasBuffers {
    double *aklg, *akls;         // per cell (I fastest) and band: cell + l*ncell
    double* fvs;                 // soot volume fraction, by loop order (K fastest)
    int *setter, *blockmax;      // the cells that set AKLS, and the prefix maxima
    int* err;                    // bit 1: BANDA argument < 0, bit 2: W_R <= 0 with CO2
    const double* sqper;         // square roots of CHIWHI's integer factors (gas_sqper_fill)
    const float* sqperf;         //   the same in FP32, for the mixed path
};
int gas_scan_blocks(int ncell);
int gas_sqper_size();
void gas_sqper_fill(double* table);
// in-place prefix maximum of a[0..n): a[i] becomes the maximum within its
// block of 1024 up to i, blockmax[b] the maximum of the blocks before b
// (gas_scan_blocks(n) entries); the full prefix at i is the larger of the two
void launch_prefix_max(int* a, int n, int* blockmax, cudaStream_t st);

// ---- minor species transport and soot (minor.cu) ---------------------------------
template <typename R>
struct MsScratch {
    R* as[6];                    // coefficient set of the minor species (SGM = SSIGMA)
    R *ap1, *ap;                 // the sum of the six; AP of the system being solved
    R *fz[7], *bs[7];            // unknowns and right-hand sides (soot in slot 0)
    double* r4;                  // each reaction cell's last RR2, by loop order
    int *setter, *blockmax;      // the reaction cells' loop-order prefix
    double* carry;               // RR2 entering the next GSLV3M call
    double* stats;               // GFM_0(L,2) of the seven species, SVF_R
    int nq;                      // cells of the reaction range
    // relaxation and soot constants (relaxfactorc.txt, &INPUT)
    double rfm, rfm_soot, rf_sf, rf_so, soot_cap, t0_sf, t0_so, aform, aoxid, esf_r, eso_r, snorm;
    int react;
};
// slots of the MSFLOW sums in the partials rows (after the gas iteration's)
constexpr int kSlMsPre = 40, kSlMsPost = 48, kSlMsBal = 56, kSlMsSoot = 57, kSlMsSmfMax = 58, kSlMsSmfMaxNc = 59;
template <typename R>
void launch_ms_rates(const Ctx<R>& c, const MinorDev<R>& m, const MsScratch<R>& s, R* const* as_spin, cudaStream_t st);
template <typename R> void launch_ms_ap(const Ctx<R>& c, const MsScratch<R>& s, cudaStream_t st);
template <typename R> void launch_ms_species(const Ctx<R>& c, const MinorDev<R>& m, const MsScratch<R>& s, cudaStream_t st);
template <typename R> void launch_ms_update(const Ctx<R>& c, const MinorDev<R>& m, const MsScratch<R>& s, cudaStream_t st);
template <typename R>
void launch_soot_system(const Ctx<R>& c, const MinorDev<R>& m, const MsScratch<R>& s, int itr_ms, cudaStream_t st);
template <typename R> void launch_soot_update(const Ctx<R>& c, const MinorDev<R>& m, const MsScratch<R>& s, cudaStream_t st);
template <typename R> void launch_ms_stats(const Ctx<R>& c, const MinorDev<R>& m, const MsScratch<R>& s, cudaStream_t st);
// RAD_GAS and SOOTA of RAD0 (Rad0.f90:116-132) on the current T, P, DNST
// and minor species: AKLG and AKLS of every open cell with T >= TG_MN
template <typename R>
int launch_gas_band(const GasBuffers& b, const GeoT<double>& g, const R* T, const R* P, const R* DNST,
                    const R* const* gfm, const R* smf, double t0, double pg0, double dnst0, int nwl, const double* wl,
                    cudaStream_t st);

// fills slab_in_smem, smem, grid and part_base from the grid, the band count
// and the SM count
int rad_plan(RadArgs& a, int sms);
template <typename R> int launch_rad_transfer(RadArgs a, R* T, long long nT, cudaStream_t const* st, cudaEvent_t const* ev);

// ---- launchers (defined in the kernel translation units) --------------------
template <typename R> void launch_wallfn(const Ctx<R>& c, const int* wall_list, int n_wall, cudaStream_t s);
template <typename R> void launch_copy_faces_to_fz(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_mom_assemble(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_p_assemble(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_bound_p(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_mom_prep(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_mom_finish(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_pcorr_source(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_velcorr(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_extrv(const Ctx<R>& c, int mex, cudaStream_t s);
template <typename R> void launch_factor(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_intpv(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_qconv(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_scalar_sources_first(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_scalar_assemble(const Ctx<R>& c, int L, bool new_as, cudaStream_t s);
template <typename R> void launch_scalar_finish(const Ctx<R>& c, int L, cudaStream_t s);
template <typename R> void launch_scalar_faces_into(const Ctx<R>& c, R* const* as_out, double sgm, cudaStream_t s);
template <typename R> void launch_props(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_tave(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_extr(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_intp(const Ctx<R>& c, cudaStream_t s);
template <typename R> void launch_initsvm(const Ctx<R>& c, const MinorDev<R>& m, int restart, cudaStream_t s);
template <typename R> void launch_extrm(const Ctx<R>& c, const MinorDev<R>& m, cudaStream_t s);
template <typename R> void launch_intpm(const Ctx<R>& c, const MinorDev<R>& m, cudaStream_t s);
template <typename R> void launch_rad_emission(const Ctx<R>& c, cudaStream_t s, const double* gas_aklg = nullptr,
                                               const double* gas_akls = nullptr);
template <typename R> void launch_residual(const Ctx<R>& c, const Sys<R>& sys, int slot, cudaStream_t s);
template <typename R> void launch_refine_rhs(const GeoT<R>& g, const Sys<R>& sys, R* rhs, cudaStream_t s);
template <typename R> void launch_refine_add(const GeoT<R>& g, const Sys<R>& sys, const R* dx, cudaStream_t s);
// red-black line-solver options: kRbPlane runs each plane visit in one CTA
// (adi_plane.cu) wherever every plane of the batch fits, else the segmented
// colour passes below run; kRbPdl launches the line-solver kernels with
// programmatic dependent launch; kRbAvgInPass lets pass L=2 of the segmented
// form average the pass L=1 results where it reads them, in place of the
// averaging launch between the passes
// kRbNoSmall keeps planes that fit 8 warps on the 768-thread visit CTAs;
// kRbSmallF64 lets small FP64 planes take the plane visit (by default they
// take the segmented passes)
constexpr int kRbPlane = 1, kRbPdl = 2, kRbAvgInPass = 4, kRbNoSmall = 16, kRbSmallF64 = 32;
// the plane-visit form of one ADLBL3 call on a batch; returns the kernels it
// launched, or 0 (nothing launched) when a plane of the batch does not fit
template <typename R> int launch_rbp(const GeoT<R>& g, const Sys<R>* sys, const AdiScratch<R>* scr, int nsys,
                                     cudaStream_t s, int rb_flags);
int prepare_rbp();
// returns the number of kernels it launched
template <typename R> int launch_adlbl3_scr(const GeoT<R>& g, const Sys<R>* sys, const AdiScratch<R>* scr, int nsys,
                                            int mode, cudaStream_t s, int rb_flags);
int prepare_line_solver();   // once per process, before any stream capture
int prepare_rif_table();     // the RIF3 term table of the emission update, likewise
// deterministic finish of block partials: op 0 sum, 1 max, 2 residual
// (sum/NCELLS floored at 1e-16, NaN -> 1e-16), 3 sum/NCELLS
struct FinishSpec {
    int n;
    int slot[40], dst[40], op[40];
};
void launch_finish(const double* partials, double* scal, const FinishSpec& f, double ncells, cudaStream_t s);
template <typename R> void launch_pref_idx(const Ctx<R>& c, int I1, int J1, int K1, int I2, int J2, int K2, double F1,
                                           double F2, cudaStream_t s);


// learned p' initial guess (lpsolve.cu): network inputs (BF16, 16 channels per
// voxel of the p' solve range), guess + fallback into x, training target
template <typename R> void launch_lp_features(const Ctx<R>& c, void* feats, int nx, int ny, int nz, cudaStream_t s);
template <typename R> void launch_lp_guess(const Ctx<R>& c, const float* out16, R* x, int nx, int ny, int nz, cudaStream_t s);
template <typename R> void launch_lp_target(const Ctx<R>& c, const R* x, float* tgt, int nx, int ny, int nz, cudaStream_t s);

// layout conversion doubled <-> parity split (host-layout arrays on device)
template <typename R> void launch_to_split(const GeoT<R>& g, const double* src, R* dst, cudaStream_t s);
template <typename R> void launch_to_split_count(const GeoT<R>& g, const double* src, R* dst, unsigned int* cnt, cudaStream_t s);
template <typename R> void launch_from_split(const GeoT<R>& g, const R* src, double* dst, cudaStream_t s);
template <typename R> void launch_cells_to_split(const GeoT<R>& g, const double* src, R* dst, cudaStream_t s);
template <typename R> void launch_cells_from_split(const GeoT<R>& g, const R* src, double* dst, cudaStream_t s);

}  // namespace gfm
