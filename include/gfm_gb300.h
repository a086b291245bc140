/*
 * gfm_gb300.h -- C ABI of the GB300-native GFM combustion-space solver.
 *
 * The reference solver (GFM v4, Fortran 90) runs its steady SIMPLER outer
 * iteration as argument-less subroutines over module state (module GBL_VAR,
 * combustion/Code/Var_mod.f90).  This header replaces three seams of it:
 *
 *   CALL GFLOW                       combustion/Code/Sphase.f90:51
 *   CALL ADLBL3(XT,IB,IE,JB,JE,KB,KE) combustion/Code/Adlbl3.f90:10
 *   CALL rad_qe_only                 combustion/Code/Sphase.f90:226
 *
 * plus the start-up work a Fortran host would otherwise do before the first
 * GFLOW (GRID3/SETUP/SBC/INITSV, combustion/Code/A0main.f90:158-190), for the
 * synthetic furnace cases and from a GFM case directory's own files, and the
 * restart file of SAV3F (combustion/Code/Sav3f.f90:21-88).
 *
 * Layout at the boundary is the reference's own: every field is a Fortran
 * column-major array over the doubled staggered grid A(MP,NP,LP) (I fastest,
 * 1-based in Fortran, element (I,J,K) at offset (I-1)+MP*((J-1)+NP*(K-1)) here),
 * UG(MP,NP,LP,3) and GF(MP,NP,LP,9) append the component as the slowest index,
 * IBCELL is integer(2).  Cell arrays QA/QE are (MZ,NZ,LZ) with MZ=MP/2.
 *
 * Conventions: every entry point returns an int status (0 = ok, <0 = error,
 * see GFM_E_*), never aborts and never exits.  One handle per host thread;
 * calls on one handle are serialised on the handle's own CUDA stream.
 */
#ifndef GFM_GB300_H
#define GFM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define GFM_OK              0
#define GFM_E_ARG         (-1)   /* bad argument / dimension                */
#define GFM_E_CUDA        (-2)   /* CUDA runtime error                      */
#define GFM_E_NAN         (-3)   /* non-finite value detected               */
#define GFM_E_UNSUPPORTED (-4)   /* input outside the supported case set    */
#define GFM_E_NOMEM       (-5)   /* allocation failed                       */
#define GFM_E_TIMEOUT     (-6)   /* bounded device wait ran out             */
#define GFM_E_NODEVICE    (-7)   /* no CUDA device / extension not usable   */
#define GFM_E_LIMIT       (-8)   /* input beyond a fixed size limit         */
#define GFM_E_IO          (-9)   /* input file missing, short or malformed  */

/* ADI line-solver ordering (gfm_params.adi_mode) */
#define GFM_ADI_MARCH      0     /* reference order: x-plane Gauss-Seidel march,
                                    forward then backward (Adlbl3.f90:39-51)   */
#define GFM_ADI_REDBLACK   1     /* red-black x-plane ordering, all planes of
                                    one colour at once                          */

/* arithmetic of the bulk stencil / line-solve work (gfm_params.precision) */
#define GFM_PREC_FP64      0     /* plain FP64, the reference's arithmetic      */
#define GFM_PREC_MIXED     1     /* FP32 stencil assembly, property updates and
                                    line solves; FP64 global reductions and an
                                    FP64-residual refinement step on p'         */

/* ---- grid: geometry, cell map, boundary patches, tables ------------------ */
typedef struct gfm_grid {
    int mp, np, lp;              /* doubled extents MP,NP,LP (Grid3.f90:36)   */
    const double *x, *dx;        /* X(MP), DX(MP)  (Grid3.f90:79-109)         */
    const double *r, *dr, *rs;   /* R(NP), DR(NP), RS(NP) (Grid3.f90:117-171) */
    const double *z, *dz;        /* Z(LP), DZ(LP)  (Grid3.f90:177-226)        */
    const int16_t *ibcell;       /* IBCELL(MP,NP,LP) after the 27-neighbour
                                    propagation (Grid3.f90:259-275)           */
    int ncells;                  /* NCELLS (Grid3.f90:259-268)                */
    int i_ref, j_ref, k_ref;     /* pressure reference cell (Sbc.f90:57)      */
    double p_ref;                /* P_REF/PG0                                 */
    /* wall patches of the fixed-temperature wall sink (Qwall.f90:395-513) */
    int b_cnt;
    const int16_t *b_typ, *b_i, *b_j, *b_k, *b_orient, *b_direct;
    const double *b_t;           /* patch temperature b_T (K)                 */
    /* integral-reaction kinetics table (Setup.f90:858-888) */
    int nr0;
    const double *rtim, *delrt, *hrt, *delr, *timed, *hrd;
    /* gray radiation bands: edges WL (m) and absorption coefficients (1/m) */
    int nwl;
    const double *wl, *akl0;
    /* half-blocked cells, IBCELL = -1 or -2 (gd digits 9 and 8): the volume
     * factor BV_F(IBC) and the face-area factors BA_F(IX,IBC), stored at
     * ba_f[3*(IBC-1) + IX-1], read from &GRD (Grid3.f90:12-13,252-255) and
     * applied by VOL_C0 and AREA_C (Grid3.f90:395-471); 1 when absent */
    double bv_f[2];
    double ba_f[6];
} gfm_grid;

/* ---- scalar constants of module GBL_VAR after SETUP ---------------------- */
typedef struct gfm_params {
    double t0, h_0, dnst0, ug0, gmfr, pg0, r0;           /* Setup.f90:542-543 */
    double reyg, reyg2, epsr, taur, eun, qr0, q0, tk0;   /* Setup.f90:662-721 */
    double gra[3];               /* GRA/UG0**2*R0 (Setup.f90:544)             */
    double amu, trdg, wt0, stoich;
    double cmu, ct1, ct2;        /* k-eps constants (Var_mod.f90:203-208)     */
    double p_mx, p_mn, t_mx, t_mn, u_mx, u_mn, f_mx, f_mn;  /* bounds         */
    double rf[21], rfl[21];      /* relaxation factors (Setup.f90:443-472)    */
    double sigma[12];            /* Prandtl/Schmidt numbers (Var_mod.f90:211) */
    int    ntimesg[20];          /* ADI sweeps per NELG (Setup.f90:495-509)   */
    double rf_hsource;           /* enthalpy-source relaxation (Setup.f90:486) */
    int    react, turb;
    /* configuration-level switches (applied identically by every path) */
    int    wall_sink;            /* fixed-T wall convective sink every iteration */
    double h_g;                  /* internal wall heat-transfer floor (W/m2/K) */
    int    rad_emission;         /* emission-only radiation source (rad_qe_only) */
    int    rad_qe_frequency;     /* iterations between emission updates (10)   */
    double sig, ri, hck;         /* Stefan-Boltzmann, refraction index, hc/k   */
    double bgcon;                /* convergence on res_mass (Sphase.f90:193)  */
    int    maxgi;
    int    adi_mode;             /* GFM_ADI_*                                  */
    int    precision;            /* GFM_PREC_*                                 */
    /* minor species, soot and the gas band model (Var_mod.f90:134-137,
     * 215-235, 465-509; &INPUT and relaxfactorc.txt, Setup.f90:476-511) */
    int    gas_model;            /* 0: gray bands akl0; 1: RAD_GAS and SOOTA
                                    from the minor species (Rad0.f90:116-132) */
    int    maxms;                /* MSFLOW iterations, MAXMS (300)             */
    int    ntimesm;              /* line-solver sweeps of the minor species    */
    int    irstypm;              /* 1: minor species restart (IRSTYPM)         */
    double bmcon;                /* MSFLOW convergence on resid_ms (BMCON)     */
    double ssigma;               /* Schmidt number of the minor species (0.7) */
    double rfm, rfm_soot;        /* relaxation of the species and of soot      */
    double rf_soot_form, rf_soot_oxid;   /* soot source relaxation             */
    double soot_cap, t0_sf, t0_so;       /* soot bound, cut-off T (K)          */
    double aform, aoxid;         /* soot formation and oxidation constants     */
    double esf_r, eso_r;         /* their activation energies over Ru (K)      */
} gfm_params;

/* ---- fields in the reference layout -------------------------------------- */
typedef struct gfm_fields {
    double *p, *t, *dnst, *theta, *tmu, *gama;   /* (MP,NP,LP)                 */
    double *crate, *hrate, *bs_hprev;            /* (MP,NP,LP)                 */
    double *ug;                  /* UG(MP,NP,LP,3)                             */
    double *gf;                  /* GF(MP,NP,LP,9): 1 fuel 2 O2 3 h 4 k 5 eps
                                    6 CO2 7 N2 9 H2O (Var_mod.f90:116-123)     */
    double *qa, *qe;             /* QA, QE (MZ,NZ,LZ), W per cell              */
    /* iteration state carried between GFLOW calls */
    int    itr_gas, do_rad_qe_only_cnt, i1st_rad_qe_done;
    double factor, fadj, gfin0, q_h_in;
} gfm_fields;

/* ---- minor species and soot: the state of MSFLOW ------------------------- */
#define GFM_NSP_MINOR 7
typedef struct gfm_minor {
    double *gfm;                 /* GFM(MP,NP,LP,7): CH4 O2 CO H2O CO2 N2 NO
                                    mass fractions (Gslv3m.f90:122-129)        */
    double *smf;                 /* soot mass fraction (MP,NP,LP)              */
    double *bs_soot_prev, *sfp_soot_prev;   /* the last soot sources (MP,NP,LP) */
    double *rrms;                /* RRMS(MZ,NZ,LZ,5) reaction rates            */
    int    itr_ms;               /* MSFLOW iterations so far                   */
    int    imscon;               /* the last MSFLOW met BMCON                  */
} gfm_minor;

/* What one MSFLOW call did (Msflow.f90:48-162, Gslv3m.f90:171-284). */
typedef struct gfm_msflow_stats {
    int    itr_ms;               /* cumulative MSFLOW iteration count          */
    int    iterations;           /* iterations of this call                    */
    int    converged;            /* imscon: every resid_ms <= BMCON            */
    int    reserved;
    double resid_ms_pre[8], resid_ms[8];    /* 7 species then soot             */
    double bal_ms;               /* mean |1 - sum of GFM| (Gslv3m.f90:196-218) */
    double soot_tot;             /* soot mass in the furnace (kg)              */
    double smf_max, smf_max_noclip;
    double gfm_out[7];           /* GFM_0(L,2): species flow out (kg/s)        */
    double svf_r;                /* area-mean soot volume fraction at the exits */
} gfm_msflow_stats;

/* ---- per-iteration statistics (the reference's .plt log quantities) ------ */
typedef struct gfm_iter_stats {
    int    itr_gas;
    int    converged;            /* res_mass < BGCON (Sphase.f90:193)          */
    double res_mass, res_mass_max;          /* Source.f90:41-101              */
    double p_resid_pre, p_resid, pcorr_resid;
    double u_resid_pre[3], u_resid[3];
    double gf_resid_pre[10], gf_resid[10];  /* index L-1, L=1..7              */
    double factor, gfin, gfex;
    double q_react, q_exhaust, q_conv_total, q_global_bal;
    double tave, tmean_ex;
    int    lp_used;              /* learned p' guess kept (1) or replaced by 0 */
    double lp_ratio;             /* |b - A x_guess| / |b| of that guess         */
} gfm_iter_stats;

/* ---- synthetic furnace specification (stands in for gd/sbc files) -------- */
typedef struct gfm_inlet_spec {
    double y0, y1, z0, z1;       /* opening on the x=0 wall (m)               */
    double t_k;                  /* inlet temperature (K)                      */
    double yf, yo2, yn2, yco2, yh2o;
    double u_ms;                 /* nominal velocity (m/s), rescaled to keep
                                    the mass flow after snapping to cells      */
} gfm_inlet_spec;

typedef struct gfm_case_spec {
    int    nx, ny, nz;           /* interior cells                             */
    double lx, ly, lz;           /* box (m)                                    */
    int    n_inlets;
    gfm_inlet_spec inlets[8];    /* inlets[0] holds the pressure reference     */
    double exit_y0, exit_y1, exit_z0, exit_z1;   /* flue on the x=lx wall      */
    double t_init_k;             /* initial gas temperature (K)                */
    double noise_amp;            /* uniform +-noise on initial T and species   */
    uint64_t seed;
    double inlet_jitter;         /* uniform +-jitter on inlet velocities       */
    double t_wall_k;             /* fixed wall temperature (K)                 */
    double rf_uvw, rfl_h, rfl_k, rfl_eps, rfl_species, rf_hsource;
    int    ntimesg[12];          /* sweeps for NELG 1..12                      */
    double sigma_k, sigma_eps;
    int    nwl;
    double kappa[16];            /* gray band absorption coefficients (1/m)    */
    double wl_um[16];            /* band upper edges (um), as WL in &RADIN     */
    double pg0, q0_jkg, h_g;
    int    react, wall_sink, rad_emission, maxgi;
    double bgcon;
    int    adi_mode, precision;
} gfm_case_spec;

/* The records of the restart file rg####c.d that follow the per-cell fields
 * and are not part of gfm_fields (Sav3f.f90:75-82, Initsv.f90:290-303). */
typedef struct gfm_restart_tail {
    int     mz, nz;              /* extents of T_surf_prev: MP/2, NP/2          */
    double *t_surf_prev;         /* T_surf_prev(MZ,NZ): melt-surface T (K) the
                                    next melt_surf_T relaxes against           */
    int     i1st_rad_done;       /* a full radiation call has run               */
    int     itr_rad, itr_gend;   /* radiation call count, end of the current
                                    gas-iteration interval                     */
    int     interval_rad;        /* gas iterations between radiation calls      */
} gfm_restart_tail;

/* Wall radiation inputs: the &RADIN wall entries (Sbc.f90:25-35, defaults
 * Sbc.f90:317-331) and the exhaust table of the sbc file (Sbc.f90:273-284).
 * Wall-property blocks (NRADWALL > 0, IWALL) are not supported. */
#define GFM_MAX_EXHAUSTS 16
typedef struct gfm_wall_spec {
    double eps_w, eps_c, eps_m;  /* wall, crown and melt-surface emissivity     */
    int    have_crown;           /* 1: walls at z >= height_to_ceiling are crown */
    double height_to_ceiling;    /* m                                          */
    int    maxri1, maxri2, minri2;   /* radiosity solver loop limits (wallq)   */
    double t_a, h_a, w_k, w_d;   /* ambient T (K), outside h (W/m2/K), wall
                                    conductivity (W/m/K) and thickness (m)    */
    double t_mnk;                /* lower bound of a wall T (K), T_mnK         */
    int    nex;                  /* exhausts                                   */
    int    exh_i1[GFM_MAX_EXHAUSTS], exh_j1[GFM_MAX_EXHAUSTS], exh_k1[GFM_MAX_EXHAUSTS];
    int    exh_i2[GFM_MAX_EXHAUSTS], exh_j2[GFM_MAX_EXHAUSTS], exh_k2[GFM_MAX_EXHAUSTS];
    int    exh_orient[GFM_MAX_EXHAUSTS], exh_direct[GFM_MAX_EXHAUSTS], exh_type[GFM_MAX_EXHAUSTS];
    double exh_frac[GFM_MAX_EXHAUSTS], exh_fixed[GFM_MAX_EXHAUSTS];
} gfm_wall_spec;

/* A built case: host-owned arrays allocated by gfm_case_build or
 * gfm_case_read. */
typedef struct gfm_case {
    gfm_grid   grid;
    gfm_params params;
    gfm_fields fields;
    void      *priv;             /* owns the storage behind the pointers       */
    gfm_restart_tail tail;       /* restart records beyond the fields           */
    gfm_wall_spec wall;          /* wall radiation inputs (sbc file, or the
                                    synthetic furnace's defaults)             */
} gfm_case;

/* Opaque GPU solver handle. */
typedef struct gfm_handle gfm_handle;
/* Opaque learned p' initial-guess network. */
typedef struct gfm_lp gfm_lp;

/* ---- host side: synthetic case construction ------------------------------ */
/* Builds grid, constants and the fresh-start state the reference reaches after
 * GRID3 + SETUP + SBC + gen_initial_guess (Grid3.f90:8-300, Setup.f90:223-731,
 * Sbc.f90:19-388, Initsv.f90:97-162).  The interpolation part of INITSV
 * (INTPV, EXTR(1), INTP; Initsv.f90:63-84) is left to gfm_gpu_initsv. */
int  gfm_case_build(const gfm_case_spec *spec, const char *kinetic_path,
                    gfm_case *out);
void gfm_case_free(gfm_case *c);

/* ---- host side: a case from the reference's own input files -------------- */
/* Paths of the files a GFM case directory holds. */
typedef struct gfm_case_files {
    const char *gd;       /* gd####c.dat: grid and cell map (Grid3.f90:31-280)   */
    const char *sbc;      /* sbc####c.dat: &INPUT, inlet blocks, exhausts, wall
                             properties, &RADIN, band edges (Setup.f90:227-335,
                             Sbc.f90:57-355)                                     */
    const char *relax;    /* relaxfactorc.txt (Setup.f90:443-509)                */
    const char *it;       /* it####t.dat melt-surface temperatures
                             (Initsv.f90:394-547); needed when the cell map has
                             melt-surface cells (IBCELL=4), else may be NULL     */
    const char *rg;       /* rg####c.d restart (Initsv.f90:225-316); NULL: fresh
                             start by gen_initial_guess (Initsv.f90:97-162)      */
    const char *kinetic;  /* Kinetic.d (Setup.f90:858-888)                       */
    const char *rr;       /* rr####c.d radiation restart (rad_emis_rr,
                             Rad_emis.f90:17-110), read after rg: QE, QA and
                             the wall temperatures of the last exchange
                             (wall_rad_T into T and H at the closed wall
                             cells); NULL: QE and QA start from zero         */
} gfm_case_files;

/* Choices the input files do not carry. */
typedef struct gfm_case_options {
    double sigma_eps;     /* turbulent Prandtl number of epsilon, sigma(5); the
                             reference's value is 1.0 (Var_mod.f90:211-212)      */
    int    wall_sink;     /* fixed-temperature wall sink every iteration
                             (Source.f90:473-509); the reference starts it only
                             after its first full radiation call: 0            */
    double t_wall_k;      /* wall-patch temperature of that sink (K)             */
    int    rad_emission;  /* emission-only radiation source (rad_qe_only)        */
    double kappa[16];     /* gray absorption coefficient per band (1/m), in the
                             place of the band model of RAD_GAS                  */
    int    maxgi;         /* > 0: replaces &INPUT MAXGI                           */
    int    adi_mode, precision;
    int    gas_model;     /* 1: RAD_GAS and SOOTA on the minor species in the
                             place of kappa (needs MS=1 in &INPUT)               */
} gfm_case_options;

/* What GRID3 and SBC derived, as the reference prints it at the head of
 * summary####c.txt (Utility.f90:99-105), plus the run controls read. */
typedef struct gfm_case_summary {
    int    ncells;              /* open cells                                  */
    double area_melt_surf;      /* m2 (Grid3.f90:288-293)                      */
    double fr_f, fr_ox, fr_n2;  /* inlet fuel, O2, N2 mass flows (kg/s)        */
    double heat_in_fuel;        /* FR_F*Q0 (W)                                 */
    double q_h_in;              /* sum of inlet mdot*h (W)                     */
    double gmfr, gfin0;         /* &INPUT GMFR (kg/s); inflow / GMFR           */
    int    irstyp, id_rad, interval_rad;
    int    n_inlet_blocks, n_exhausts, n_wall_blocks, n_melt_cells;
    int    restarted;           /* the fields come from files->rg              */
    int    itr_gas;             /* restored iteration count (0 on a fresh start) */
} gfm_case_summary;

/* GRID3 + SETUP + SBC + INITSV (fresh start or restart) from the case files:
 * the start-up a Fortran host does before the first GFLOW
 * (A0main.f90:158-190).  Parse errors return GFM_E_IO.  Half-blocked cells
 * (digits 9 and 8, IBCELL -1 and -2) are read with the &GRD factors BV_F
 * and BA_F into the grid; digits 7 and 6 (IBCELL -3, -4, past the two
 * entries of BV_F, Grid3.f90:12) and two-phase cases return
 * GFM_E_UNSUPPORTED.  summary may be NULL. */
int  gfm_case_read(const gfm_case_files *files, const gfm_case_options *opt,
                   gfm_case *out, gfm_case_summary *summary);

/* Writes the synthetic furnace of a gfm_case_spec as a GFM case directory:
 * gd<runum>c.dat, sbc<runum>c.dat and relaxfactorc.txt in dir, in the
 * formats GRID3, SETUP and SBC read (Grid3.f90:31-280, Setup.f90:227-509,
 * Sbc.f90:57-355).  No reference counterpart: the reference's GUI writes
 * these files.  gfm_case_read of the written files, with the spec's
 * sigma_eps, wall sink, wall temperature, emission switch, kappa, line order
 * and precision as options, gives the case gfm_case_build gives.  A spec with
 * a seeded perturbation (noise_amp) or sigma_k other than 1 returns
 * GFM_E_UNSUPPORTED: the files cannot carry them. */
int  gfm_case_write_files(const gfm_case_spec *spec, const char *dir,
                          const char *runum);

/* Writes the restart file rg####c.d of the state (grid, fields, tail) in
 * the record layout of SAV3F (Sav3f.f90:21-88): sequential unformatted,
 * 4-byte little-endian record-length markers, one (P, U(i+1), V(j+1),
 * W(k+1), T, THETA) record and one GF(1:7) record per cell centre in I, J, K
 * loop order, then bs_hprev, T_surf_prev, FACTOR/FADJ, i1st_rad_qe_done,
 * i1st_rad_done, itr_gas, itr_rad/itr_gend and interval_rad. */
int  gfm_restart_write(const char *path, const gfm_grid *grid,
                       const gfm_fields *f, const gfm_restart_tail *tail);

/* Reads / writes the minor species restart rs####c.d in the record layout of
 * SAV3FM (Sav3f.f90:96-117; read by INITSVM, Initsv.f90:350-372): one record
 * GFM(1:7), smf per cell centre in I, J, K loop order, then bs_soot_prev,
 * sfp_soot_prev, RRMS and itr_ms.  `out`'s arrays are the caller's, sized
 * by the grid. */
int  gfm_minor_read(const char *path, const gfm_grid *grid, gfm_minor *out);
int  gfm_minor_write(const char *path, const gfm_grid *grid, const gfm_minor *m);

/* ---- GPU solver ---------------------------------------------------------- */
/* Query: number of CUDA devices usable (>=1) or a negative status. */
int  gfm_gpu_device_count(void);
/* Allocates device mirrors for the grid and the constants; uploads the static
 * geometry and the boundary index tables. */
int  gfm_gpu_create(const gfm_grid *grid, const gfm_params *params,
                    gfm_handle **out);
/* Host fields (reference layout) -> device. */
int  gfm_gpu_upload(gfm_handle *h, const gfm_fields *f);
/* INTPV, EXTR(1), INTP on the device: the tail of INITSV (Initsv.f90:63-84). */
int  gfm_gpu_initsv(gfm_handle *h);
/* n_iter passes of SPHASE's loop body: itr_gas+=1, GFLOW, convergence test,
 * emission-only radiation cadence (Sphase.f90:37-235).  Stops early when
 * res_mass < BGCON.  `out` (may be NULL) receives the last iteration's stats;
 * `n_done` (may be NULL) the number of iterations run. */
int  gfm_gpu_gflow(gfm_handle *h, int n_iter, gfm_iter_stats *out, int *n_done);
/* The same for n independent handles (furnace variants) at once: every
 * iteration is queued on all handles' streams before any is waited for, so
 * their kernels overlap on the GPU.  A handle stops at its own convergence;
 * out[i] / n_done[i] (either may be NULL) receive each handle's result.  No
 * counterpart in the reference, which runs one furnace per process. */
int  gfm_gpu_gflow_batch(gfm_handle *const *hs, int n, int n_iter,
                         gfm_iter_stats *out, int *n_done);
/* Device -> host fields (reference layout). */
int  gfm_gpu_download(gfm_handle *h, gfm_fields *f);
/* One ADLBL3 call on a user system (Adlbl3.f90:10-97): xt, ap, as (6 arrays
 * AS(..,L,M) in the order (1,1),(1,2),(2,1),(2,2),(3,1),(3,2)), bs in the
 * reference layout; solves in place on the class of (ib,jb,kb) with the sweep
 * count nim.  Uses the handle's grid (IBCELL) and adi_mode/precision. */
int  gfm_gpu_adlbl3(gfm_handle *h, double *xt, const double *ap,
                    const double *const as[6], const double *bs,
                    int ib, int ie, int jb, int je, int kb, int ke, int nim);
/* Emission-only radiation QE on the device from the current T, P
 * (rad_qe_only, Rad_emis.f90:411-466 with RAD0 Rad0.f90:112-157). */
int  gfm_gpu_rad_emission(gfm_handle *h);

/* Results of one wall radiosity exchange (wallq, Qwall.f90:990-1365;
 * wall_q_amb, Qwall.f90:1585-1660), W unless stated. */
typedef struct gfm_wall_totals {
    int    b_cnt;                /* boundary patches                           */
    int    sweeps;               /* radiosity sweeps done (iterw increments)   */
    int    outer;                /* outer passes (q_conv, T update, q_amb)     */
    int    reserved;
    double avg_wall_T;           /* area-weighted mean wall T (K)              */
    double q_melt;               /* net flux into the melt surface             */
    double q_wall_loss;          /* loss through the walls to ambient          */
    double q_incident_total, q_incident_wall, q_incident_inlet, q_incident_exit, q_incident_melt;
    double qconv_total;          /* convection from the gas to the boundaries  */
    double q_rad_inlet, q_rad_outlet;
    double qm_flame, qm_bnds, qm_conv;
    double rel_rad_chg_mean;     /* last sweep's mean relative radiosity change */
} gfm_wall_totals;

/* Totals of one volume radiation transfer, W (Qrn.f90:73-87, Qre.f90:511-514,
 * Rad0.f90:137-148). */
typedef struct gfm_rad_totals {
    double qe_sum_from_open;     /* emission of the traced open cells          */
    double qa_sum_to_open;       /* absorbed in open cells                     */
    double qa_sum_to_wall, qa_sum_to_inlet, qa_sum_to_exit, qa_sum_to_melt;
                                 /* deposited on boundary cells, by IBCELL      */
    double tot_qe_h2o_co2, tot_qe_soot;    /* RAD0 band-emission totals         */
    int    n_emitters;           /* open cells with T > TG_MN that were traced  */
    int    reserved;
} gfm_rad_totals;
/* Volume radiation transfer on the device from the current T: the volume part
 * of CALL RAD_EMIS (A0main.f90:232) -- wall markers (Rad_emis.f90:144-178),
 * RAD0 with ID_RAD=10 (Rad0.f90:112-166), the QRNF emitter loop
 * (Qrn.f90:58-229) with QREF and QRTX/QRTY/QRTZ (Qre.f90:31-515,
 * Qrtx.f90:15-209, Qrty.f90:9-224, Qrtz.f90:15-234), and QA = sum of QAL over
 * the bands (QRN1, Qrn.f90:250-259).  QE and QA of the handle are replaced and
 * the enthalpy source uses QA - QE from then on (Source.f90:437-439).  The
 * wall exchange that follows in QRNF (wall_q_amb, wallq, qrn2) is not done.
 * `out` (may be NULL) receives the totals.  Grids whose slab work arrays
 * exceed the device limit, or geometries that reach the reference's
 * undefined corner case (a wall-corner split on the emitter's own column),
 * return GFM_E_UNSUPPORTED / GFM_E_LIMIT. */
int  gfm_gpu_rad_transfer(gfm_handle *h, gfm_rad_totals *out);
/* The wall radiosity exchange that follows the volume transfer in QRNF
 * (Qrn.f90:209-211: wall_q_amb, wallq; Qwall.f90:990-1245, 1585-1655).
 * gfm_gpu_wall_setup forms the patch data of the case's boundary patches
 * (prepare_for_wall_radiation_calculation steps 5-8, Qwall.f90:395-736) and
 * the normalised view factors on the device (nb x nb, FP64 on the FP64 path,
 * FP32 on the mixed one; GFM_E_NOMEM when they do not fit); from then on every
 * gfm_gpu_rad_transfer ends with the exchange: patch temperatures at the
 * first call (Rad_emis.f90:186-273), radiosity sweeps with the reference's
 * stopping rules, wall temperatures written into T, and the wall sink and EXTR
 * of the following iterations use them (Extr.f90:194-197).  The sweeps read
 * the previous sweep's radiosities (Jacobi) where the reference updates in
 * patch order; both reach the same fixed point.  Every exit patch must lie in
 * an exhaust of `spec`.  gfm_gpu_wall_totals returns the last exchange's
 * results; gfm_gpu_wall_get copies one per-patch array ("b_t", "radiosity",
 * "q_amb", "q_conv", "qc", "qeb", "emis", "b_face_area", "patch_area", "rad" the
 * radiation from the boundaries, "qrs" the melt-surface heat flux of the melt
 * patches, Qwall.f90:1166; the patch list "b_typ", "b_i", "b_j", "b_k",
 * "b_orient", "b_direct", the closed cell "bc_i", "bc_j", "bc_k", the exhaust
 * "b_exh" and "vf_sum", the view factors' row sums before normalisation,
 * Qwall.f90:562-666) and returns the patch count.  gfm_gpu_wall_vf copies the
 * normalised view factors, row n (the near patch) at out[n*b_cnt .. ], and
 * returns b_cnt*b_cnt (cap: elements of out).
 * gfm_gpu_wall_put restores the state the radiation restart holds
 * (rad_emis_rr, Rad_emis.f90:17-88): "radiosity" and "b_t" (n = b_cnt; the
 * next exchange then keeps the given wall temperatures, as after an earlier
 * exchange), and the scalars "iterw", "q_melt" and "avg_wall_T" (n = 1). */
int  gfm_gpu_wall_setup(gfm_handle *h, const gfm_wall_spec *spec);
int  gfm_gpu_wall_totals(gfm_handle *h, gfm_wall_totals *out);
int  gfm_gpu_wall_get(gfm_handle *h, const char *name, double *out, int cap);
long long gfm_gpu_wall_vf(gfm_handle *h, double *out, long long cap);
int  gfm_gpu_wall_put(gfm_handle *h, const char *name, const double *src, int n);
/* Minor species and soot on the device (ms=1 of the reference).
 * gfm_gpu_minor_upload / _download move the MSFLOW state.  gfm_gpu_initsvm is
 * INITSVM (Initsv.f90:329-378): restart = 0 starts from the major species
 * (GFM 1, 2, 4, 5, 6 from GF, CO, NO and soot zero); restart = 1 keeps the
 * uploaded state but resets the inlet cells to the major species and
 * extrapolates the exits (EXTRM); both end with INTPM.  gfm_gpu_msflow runs
 * MSFLOW (Msflow.f90:10-169) on the frozen flow: up to maxms iterations of
 * GSLV3M (reaction rates, the seven species and soot, Gslv3m.f90:8-286),
 * EXTRM and INTPM, stopping when every resid_ms <= BMCON after iteration 10;
 * `out` (may be NULL) receives the last iteration's figures.
 * With params.gas_model = 1 the emission and the volume transfer take their
 * absorption coefficients from RAD_GAS and SOOTA on this state
 * (Rad0.f90:116-132, Rad_gas.f90:16-395, Rad_soot.f90:26-69) instead of the
 * gray akl0, and gfm_gpu_gflow's first emission update runs INITSVM (a
 * restart when IRSTYPM = 1 and a state was uploaded) and MSFLOW(300) before
 * it, as SPHASE does (Sphase.f90:210-224).  Without a minor species state
 * the band model returns GFM_E_ARG. */
int  gfm_gpu_minor_upload(gfm_handle *h, const gfm_minor *m);
int  gfm_gpu_minor_download(gfm_handle *h, gfm_minor *m);
int  gfm_gpu_initsvm(gfm_handle *h, int restart);
int  gfm_gpu_msflow(gfm_handle *h, int maxms, gfm_msflow_stats *out);
/* Device times (CUDA events on the handle's stream) accumulated since the
 * last reset: adi_ms = line-solver batches, gflow_ms = whole GFLOW calls
 * (first to last iteration of each gfm_gpu_gflow), other_ms reserved;
 * launches = kernels launched by gfm_gpu_gflow. */
int  gfm_gpu_kernel_times(gfm_handle *h, double *adi_ms, double *gflow_ms,
                          double *other_ms, long long *launches);
int  gfm_gpu_reset_kernel_times(gfm_handle *h);
/* Shape of one captured iteration: kernel launches per GFLOW, line-solver
 * kernel launches per GFLOW, and cells x plane-visits of all line solves. */
int  gfm_gpu_iteration_profile(gfm_handle *h, long long *kernels_per_iter,
                               long long *adi_kernels_per_iter,
                               double *adi_cell_visits_per_iter);
/* Last error text of this handle (never NULL). */
const char *gfm_gpu_last_error(gfm_handle *h);
void gfm_gpu_destroy(gfm_handle *h);

/* ---- learned initial guess for the p' equation --------------------------- */
/* No counterpart in the reference (which starts every p' solve from zero,
 * Gslv3v.f90:157-161).  A 3-D convolutional encoder-decoder (BF16 tensor-core
 * kernels, FP32 accumulation) maps the Jacobi-scaled right-hand side of the
 * p' system on the voxel grid of its solve range (nx = MP/2-2, ny = NP/2-2,
 * nz = LP/2-2, all even) to the shape of p' (unit RMS); in the solver the
 * guess is that shape times the factor minimising the p' residual, and the
 * line solver starts from it.
 * Inputs are BF16 tensors of 16 channels per voxel, voxel (z*ny+y)*nx+x;
 * targets and outputs are FP32, one value per voxel.  Device pointers; calls
 * are queued on `stream` (NULL = legacy default stream). */
int  gfm_lp_create(int nx, int ny, int nz, uint64_t seed, gfm_lp **out);
void gfm_lp_destroy(gfm_lp *lp);
int  gfm_lp_num_params(void);
/* FP32 parameters / accumulated gradients to host (either may be NULL);
 * setting the parameters resets the optimiser. */
int  gfm_lp_get_params(gfm_lp *lp, float *params, float *grads);
int  gfm_lp_set_params(gfm_lp *lp, const float *params);
int  gfm_lp_forward(gfm_lp *lp, const void *feats, float *out,
                    int nx, int ny, int nz, void *stream);
/* One sample: forward, loss (mean squared error over open voxels, returned in
 * *loss when not NULL, which waits for the stream), gradients; an Adam step
 * with learning rate lr when update != 0. */
int  gfm_lp_train_step(gfm_lp *lp, const void *feats, const float *target,
                       int nx, int ny, int nz, float lr, int update,
                       double *loss, void *stream);
/* Forward convolutions on the tcgen05 tensor cores (1, the default) or on
 * warp-level mma.sync (0); gradients always use mma.sync.  Status since
 * creation (waits for the device): 0 when every tcgen05 tile's bounded wait
 * for its MMAs succeeded; 1 when a tile's first wait ran out, after which it
 * waited again, saw its MMAs end and wrote its output; 2 when a tile's second
 * wait ran out too: the tile released its tensor memory without writing its
 * output, so the forward pass's result is invalid. */
int  gfm_lp_set_tensor_path(gfm_lp *lp, int tcgen05);
int  gfm_lp_tensor_status(gfm_lp *lp);
const char *gfm_lp_last_error(void);
/* Training sample from the p' system of the handle's last iteration: inputs
 * to `feats`, and to `target` the system's solution after `nsweeps` line-
 * solver sweeps from zero, scaled to unit RMS over the open cells.  dims
 * receives nx, ny, nz.  Synchronous. */
int  gfm_gpu_pcorr_sample(gfm_handle *h, int nsweeps, void *feats,
                          float *target, int *dims);
/* Use the network's guess as the start of every p' solve (NULL: start from
 * zero, as the reference).  The guess g is scaled by alpha minimising
 * |b - alpha*A g| (FP64) and kept when that residual is below |b|, the
 * residual of the zero start (gfm_iter_stats.lp_used, lp_ratio). */
int  gfm_gpu_set_lp(gfm_handle *h, gfm_lp *lp);

/* ---- line solve without any device allocation ---------------------------- */
/* No counterpart in the reference: an addition for callers that cannot
 * allocate device memory -- code running inside a host program that owns all
 * of it (another framework's caching allocator, a pool sized once at start-up,
 * a process under a device-memory quota) must not call cudaMalloc behind that
 * host's back, so it cannot create a gfm_gpu handle.
 *
 * Same solve as gfm_gpu_adlbl3 in GFM_ADI_MARCH order with FP64 arithmetic, but
 * every array is a DEVICE pointer owned by the caller, in the reference layout
 * (column-major A(MP,NP,LP), mp*np*lp doubles each; ibcell mp*np*lp int16):
 * xt is solved in place, ap, the six as[q] (the array of six pointers itself is
 * host memory) and bs are read.  Nothing is allocated: the working storage is
 * one fixed device array inside the library, 2 MiB per GPU that loads it, held
 * until the process exits.  Limit: one x-plane of the solved class may hold at
 * most 65536 (J,K) points, ((je-jb)/2+1)*((ke-kb)/2+1) <= 65536; larger planes
 * return GFM_E_LIMIT.  Index ranges as for gfm_gpu_adlbl3; pointers that are
 * not device memory of the current device return GFM_E_ARG.
 *
 * The kernel is queued on `stream` (a cudaStream_t; NULL = the legacy default
 * stream) and the call returns without waiting for it.  Each call looks up the
 * device address of the working storage in the current context
 * (cudaGetSymbolAddress); a call on a capturing stream uses the address found
 * by the last call on that device outside a capture, so make the first call on
 * each device before any stream capture starts.  The CUDA runtime may load the
 * working storage only at the first call on a device (lazy module loading): a
 * host that reserves the device's memory for its own pool should make one call
 * with nim = 0 (no device work) before it does.  A plane with a single z-row
 * (kb == ke) takes the y-line pass alone, as the reference's ADLZ does
 * (Adlbl3.f90:124-130).  Every call uses the same working storage, so calls
 * whose kernels can overlap on the GPU (other streams, other host threads)
 * race and give wrong results: order them. */
int  gfm_adlbl3_noalloc(int mp, int np, int lp, const int16_t *ibcell,
                        double *xt, const double *ap,
                        const double *const as[6], const double *bs,
                        int ib, int ie, int jb, int je, int kb, int ke,
                        int nim, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GFM_GB300_H */
