// solver.cu -- host orchestration of the GB300 solver behind the C ABI
// (include/gfm_gb300.h): geometry and boundary tables built once on the host,
// device state, upload/download in the reference layout, and the GFLOW
// sequence (Gflow.f90:6-408) issued on one CUDA stream per handle.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <map>
#include <mutex>
#include <type_traits>

#include <cuda_bf16.h>
#include <cmath>
#include <initializer_list>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/gfm_gb300.h"
#include "state.cuh"
#include "lp.cuh"

using namespace gfm;

namespace {

// reduction slots (partials rows)
enum Slot {
    SL_RESM = 0, SL_RESMAX = 1, SL_QCONV = 4, SL_QREACT = 5, SL_TA = 6, SL_TB = 7, SL_GFIN0 = 8, SL_QEX = 9,
    SL_GFEX = 10, SL_TM = 11, SL_TAREA = 12, SL_AREA = 13,
    SL_P_PRE = 16, SL_P_POST = 17, SL_PC_POST = 18, SL_U_PRE = 19, SL_U_POST = 22, SL_GF_PRE = 25, SL_GF_POST = 32
};

struct HostGrid {
    int MP, NP, LP;
    std::vector<int16_t> ib;   // doubled layout
    std::vector<double> X, DX, R, DR, RS, Z, DZ;   // 1-based
    double bvf[2], baf[6];     // half-block factors BV_F, BA_F
    int half;                  // the grid has half-blocked cells
    int at(int i, int j, int k) const { return ib[(i - 1) + (long)MP * ((j - 1) + (long)NP * (k - 1))]; }
};

}  // namespace

constexpr int kXferSlots = 22;   // P T DNST THETA TMU GAMA CRATE HRATE BSH, UG x3, GF x8, QA, QE
// Copies of one transfer go round-robin over this many streams.  From 1 to 8
// streams the rate stayed at about 215 GB/s host-to-device and 173 GB/s back
// (1.71 GB of FP64 state); kernels reading and writing page-locked host arrays
// in place reached the same rates, so the copies are kept.
constexpr int kXferStreams = 2;

struct gfm_handle {
    int prec = GFM_PREC_FP64;
    int adi_mode = GFM_ADI_MARCH;
    gfm_params params{};
    HostGrid hg;
    long long N = 0, CB = 0, NS = 0;
    int ncells = 0;
    GeoT<double> gd{};
    GeoT<float> gfl{};
    Ctx<double> cd{};
    Ctx<float> cf{};
    AdiScratch<double> scr_d[8]{};
    AdiScratch<float> scr_f[8]{};
    std::vector<void*> allocs;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_adi0 = nullptr, ev_adi1 = nullptr;
    int* d_wall = nullptr;
    int n_wall = 0;
    double* d_stage = nullptr;      // doubled-layout staging buffer (N doubles)
    // upload/download of the whole state: one staging slot per field, host
    // copies on their own stream, ordered by events against the layout kernels
    double* d_stage_all = nullptr;  // kXferSlots x N doubles (allocated at the first transfer)
    unsigned int* d_bad_all = nullptr;
    cudaStream_t copy_stream[kXferStreams]{};   // fields go round-robin over these
    cudaEvent_t ev_xfer[kXferSlots + 1]{};
    unsigned int* d_bad = nullptr;  // non-finite counter of uploaded arrays
    double* h_scal = nullptr;       // pinned copy of the device scalars
    int pref_i1 = 0, pref_j1 = 0, pref_k1 = 0, pref_i2 = 0, pref_j2 = 0, pref_k2 = 0;
    double pref_f1 = 1, pref_f2 = 0;
    int itr_gas = 0, cnt_qe = 0, rad_active = 0;
    double q_h_in = 0;
    double adi_ms = 0, asm_ms = 0, other_ms = 0;
    long long launches = 0;
    std::string err;
    // one GFLOW captured as a CUDA graph and replayed every iteration
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    bool use_graph = true;
    double* h_flags = nullptr;          // pinned: itr_gas, rad_active for the next replay
    cudaEvent_t ev[16]{};
    cudaEvent_t ev_g0 = nullptr, ev_g1 = nullptr;   // around a whole gfm_gpu_gflow call
    int n_ev = 0;                       // events recorded per iteration (pairs around line solves)
    long long kernels_per_iter = 0;     // kernel nodes of the captured iteration
    long long adi_kernels_per_iter = 0;
    double adi_cells_visits = 0;        // cells x plane visits per iteration (all line solves)
    // learned p' initial guess (not owned)
    gfm::lp::Net* lp = nullptr;
    void* lp_feats = nullptr;           // BF16 inputs, 16 channels per voxel
    int lp_nx = 0, lp_ny = 0, lp_nz = 0;
    // volume radiation transfer (allocated by the first gfm_gpu_rad_transfer)
    RadArgs rad{};                      // buffers and launch plan of the transfer (once per handle)
    bool rad_ready = false;
    cudaStream_t rad_stream[2]{};       // the y- and z-direction traces run beside the x-direction
    cudaEvent_t rad_ev[3]{};
    int rb_flags = kRbPlane | kRbPdl | kRbAvgInPass;   // red-black options (environment at create): GFM_RB_PLANE=0
                                                       // drops kRbPlane, GFM_PDL=0 kRbPdl, GFM_RB_AVG_IN_PASS=0
                                                       // kRbAvgInPass
    // line-solver autotuning (red-black order): the line-solver calls of one
    // iteration are recorded while it is captured; before the first
    // iteration each is timed in every form on stand-in systems of its shape
    // and the fastest form's flags are kept for it (GFM_RB_TUNE=0: no tuning)
    struct AdiSite {
        int nsys;
        int rng[8][7];                  // ib, ie, jb, je, kb, ke, nim of each system
    };
    std::vector<AdiSite> sites;
    bool record_sites = false, tune = true, tuned = false;
    int adi_site = 0;                   // call index inside the iteration being issued
    std::vector<int> site_flags;        // chosen flags per call site (empty: rb_flags)
    std::vector<std::array<float, 3>> site_ms;   // measured ms of the three forms per call site
    // wall radiosity exchange (gfm_gpu_wall_setup): the case's patch list,
    // the device data, and the state that carries from one exchange to the next
    std::vector<int16_t> bp_typ, bp_i, bp_j, bp_k, bp_ori, bp_dir;
    Patch* d_patches = nullptr;         // the wall-sink patches (b_T written by the exchange)
    bool wall_on = false;
    gfm_wall_spec wspec{};
    WallArgs wall{};
    std::vector<int> wall_typ, wall_exh;
    double wall_area_total = 0;
    int wall_first = 1, iterw = 0, wall_frac_exits = 0;
    int* d_frac_exit = nullptr;
    double* d_frac = nullptr;
    double avg_wall_T = 1600.0, q_melt = 0.0;   // Qwall.f90:68; q_melt starts at zero
    gfm_wall_totals wall_last{};        // results of the last exchange
    // minor species and soot (gfm_gpu_minor_upload), the band model's buffers
    MinorDev<double> mnd{};
    MinorDev<float> mnf{};
    bool minor_on = false, minor_from_host = false;
    int itr_ms = 0, imscon = 0;
    GasBuffers gas{};
    // MSFLOW's scratch; the coefficient array of the reference holds the
    // minor species' set (true) or the last gas equation's (false)
    MsScratch<double> msd{};
    MsScratch<float> msf{};
    bool as_minor_current = false;
    int igs0 = 0;
    double resid_ms_pre[8]{}, resid_ms[8]{};
    double vol_tot = 0;                 // open volume (IBCELL = 0), Grid3.f90:286-294
};

namespace {

#define CK(x)                                                                          \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess) {                                                       \
            h->err = std::string(#x) + ": " + cudaGetErrorString(e_);                  \
            return GFM_E_CUDA;                                                         \
        }                                                                              \
    } while (0)

template <typename T>
int dalloc(gfm_handle* h, T** p, long long n) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, (size_t)n * sizeof(T));
    if (e != cudaSuccess) {
        h->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return GFM_E_NOMEM;
    }
    cudaMemset(q, 0, (size_t)n * sizeof(T));
    h->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return GFM_OK;
}

template <typename T>
int dupload(gfm_handle* h, T** p, const std::vector<T>& v) {
    long long n = v.empty() ? 1 : (long long)v.size();
    int rc = dalloc(h, p, n);
    if (rc) return rc;
    if (!v.empty()) CK(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return GFM_OK;
}

// ---- host replicas of the reference index helpers (Extr.f90:311-661) --------
void extr1(const HostGrid& g, double& F1, double& F2, int I, int J, int K, int I1, int J1, int K1, int I2, int J2, int K2, int IX) {
    F2 = 0.0;
    int ibc0 = g.at(I, J, K) % 10;
    if (IX == 3) {
        double d = g.Z[K2] - g.Z[K1];
        if (d != 0.0) { int K0 = ibc0 == 2 ? (K + K1) / 2 : K; F2 = (g.Z[K0] - g.Z[K1]) / d; }
    } else if (IX == 2) {
        double d = g.R[J2] - g.R[J1];
        if (d != 0.0) { int J0 = ibc0 == 2 ? (J + J1) / 2 : J; F2 = (g.R[J0] - g.R[J1]) / d; }
    } else if (IX == 1) {
        double d = g.X[I2] - g.X[I1];
        if (d != 0.0) { int I0 = ibc0 == 2 ? (I + I1) / 2 : I; F2 = (g.X[I0] - g.X[I1]) / d; }
    }
    F1 = 1.0 - F2;
}
bool ext01(const HostGrid& g, bool wall, int I, int J, int K, int& I1, int& J1, int& K1, int& I2, int& J2, int& K2, int& IX) {
    auto cl = [](int v, int hi) { return v < 2 ? 2 : (v > hi ? hi : v); };
    for (IX = 1; IX <= 3; ++IX) {
        int nx = IX == 1, ny = IX == 2, nz = IX == 3;
        for (int M = -2; M <= 2; M += 4) {
            I1 = cl(I + M * nx, g.MP); J1 = cl(J + M * ny, g.NP); K1 = cl(K + M * nz, g.LP);
            bool hit = wall ? (g.at(I1, J1, K1) % 10 != 1) : (g.at(I1, J1, K1) <= 0);
            if (hit) {
                I2 = cl(I1 + M * nx, g.MP); J2 = cl(J1 + M * ny, g.NP); K2 = cl(K1 + M * nz, g.LP);
                if (g.at(I2, J2, K2) % 10 == 1) { I2 = I1; J2 = J1; K2 = K1; }
                return true;
            }
        }
    }
    IX = 4;
    I2 = I1; J2 = J1; K2 = K1;
    return false;
}

int build_tables(gfm_handle* h, const gfm_grid* gr, std::vector<int>& wall_list, std::vector<ExtrRec>& io,
                 std::vector<ExtrRec>& walls, std::vector<ExtrRec>& ft, std::vector<int>& ft_start,
                 std::vector<ExtrvRec>& ev, int nev[3], std::vector<Patch>& patches, std::vector<int>& cp_start,
                 std::vector<int>& cp_list, std::vector<int8_t>& intp_mode_split) {
    const HostGrid& g = h->hg;
    const int MP = g.MP, NP = g.NP, LP = g.LP;
    // ---- wall positions of the wall-function pass (Gflow.f90:67-130)
    for (int K = 2; K <= LP; ++K)
        for (int J = 2; J <= NP; ++J)
            for (int I = 2; I <= MP; ++I) {
                if (g.at(I, J, K) != 1) continue;
                const int dirs[6][4] = {{1, 0, 0, 1}, {0, 1, 0, 1}, {0, 0, 1, 1}, {0, 0, 1, -1}, {0, 1, 0, -1}, {1, 0, 0, -1}};
                for (int q = 0; q < 6; ++q) {
                    int s = dirs[q][3];
                    int In = I + s * dirs[q][0], Jn = J + s * dirs[q][1], Kn = K + s * dirs[q][2];
                    if (In < 2 || In > MP || Jn < 2 || Jn > NP || Kn < 2 || Kn > LP) continue;
                    if (g.at(In, Jn, Kn) >= 1) continue;
                    int If = In + 2 * s * dirs[q][0], Jf = Jn + 2 * s * dirs[q][1], Kf = Kn + 2 * s * dirs[q][2];
                    if (If < 1 || If > MP || Jf < 1 || Jf > NP || Kf < 1 || Kf > LP || g.at(If, Jf, Kf) == 1) {
                        h->err = "geometry: wall-function extrapolation point is a wall (channel narrower than 2 cells)";
                        return GFM_E_UNSUPPORTED;
                    }
                }
                wall_list.push_back(I); wall_list.push_back(J); wall_list.push_back(K);
            }
    // ---- EXTR records (Extr.f90:31-250)
    for (int I = 2; I <= MP; I += 2)
        for (int J = 2; J <= NP; J += 2)
            for (int K = 2; K <= LP; K += 2) {
                int b = g.at(I, J, K) % 10;
                if (b != 2 && b != 3) continue;
                ExtrRec e{};
                e.I = I; e.J = J; e.K = K; e.kind = b;
                if (!ext01(g, false, I, J, K, e.I1, e.J1, e.K1, e.I2, e.J2, e.K2, e.IX)) {
                    h->err = "geometry: inlet/exit cell without an open neighbour";
                    return GFM_E_UNSUPPORTED;
                }
                if (g.at(e.I2, e.J2, e.K2) > 0) {
                    h->err = "geometry: inlet/exit extrapolation reads another boundary cell";
                    return GFM_E_UNSUPPORTED;
                }
                extr1(g, e.F1, e.F2, I, J, K, e.I1, e.J1, e.K1, e.I2, e.J2, e.K2, e.IX);
                e.I3 = (I + e.I1) / 2; e.J3 = (J + e.J1) / 2; e.K3 = (K + e.K1) / 2;
                io.push_back(e);
            }
    std::vector<std::vector<ExtrRec>> cols;
    std::vector<long> col_key;
    for (int I = 2; I <= MP; I += 2)
        for (int J = 2; J <= NP; J += 2) {
            std::vector<ExtrRec> col;
            for (int K = 2; K <= LP; K += 2) {
                if (g.at(I, J, K) % 10 != 1) continue;
                ExtrRec e{};
                e.I = I; e.J = J; e.K = K; e.kind = 1;
                bool found = ext01(g, true, I, J, K, e.I1, e.J1, e.K1, e.I2, e.J2, e.K2, e.IX);
                extr1(g, e.F1, e.F2, I, J, K, e.I1, e.J1, e.K1, e.I2, e.J2, e.K2, e.IX);
                if (found) walls.push_back(e); else col.push_back(e);
            }
            if (!col.empty()) cols.push_back(col);
        }
    ft_start.push_back(0);
    for (auto& col : cols) {
        for (auto& e : col) ft.push_back(e);
        ft_start.push_back((int)ft.size());
    }
    // ---- EXTRV records (Extr.f90:358-567), per direction in loop order
    std::vector<char> wmark((size_t)MP * NP * LP * 3, 0);
    auto lin = [&](int i, int j, int k) { return (size_t)(i - 1) + (size_t)MP * ((j - 1) + (size_t)NP * (k - 1)); };
    for (int IU = 1; IU <= 3; ++IU) {
        int cnt = 0;
        std::vector<size_t> writes, reads;
        auto visit = [&](int I, int J, int K) {
            if (g.at(I, J, K) % 10 != 3) return;
            ExtrvRec e{};
            e.I = I; e.J = J; e.K = K; e.IU = IU; e.mode = 2;
            for (int M = -1; M <= 1; M += 2) {
                int In = I + (IU == 1) * M, Jn = J + (IU == 2) * M, Kn = K + (IU == 3) * M;
                if (g.at(In, Jn, Kn) >= 1) continue;
                e.mode = 0; e.m = M;
                break;
            }
            if (e.mode == 0) {
                int I1 = I + (IU == 1) * 2 * e.m, J1 = J + (IU == 2) * 2 * e.m, K1 = K + (IU == 3) * 2 * e.m;
                int I0 = I - (IU == 1) * e.m, J0 = J - (IU == 2) * e.m, K0 = K - (IU == 3) * e.m;
                writes.push_back(lin(I1, J1, K1));
                if (IU != 3) { writes.push_back(lin(I, J, K)); writes.push_back(lin(I0, J0, K0)); }
            } else {
                // fallback copies in the reference's priority order
                int Is = 0, Js = 0, Ks = 0;
                bool ok = false;
                if (IU == 1) {
                    if (J > 2 && g.at(I, J - 2, K) <= 0) { Is = I; Js = J - 2; Ks = K; ok = true; }
                    else if (J < NP && g.at(I, J + 2, K) <= 0) { Is = I; Js = J + 2; Ks = K; ok = true; }
                    else if (K > 2 && g.at(I, J, K - 2) <= 0) { Is = I; Js = J; Ks = K - 2; ok = true; }
                    else if (K < LP && g.at(I, J, K + 2) <= 0) { Is = I; Js = J; Ks = K + 2; ok = true; }
                } else if (IU == 2) {
                    if (K > 2 && g.at(I, J, K - 2) <= 0) { Is = I; Js = J; Ks = K - 2; ok = true; }
                    else if (K < LP && g.at(I, J, K + 2) <= 0) { Is = I; Js = J; Ks = K + 2; ok = true; }
                    else if (I > 2 && g.at(I - 2, J, K) <= 0) { Is = I - 2; Js = J; Ks = K; ok = true; }
                    else if (I < MP && g.at(I + 2, J, K) <= 0) { Is = I + 2; Js = J; Ks = K; ok = true; }
                } else {
                    if (I > 2 && g.at(I - 2, J, K) <= 0) { Is = I - 2; Js = J; Ks = K; ok = true; }
                    else if (I < MP && g.at(I + 2, J, K) <= 0) { Is = I + 2; Js = J; Ks = K; ok = true; }
                    else if (J > 2 && g.at(I, J - 2, K) <= 0) { Is = I; Js = J - 2; Ks = K; ok = true; }
                    else if (J < NP && g.at(I, J + 2, K) <= 0) { Is = I; Js = J + 2; Ks = K; ok = true; }
                }
                if (ok) {
                    e.mode = 1; e.Is = Is; e.Js = Js; e.Ks = Ks;
                    writes.push_back(lin(I, J, K));
                    reads.push_back(lin(Is, Js, Ks));
                }
            }
            ev.push_back(e);
            ++cnt;
        };
        if (IU == 1) { for (int I = 3; I <= MP - 1; I += 2) for (int J = 2; J <= NP; J += 2) for (int K = 2; K <= LP; K += 2) visit(I, J, K); }
        else if (IU == 2) { for (int J = 3; J <= NP - 1; J += 2) for (int K = 2; K <= LP; K += 2) for (int I = 2; I <= MP; I += 2) visit(I, J, K); }
        else { for (int K = 3; K <= LP - 1; K += 2) for (int I = 2; I <= MP; I += 2) for (int J = 2; J <= NP; J += 2) visit(I, J, K); }
        for (size_t w : writes) {
            if (wmark[w * 3 + IU - 1]) { h->err = "geometry: exit faces write one velocity twice"; return GFM_E_UNSUPPORTED; }
            wmark[w * 3 + IU - 1] = 1;
        }
        for (size_t r : reads)
            if (wmark[r * 3 + IU - 1]) { h->err = "geometry: exit face copy reads a rescaled velocity"; return GFM_E_UNSUPPORTED; }
        nev[IU - 1] = cnt;
    }
    // ---- wall patches and the per-cell patch lists (Qwall.f90:395-513)
    cp_start.assign((size_t)h->CB + 1, 0);
    std::vector<std::vector<int>> per_cell;
    std::vector<long long> cell_of;
    std::vector<int> counts((size_t)h->CB, 0);
    for (int n = 0; n < gr->b_cnt; ++n) {
        int typ = gr->b_typ[n];
        if (typ != 1 && typ != 4) continue;
        int bi = gr->b_i[n], bj = gr->b_j[n], bk = gr->b_k[n];
        Patch q{};
        q.inc = bi; q.jnc = bj; q.knc = bk;
        if (gr->b_orient[n] == 1) {
            if (gr->b_direct[n] == 0) { q.inc = bi + 1; q.ds_q = g.X[bi + 1] - g.X[bi]; } else { q.inc = bi - 1; q.ds_q = g.X[bi] - g.X[bi - 1]; }
            q.ds_src = g.DX[q.inc];
            q.area = g.DR[bj] * g.DZ[bk];
        } else if (gr->b_orient[n] == 2) {
            if (gr->b_direct[n] == 0) { q.jnc = bj + 1; q.ds_q = g.R[bj + 1] - g.R[bj]; } else { q.jnc = bj - 1; q.ds_q = g.R[bj] - g.R[bj - 1]; }
            q.ds_src = g.DR[q.jnc];
            q.area = g.DX[bi] * g.DZ[bk];
        } else {
            if (gr->b_direct[n] == 0) { q.knc = bk + 1; q.ds_q = g.Z[bk + 1] - g.Z[bk]; } else { q.knc = bk - 1; q.ds_q = g.Z[bk] - g.Z[bk - 1]; }
            q.ds_src = g.DZ[q.knc];
            q.area = g.DX[bi] * g.DR[bj];
        }
        q.bT = gr->b_t[n];
        if ((q.inc & 1) || (q.jnc & 1) || (q.knc & 1)) { h->err = "geometry: wall patch not next to a cell centre"; return GFM_E_UNSUPPORTED; }
        long long o = pidx(h->gd, q.inc, q.jnc, q.knc);
        counts[(size_t)o]++;
        patches.push_back(q);
    }
    for (long long o = 0; o < h->CB; ++o) cp_start[(size_t)o + 1] = cp_start[(size_t)o] + counts[(size_t)o];
    cp_list.assign(patches.size(), 0);
    std::vector<int> fill(cp_start.begin(), cp_start.end() - 1);
    for (size_t n = 0; n < patches.size(); ++n) {
        long long o = pidx(h->gd, patches[n].inc, patches[n].jnc, patches[n].knc);
        cp_list[(size_t)fill[(size_t)o]++] = (int)n;
    }
    // ---- INTP carried-F1 codes (Intp.f90:32-72, 145-175)
    intp_mode_split.assign((size_t)h->NS, 0);
    auto setm = [&](int I, int J, int K, int m) { intp_mode_split[(size_t)pidx(h->gd, I, J, K)] = (int8_t)m; };
    auto step = [&](int& cf, int I, int J, int K, int I1, int J1, int K1, int I2, int J2, int K2) {
        int b = g.at(I, J, K);
        if (b == 1 || b == 3) return;
        if (b == 2) {
            if (g.at(I1, J1, K1) == 2 && g.at(I2, J2, K2) == 0) cf = 2;
            else if (g.at(I1, J1, K1) == 0 && g.at(I2, J2, K2) == 2) cf = 3;
        }
        setm(I, J, K, cf);
    };
    for (int I = 2; I <= MP; I += 2) {
        for (int K = 3; K <= LP - 1; K += 2) {
            int cf = 1;
            for (int J = 2; J <= NP; J += 2) step(cf, I, J, K, I, J, K + 1, I, J, K - 1);
        }
        for (int J = 3; J <= NP - 1; J += 2) {
            int cf = 1;
            for (int K = 2; K <= LP; ++K) step(cf, I, J, K, I, J + 1, K, I, J - 1, K);
        }
    }
    for (int I = 3; I <= MP - 1; I += 2) {
        int cf = 1;
        for (int K = 2; K <= LP; ++K)
            for (int J = 2; J <= NP; ++J) step(cf, I, J, K, I + 1, J, K, I - 1, J, K);
    }
    // ---- pressure re-reference indices (Gflow.f90:182-242)
    {
        int I = gr->i_ref, J = gr->j_ref, K = gr->k_ref, I1 = I, J1 = J, K1 = K, I2 = I, J2 = J, K2 = K, NX = 0;
        int MPM2 = MP - 2, NPM2 = NP - 2, LPM2 = LP - 2;
        if (I < MPM2 && g.at(I + 2, J, K) == 0) { NX = 1; I1 = I + 2; I2 = g.at(I + 4, J, K) == 0 ? I + 4 : I1; }
        else if (I > 2 && g.at(I - 2, J, K) == 0) { NX = 1; I1 = I - 2; I2 = g.at(I - 4, J, K) == 0 ? I - 4 : I1; }
        else if (J < NPM2 && g.at(I, J + 2, K) == 0) { NX = 2; J1 = J + 2; J2 = (J < NPM2 && g.at(I, J + 4, K) <= 0) ? J + 4 : J1; }
        else if (J > 2 && g.at(I, J - 2, K) <= 0) { NX = 2; J1 = J - 2; J2 = (J > 4 && g.at(I, J - 4, K) <= 0) ? J - 4 : J1; }
        else if (K < LPM2 && g.at(I, J, K + 2) <= 0) { NX = 3; K1 = K + 2; K2 = (K < LPM2 && g.at(I, J, K + 4) <= 0) ? K + 4 : K1; }
        else if (K > 2 && g.at(I, J, K - 2) <= 0) { NX = 3; K1 = K - 2; K2 = (K > 4 && g.at(I, J, K - 4) <= 0) ? K - 4 : K1; }
        extr1(g, h->pref_f1, h->pref_f2, I, J, K, I1, J1, K1, I2, J2, K2, NX);
        h->pref_i1 = I1; h->pref_j1 = J1; h->pref_k1 = K1; h->pref_i2 = I2; h->pref_j2 = J2; h->pref_k2 = K2;
    }
    return GFM_OK;
}

template <typename R>
int setup_ctx(gfm_handle* h, Ctx<R>& c, GeoT<R>& g, AdiScratch<R>* scr, const gfm_grid* gr) {
    const HostGrid& hg = h->hg;
    // geometry in R
    auto up1 = [&](const std::vector<double>& v, const R** out) -> int {
        std::vector<R> t(v.begin(), v.end());
        R* p = nullptr;
        int rc = dupload(h, &p, t);
        *out = p;
        return rc;
    };
    const int8_t* ib_shared = h->gd.ib;
    g = GeoT<R>{};
    g.MP = hg.MP; g.NP = hg.NP; g.LP = hg.LP;
    g.HX = hg.MP / 2 + 1; g.HY = hg.NP / 2 + 1; g.HZ = hg.LP / 2 + 1;
    g.PX = ((g.HX + 15) / 16) * 16;
    g.CB = (long long)g.PX * g.HY * g.HZ;
    g.PXH = ((g.HX + 1) / 2 + 15) / 16 * 16;
    g.CBH = g.PXH * g.HY * g.HZ;
    g.MPM1 = hg.MP - 1; g.MPM2 = hg.MP - 2; g.NPM1 = hg.NP - 1; g.NPM2 = hg.NP - 2; g.LPM1 = hg.LP - 1; g.LPM2 = hg.LP - 2;
    g.NJY1 = 4; g.NJY2 = g.NPM2; g.LKZ1 = 4; g.LKZ2 = g.LPM2;
    g.NJY1V[1] = 4; g.NJY2V[1] = g.NPM2; g.NJY1V[2] = 5; g.NJY2V[2] = hg.NP - 3; g.NJY1V[3] = 4; g.NJY2V[3] = g.NPM2;
    g.LKZ1V[1] = 4; g.LKZ2V[1] = g.LPM2; g.LKZ1V[2] = 4; g.LKZ2V[2] = g.LPM2; g.LKZ1V[3] = 5; g.LKZ2V[3] = hg.LP - 3;
    g.NCELLS = h->ncells;
    for (int q = 0; q < 2; ++q) g.BVF[q] = R(hg.bvf[q]);
    for (int q = 0; q < 6; ++q) g.BAF[q] = R(hg.baf[q]);
    g.HALF = hg.half;
    int rc;
    if ((rc = up1(hg.X, &g.X)) || (rc = up1(hg.DX, &g.DX)) || (rc = up1(hg.R, &g.Rr)) || (rc = up1(hg.DR, &g.DR)) ||
        (rc = up1(hg.RS, &g.RS)) || (rc = up1(hg.Z, &g.Z)) || (rc = up1(hg.DZ, &g.DZ)))
        return rc;
    g.ib = ib_shared;   // shared int8 map
    c.g = g;
    const long long NS = h->NS, CB = h->CB;
    R** full[] = {&c.P, &c.T, &c.DNST, &c.THETA, &c.TMU, &c.GAMA, &c.CRATE, &c.HRATE, &c.GTE, &c.BSH, &c.FZ,
                  &c.APm, &c.BSm, &c.SFPm, &c.UG[0], &c.UG[1], &c.UG[2]};
    for (R** p : full) if ((rc = dalloc(h, p, NS))) return rc;
    for (int l = 0; l < 9; ++l) {
        if (l == 7) { c.GF[l] = nullptr; continue; }
        if ((rc = dalloc(h, &c.GF[l], NS))) return rc;
    }
    for (int q = 0; q < 6; ++q) if ((rc = dalloc(h, &c.ASm[q], NS))) return rc;
    R** cent[] = {&c.APc, &c.BSp, &c.BSq, &c.QA, &c.QE, &c.DPc, &c.BSr};
    for (R** p : cent) if ((rc = dalloc(h, p, CB))) return rc;
    for (int q = 0; q < 6; ++q) if ((rc = dalloc(h, &c.ASc[q], CB))) return rc;
    for (int l = 0; l < 7; ++l) {
        if ((rc = dalloc(h, &c.APs[l], CB)) || (rc = dalloc(h, &c.BSs[l], CB)) || (rc = dalloc(h, &c.FZs[l], CB)) ||
            (rc = dalloc(h, &c.SFPs[l], CB)))
            return rc;
    }
    for (int s = 0; s < 3; ++s)
        for (int q = 0; q < 6; ++q) if ((rc = dalloc(h, &c.ASs[s][q], CB))) return rc;
    for (int e = 0; e < 8; ++e) {
        AdiScratch<R>& w = scr[e];
        if (h->adi_mode == GFM_ADI_MARCH) {
            if ((rc = dalloc(h, &w.xt2, NS)) || (rc = dalloc(h, &w.xt3, NS)) || (rc = dalloc(h, &w.pty, NS)) ||
                (rc = dalloc(h, &w.ptz, NS)))
                return rc;
        } else {
            const long long NH = 2LL * g.CBH;
            R** arrs[] = {&w.xs, &w.x2, &w.x3, &w.sby, &w.sbz, &w.x2b, &w.x3b};
            for (R** a : arrs) if ((rc = dalloc(h, a, NH))) return rc;
            Quad<R>** quads[] = {&w.ya, &w.yb, &w.za, &w.zb};
            for (Quad<R>** a : quads) if ((rc = dalloc(h, a, NH))) return rc;
        }
    }
    if ((rc = dalloc(h, &c.qconv, gr->b_cnt > 0 ? gr->b_cnt : 1))) return rc;
    if ((rc = dalloc(h, &c.ft_buf, (long long)kFtVals * (c.n_extr_ft > 0 ? c.n_extr_ft : 1)))) return rc;
    return GFM_OK;
}

template <typename R>
void fill_ctx_common(gfm_handle* h, Ctx<R>& c, const Ctx<double>& src) {
    c.p = src.p;
    c.rtim = src.rtim; c.delrt = src.delrt; c.delr = src.delr; c.timed = src.timed; c.nr0 = src.nr0;
    c.extr_io = src.extr_io; c.extr_wall = src.extr_wall; c.extr_ft = src.extr_ft;
    c.n_extr_io = src.n_extr_io; c.n_extr_wall = src.n_extr_wall; c.n_extr_ft = src.n_extr_ft;
    c.ft_col_start = src.ft_col_start; c.n_ft_cols = src.n_ft_cols;
    c.extrv = src.extrv;
    for (int d = 0; d < 3; ++d) c.n_extrv[d] = src.n_extrv[d];
    c.patch = src.patch; c.cell_patch_start = src.cell_patch_start; c.cell_patch_list = src.cell_patch_list;
    c.n_patch = src.n_patch; c.n_patch_cells = src.n_patch_cells;
    c.intp_mode = src.intp_mode; c.scal = src.scal; c.partials = src.partials;
    c.nwl = src.nwl;
    for (int l = 0; l < 16; ++l) { c.wl[l] = src.wl[l]; c.akl0[l] = src.akl0[l]; }
    c.i_ref = src.i_ref; c.j_ref = src.j_ref; c.k_ref = src.k_ref; c.p_ref = src.p_ref;
    for (int l = 0; l < 7; ++l) c.as_set[l] = src.as_set[l];
    (void)h;
}

// ---- one GFLOW ------------------------------------------------------------------
template <typename R>
Sys<R> sys_of(R* xt, const R* ap, R* const* as, const R* bs, int ib, int ie, int jb, int je, int kb, int ke, int nim) {
    Sys<R> s;
    s.xt = xt; s.ap = ap;
    for (int q = 0; q < 6; ++q) s.as[q] = as[q];
    s.bs = bs;
    s.ib = ib; s.ie = ie; s.jb = jb; s.je = je; s.kb = kb; s.ke = ke; s.nim = nim;
    return s;
}

template <typename R>
void finish(gfm_handle* h, Ctx<R>& c, std::initializer_list<std::array<int, 3>> items) {
    FinishSpec f{};
    for (auto& it : items) { f.slot[f.n] = it[0]; f.dst[f.n] = it[1]; f.op[f.n] = it[2]; ++f.n; }
    launch_finish(c.partials, c.scal, f, (double)h->ncells, h->stream);
}

// one line-solver batch bracketed by CUDA events (device time of the dominant kernel)
template <typename R>
void adi_call(gfm_handle* h, const GeoT<R>& g, const Sys<R>* sys, AdiScratch<R>* scr, int nsys, cudaStream_t st) {
    // external records: inside a captured graph these become real event nodes
    const int site = h->adi_site++;
    if (h->record_sites) {
        gfm_handle::AdiSite rec{};
        rec.nsys = nsys;
        for (int e = 0; e < nsys; ++e) {
            const int v[7] = {sys[e].ib, sys[e].ie, sys[e].jb, sys[e].je, sys[e].kb, sys[e].ke, sys[e].nim};
            for (int q = 0; q < 7; ++q) rec.rng[e][q] = v[q];
        }
        h->sites.push_back(rec);
    }
    const int flags = site < (int)h->site_flags.size() ? h->site_flags[site] : h->rb_flags;
    if (h->n_ev + 2 <= 16) cudaEventRecordWithFlags(h->ev[h->n_ev], st, cudaEventRecordExternal);
    const int launched = launch_adlbl3_scr(g, sys, scr, nsys, h->adi_mode, st, flags);
    if (h->n_ev + 2 <= 16) { cudaEventRecordWithFlags(h->ev[h->n_ev + 1], st, cudaEventRecordExternal); h->n_ev += 2; }
    int nim = 0;
    for (int e = 0; e < nsys; ++e) {
        nim = sys[e].nim > nim ? sys[e].nim : nim;
        double cells = (double)((sys[e].ie - sys[e].ib) / 2 + 1) * ((sys[e].je - sys[e].jb) / 2 + 1) * ((sys[e].ke - sys[e].kb) / 2 + 1);
        h->adi_cells_visits += cells * 2.0 * sys[e].nim;   // each sweep visits every plane twice
    }
    h->adi_kernels_per_iter += launched;
}

template <typename R>
int gflow_once(gfm_handle* h, Ctx<R>& c, AdiScratch<R>* scr) {
    cudaStream_t st = h->stream;
    const GeoT<R>& g = c.g;
    const gfm_params& P = h->params;
    h->n_ev = 0;
    h->adi_site = 0;
    h->adi_kernels_per_iter = 0;
    h->adi_cells_visits = 0;
    // iteration flags read by the kernels (device scalars, so one captured graph serves every iteration)
    cudaMemcpyAsync(c.scal + S_ITR_GAS, h->h_flags, sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(c.scal + S_RAD_ACTIVE, h->h_flags + 1, sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(c.partials, 0, sizeof(double) * kRedSlots * kRedBlocks, st);
    // wall functions (Gflow.f90:16-130)
    launch_wallfn(c, h->d_wall, h->n_wall, st);
    // GSLV3V: momentum coefficients and pseudo-velocities
    launch_copy_faces_to_fz(c, st);
    launch_mom_assemble(c, st);
    // pressure equation
    launch_p_assemble(c, st);
    Sys<R> sp = sys_of<R>(c.P, c.APc, c.ASc, c.BSp, 4, g.MPM2, g.NJY1, g.NJY2, g.LKZ1, g.LKZ2, P.ntimesg[3]);
    launch_residual(c, sp, SL_P_PRE, st);
    adi_call(h, g, &sp, scr, 1, st);
    launch_residual(c, sp, SL_P_POST, st);
    launch_bound_p(c, st);
    // momentum solves u, v, w (independent systems, one batch)
    launch_mom_prep(c, st);
    Sys<R> sm[3];
    for (int iu = 1; iu <= 3; ++iu) {
        int nx1 = iu == 1;
        sm[iu - 1] = sys_of<R>(c.FZ, c.APm, c.ASm, c.BSm, 4 + nx1, g.MPM2 - nx1, g.NJY1V[iu], g.NJY2V[iu], g.LKZ1V[iu],
                               g.LKZ2V[iu], P.ntimesg[iu - 1]);
        launch_residual(c, sm[iu - 1], SL_U_PRE + iu - 1, st);
    }
    adi_call(h, g, sm, scr, 3, st);
    for (int iu = 0; iu < 3; ++iu) launch_residual(c, sm[iu], SL_U_POST + iu, st);
    launch_mom_finish(c, st);
    // pressure correction
    launch_pcorr_source(c, st);
    if (h->lp) {
        // learned start for p' (FZ on the centres is zero here)
        launch_lp_features(c, h->lp_feats, h->lp_nx, h->lp_ny, h->lp_nz, st);
        h->lp->forward(static_cast<const __nv_bfloat16*>(h->lp_feats), h->lp_nx, h->lp_ny, h->lp_nz, st);
        launch_lp_guess(c, h->lp->OUT, c.FZ, h->lp_nx, h->lp_ny, h->lp_nz, st);
    }
    R* asc[6];
    for (int q = 0; q < 6; ++q) asc[q] = c.ASc[q];
    Sys<R> spc = sys_of<R>(c.FZ, c.APc, asc, c.BSq, 4, g.MPM2, g.NJY1, g.NJY2, g.LKZ1, g.LKZ2, P.ntimesg[4]);
    if (std::is_same<R, float>::value && spc.nim >= 2) {
        // Mixed precision: iterative refinement.  The first half of the sweeps
        // runs on p' itself; the rest runs on the correction system A dp = r
        // with r = b - A p' evaluated in FP64, from dp = 0 (zero on the line
        // ends and on copied rows), and p' += dp.  For a stationary splitting
        // iteration this is the same sequence of iterates in exact arithmetic.
        const int nim = spc.nim, n1 = (nim + 1) / 2;
        spc.nim = n1;
        adi_call(h, g, &spc, scr, 1, st);
        cudaMemsetAsync(c.DPc, 0, sizeof(R) * h->CB, st);
        launch_refine_rhs(g, spc, c.BSr, st);
        Sys<R> sd = sys_of<R>(c.DPc, c.APc, asc, c.BSr, 4, g.MPM2, g.NJY1, g.NJY2, g.LKZ1, g.LKZ2, nim - n1);
        adi_call(h, g, &sd, scr, 1, st);
        launch_refine_add(g, spc, c.DPc, st);
        spc.nim = nim;
    } else {
        adi_call(h, g, &spc, scr, 1, st);
    }
    launch_residual(c, spc, SL_PC_POST, st);
    launch_velcorr(c, st);
    // exit balance (EXTRV, FLX1D, FACTOR), INTPV
    launch_extrv(c, 0, st);
    finish(h, c, {{SL_GFEX, S_GFEX, 0}, {SL_TM, S_TMEAN_EX, 0}, {SL_TAREA, S_TAREA_MEAN, 0}, {SL_AREA, S_AREA_EX, 0}});
    launch_factor(c, st);
    launch_extrv(c, 1, st);
    launch_intpv(c, st);
    // pressure re-reference
    launch_pref_idx(c, h->pref_i1, h->pref_j1, h->pref_k1, h->pref_i2, h->pref_j2, h->pref_k2, h->pref_f1, h->pref_f2, st);
    // GSLV3G: scalar equations
    if (P.wall_sink) launch_qconv(c, st);
    launch_scalar_sources_first(c, st);
    const int order[6] = {1, 2, 3, 4, 6, 7};
    bool made[3] = {false, false, false};
    Sys<R> ss[6];
    for (int q = 0; q < 6; ++q) {
        int L = order[q];
        int set = c.as_set[L - 1];
        launch_scalar_assemble(c, L, !made[set], st);
        made[set] = true;
        const int nelg = L == 1 ? 6 : L == 6 ? 7 : L == 3 ? 8 : L == 4 ? 9 : L == 5 ? 10 : L == 7 ? 11 : 12;
        ss[q] = sys_of<R>(c.FZs[L - 1], c.APs[L - 1], c.ASs[set], c.BSs[L - 1], 4, g.MPM2, g.NJY1, g.NJY2, g.LKZ1, g.LKZ2,
                          P.ntimesg[nelg - 1]);
        launch_residual(c, ss[q], SL_GF_PRE + L - 1, st);
    }
    adi_call(h, g, ss, scr, 6, st);
    for (int q = 0; q < 6; ++q) {
        int L = order[q];
        launch_residual(c, ss[q], SL_GF_POST + L - 1, st);
        launch_scalar_finish(c, L, st);
    }
    {
        const int L = 5;
        int set = c.as_set[L - 1];
        launch_scalar_assemble(c, L, !made[set], st);
        Sys<R> se = sys_of<R>(c.FZs[L - 1], c.APs[L - 1], c.ASs[set], c.BSs[L - 1], 4, g.MPM2, g.NJY1, g.NJY2, g.LKZ1, g.LKZ2,
                              P.ntimesg[9]);
        launch_residual(c, se, SL_GF_PRE + L - 1, st);
        adi_call(h, g, &se, scr, 1, st);
        launch_residual(c, se, SL_GF_POST + L - 1, st);
        launch_scalar_finish(c, L, st);
    }
    // properties, mean temperature, boundary values, interpolation
    launch_props(c, st);
    launch_tave(c, st);
    launch_extr(c, st);
    launch_intp(c, st);
    finish(h, c, {{SL_RESM, S_RES_MASS, 3}, {SL_RESMAX, S_RES_MASS_MAX, 1}, {SL_QCONV, S_QCONV, 0},
                  {SL_QREACT, S_Q_REACT, 0}, {SL_TA, S_TAVE, 0}, {SL_TB, S_TAVE_DEN, 0},
                  {SL_GFIN0, S_GFIN0, 0}, {SL_QEX, S_Q_EXHAUST, 0}});
    FinishSpec f{};
    auto add = [&](int slot, int dst, int op) { f.slot[f.n] = slot; f.dst[f.n] = dst; f.op[f.n] = op; ++f.n; };
    add(SL_P_PRE, S_P_RESID_PRE, 2); add(SL_P_POST, S_P_RESID, 2); add(SL_PC_POST, S_PCORR_RESID, 2);
    for (int i = 0; i < 3; ++i) { add(SL_U_PRE + i, S_U_RESID_PRE + i, 2); add(SL_U_POST + i, S_U_RESID + i, 2); }
    for (int l = 0; l < 7; ++l) { add(SL_GF_PRE + l, S_GF_RESID_PRE + l, 2); add(SL_GF_POST + l, S_GF_RESID + l, 2); }
    launch_finish(c.partials, c.scal, f, (double)h->ncells, st);
    return GFM_OK;
}

template <typename R>
int initsv_dev(gfm_handle* h, Ctx<R>& c) {
    cudaStream_t st = h->stream;
    cudaMemsetAsync(c.partials, 0, sizeof(double) * kRedSlots * kRedBlocks, st);
    launch_intpv(c, st);
    launch_extr(c, st);
    launch_intp(c, st);
    finish(h, c, {{SL_GFIN0, S_GFIN0, 0}, {SL_QEX, S_Q_EXHAUST, 0}});
    return GFM_OK;
}

// staging slots, copy stream and events of the whole-state transfers
int xfer_prepare(gfm_handle* h) {
    if (h->d_stage_all) return GFM_OK;
    int rc;
    if ((rc = dalloc(h, &h->d_stage_all, (long long)kXferSlots * h->N)) || (rc = dalloc(h, &h->d_bad_all, kXferSlots)))
        return rc;
    for (int s = 0; s < kXferStreams; ++s) CK(cudaStreamCreateWithFlags(&h->copy_stream[s], cudaStreamNonBlocking));
    for (int i = 0; i <= kXferSlots; ++i) CK(cudaEventCreateWithFlags(&h->ev_xfer[i], cudaEventDisableTiming));
    return GFM_OK;
}

// One field of a whole-state transfer: host array, device array, element
// count (N for the doubled-layout fields, the cell count for QA/QE).
template <typename R>
struct XferItem {
    double* host;
    R* dev;
    bool cells;
    const char* name;
};

template <typename R>
int xfer_items(gfm_handle* h, Ctx<R>& c, const gfm_fields* f, std::vector<XferItem<R>>& it) {
    const long long N = h->N;
    auto add = [&](double* host, R* dev, bool cells, const char* name) { if (host) it.push_back({host, dev, cells, name}); };
    add(f->p, c.P, false, "p"); add(f->t, c.T, false, "t"); add(f->dnst, c.DNST, false, "dnst");
    add(f->theta, c.THETA, false, "theta"); add(f->tmu, c.TMU, false, "tmu"); add(f->gama, c.GAMA, false, "gama");
    add(f->crate, c.CRATE, false, "crate"); add(f->hrate, c.HRATE, false, "hrate"); add(f->bs_hprev, c.BSH, false, "bs_hprev");
    for (int l = 0; l < 3; ++l) add(f->ug ? f->ug + l * N : nullptr, c.UG[l], false, "ug");
    for (int l = 0; l < 9; ++l) if (l != 7) add(f->gf ? f->gf + l * N : nullptr, c.GF[l], false, "gf");
    add(f->qa, c.QA, true, "qa");
    add(f->qe, c.QE, true, "qe");
    return (int)it.size() <= kXferSlots ? GFM_OK : GFM_E_ARG;
}

// Host -> device: every field's copy is queued on the copy stream into its own
// staging slot; the compute stream waits for each copy, counts its non-finite
// values and converts it to the device layout while later copies run.
template <typename R>
int upload_fields(gfm_handle* h, Ctx<R>& c, const gfm_fields* f) {
    const long long N = h->N;
    const GeoT<R>& g = c.g;
    cudaStream_t st = h->stream;
    int rc;
    if ((rc = xfer_prepare(h))) return rc;
    std::vector<XferItem<R>> it;
    if ((rc = xfer_items(h, c, f, it))) return rc;
    const long long ncell = (long long)(h->hg.MP / 2) * (h->hg.NP / 2) * (h->hg.LP / 2);
    CK(cudaMemsetAsync(h->d_bad_all, 0, kXferSlots * sizeof(unsigned int), st));
    // the staging slots may still be read by earlier work on the compute stream
    CK(cudaEventRecord(h->ev_xfer[kXferSlots], st));
    for (int s = 0; s < kXferStreams; ++s) CK(cudaStreamWaitEvent(h->copy_stream[s], h->ev_xfer[kXferSlots], 0));
    for (size_t i = 0; i < it.size(); ++i) {
        double* slot = h->d_stage_all + (long long)i * N;
        const long long n = it[i].cells ? ncell : N;
        cudaStream_t cs = h->copy_stream[i % kXferStreams];
        CK(cudaMemcpyAsync(slot, it[i].host, n * sizeof(double), cudaMemcpyHostToDevice, cs));
        CK(cudaEventRecord(h->ev_xfer[i], cs));
        CK(cudaStreamWaitEvent(st, h->ev_xfer[i], 0));
        if (it[i].cells) launch_cells_to_split(g, slot, it[i].dev, st);
        else launch_to_split_count(g, slot, it[i].dev, h->d_bad_all + i, st);
    }
    unsigned int nb[kXferSlots] = {};
    CK(cudaMemcpyAsync(nb, h->d_bad_all, kXferSlots * sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (size_t i = 0; i < it.size(); ++i)
        if (nb[i]) { h->err = std::string("non-finite values in uploaded array ") + it[i].name; return GFM_E_NAN; }
    return GFM_OK;
}

// Device -> host: the compute stream converts every field into its staging
// slot; the copy stream sends each slot to the host as soon as it is ready.
template <typename R>
int download_fields(gfm_handle* h, Ctx<R>& c, gfm_fields* f) {
    const long long N = h->N;
    const GeoT<R>& g = c.g;
    cudaStream_t st = h->stream;
    int rc;
    if ((rc = xfer_prepare(h))) return rc;
    std::vector<XferItem<R>> it;
    if ((rc = xfer_items(h, c, f, it))) return rc;
    const long long ncell = (long long)(h->hg.MP / 2) * (h->hg.NP / 2) * (h->hg.LP / 2);
    for (size_t i = 0; i < it.size(); ++i) {
        double* slot = h->d_stage_all + (long long)i * N;
        if (it[i].cells) launch_cells_from_split(g, it[i].dev, slot, st);
        else launch_from_split(g, it[i].dev, slot, st);
        cudaStream_t cs = h->copy_stream[i % kXferStreams];
        CK(cudaEventRecord(h->ev_xfer[i], st));
        CK(cudaStreamWaitEvent(cs, h->ev_xfer[i], 0));
        CK(cudaMemcpyAsync(it[i].host, slot, (it[i].cells ? ncell : N) * sizeof(double), cudaMemcpyDeviceToHost, cs));
    }
    for (int s = 0; s < kXferStreams; ++s) CK(cudaStreamSynchronize(h->copy_stream[s]));
    CK(cudaStreamSynchronize(st));
    if (f->gf) std::memset(f->gf + 7 * N, 0, N * sizeof(double));   // GF(..,8) is not a field of this path
    f->itr_gas = h->itr_gas;
    f->do_rad_qe_only_cnt = h->cnt_qe;
    f->i1st_rad_qe_done = h->rad_active;
    f->factor = h->h_scal[S_FACTOR];
    f->fadj = h->h_scal[S_FADJ];
    f->gfin0 = h->h_scal[S_GFIN0];
    f->q_h_in = h->q_h_in;
    return GFM_OK;
}

void fill_stats(gfm_handle* h, gfm_iter_stats* s, int converged) {
    if (!s) return;
    const double* v = h->h_scal;
    std::memset(s, 0, sizeof *s);
    s->itr_gas = h->itr_gas;
    s->converged = converged;
    s->res_mass = v[S_RES_MASS]; s->res_mass_max = v[S_RES_MASS_MAX];
    s->p_resid_pre = v[S_P_RESID_PRE]; s->p_resid = v[S_P_RESID]; s->pcorr_resid = v[S_PCORR_RESID];
    for (int i = 0; i < 3; ++i) { s->u_resid_pre[i] = v[S_U_RESID_PRE + i]; s->u_resid[i] = v[S_U_RESID + i]; }
    for (int i = 0; i < 7; ++i) { s->gf_resid_pre[i] = v[S_GF_RESID_PRE + i]; s->gf_resid[i] = v[S_GF_RESID + i]; }
    s->factor = v[S_FACTOR]; s->gfin = v[S_GFIN]; s->gfex = v[S_GFEX];
    s->q_react = v[S_Q_REACT]; s->q_exhaust = v[S_Q_EXHAUST]; s->q_conv_total = v[S_QCONV];
    double q_in_tot = v[S_Q_REACT] + h->q_h_in, q_out_tot = v[S_Q_EXHAUST];
    s->q_global_bal = std::fabs((q_in_tot - q_out_tot) / q_in_tot);
    double tb = v[S_TAVE_DEN];
    s->tave = tb != 0.0 ? v[S_TAVE] * h->params.t0 / tb : 0.0;
    s->tmean_ex = v[S_TMEAN_EX];
    s->lp_used = h->lp ? (int)v[S_LP_USED] : 0;
    s->lp_ratio = h->lp ? v[S_LP_RATIO] : 0.0;
}

}  // namespace

// =============================================================================
// C ABI
// =============================================================================
extern "C" int gfm_gpu_device_count(void) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n < 1) return GFM_E_NODEVICE;
    return n;
}

namespace {
thread_local std::string g_create_err;
int create_impl(const gfm_grid* gr, const gfm_params* prm, gfm_handle** out);
}

extern "C" int gfm_gpu_create(const gfm_grid* gr, const gfm_params* prm, gfm_handle** out) {
    if (!out) return GFM_E_ARG;
    *out = nullptr;
    gfm_handle* h = nullptr;
    int rc = create_impl(gr, prm, &h);
    if (rc != GFM_OK) {
        g_create_err = h ? h->err : std::string("invalid arguments or no CUDA device");
        if (h) gfm_gpu_destroy(h);
        return rc;
    }
    *out = h;
    return GFM_OK;
}

namespace {
int create_impl(const gfm_grid* gr, const gfm_params* prm, gfm_handle** out) {
    if (!gr || !prm || !out) return GFM_E_ARG;
    *out = nullptr;
    if (gr->mp < 8 || gr->np < 8 || gr->lp < 8 || (gr->mp & 1) || (gr->np & 1) || (gr->lp & 1)) return GFM_E_ARG;
    if (gr->nwl < 1 || gr->nwl > 16 || gr->nr0 < 2) return GFM_E_ARG;
    if (prm->precision != GFM_PREC_FP64 && prm->precision != GFM_PREC_MIXED) return GFM_E_ARG;
    if (prm->adi_mode != GFM_ADI_MARCH && prm->adi_mode != GFM_ADI_REDBLACK) return GFM_E_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return GFM_E_NODEVICE;
    gfm_handle* h = new (std::nothrow) gfm_handle();
    if (!h) return GFM_E_NOMEM;
    *out = h;
    h->prec = prm->precision;
    h->adi_mode = prm->adi_mode;
    h->params = *prm;
    HostGrid& hg = h->hg;
    hg.MP = gr->mp; hg.NP = gr->np; hg.LP = gr->lp;
    h->N = (long long)hg.MP * hg.NP * hg.LP;
    hg.ib.assign(gr->ibcell, gr->ibcell + h->N);
    // half-blocked cells carry IBCELL -1 or -2, the two entries of BV_F and
    // BA_F (Grid3.f90:12); lower values would index past them
    hg.half = 0;
    for (long long i = 0; i < h->N; ++i) {
        if (hg.ib[i] < -2 || hg.ib[i] > 20) { h->err = "IBCELL outside -2..20"; return GFM_E_UNSUPPORTED; }
        if (hg.ib[i] < 0) hg.half = 1;
    }
    for (int q = 0; q < 2; ++q) hg.bvf[q] = gr->bv_f[q];
    for (int q = 0; q < 6; ++q) hg.baf[q] = gr->ba_f[q];
    for (int q = 0; q < 8; ++q) {
        const double v = q < 2 ? hg.bvf[q] : hg.baf[q - 2];
        if (!(v > 0.0 && v < 1.0e30)) { h->err = "half-block factors BV_F, BA_F must be positive"; return GFM_E_ARG; }
    }
    auto one_based = [](const double* s, int n) { std::vector<double> v(n + 3, 0.0); for (int i = 0; i < n; ++i) v[i + 1] = s[i]; return v; };
    hg.X = one_based(gr->x, hg.MP); hg.DX = one_based(gr->dx, hg.MP);
    hg.R = one_based(gr->r, hg.NP); hg.DR = one_based(gr->dr, hg.NP); hg.RS = one_based(gr->rs, hg.NP);
    hg.Z = one_based(gr->z, hg.LP); hg.DZ = one_based(gr->dz, hg.LP);
    h->ncells = gr->ncells;
    cudaError_t ce = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) { h->err = cudaGetErrorString(ce); return GFM_E_CUDA; }
    if (prepare_line_solver() != GFM_OK) { h->err = "cannot raise the line solver's shared-memory limit"; return GFM_E_CUDA; }
    if (prepare_rif_table() != GFM_OK) { h->err = "cannot load the emission update's RIF3 table"; return GFM_E_CUDA; }
    {
        const char* tn = std::getenv("GFM_RB_TUNE");
        h->tune = !(tn && tn[0] == '0');
        const char* pl = std::getenv("GFM_RB_PLANE");
        const char* pd = std::getenv("GFM_PDL");
        const char* ap = std::getenv("GFM_RB_AVG_IN_PASS");
        h->rb_flags = (pl && pl[0] == '0' ? 0 : kRbPlane) | (pd && pd[0] == '0' ? 0 : kRbPdl) |
                      (ap && ap[0] == '0' ? 0 : kRbAvgInPass);
    }
    cudaEventCreate(&h->ev_adi0);
    cudaEventCreate(&h->ev_adi1);
    // double geometry first: its int8 map is shared by the float copy
    GeoT<double>& g = h->gd;
    g.MP = hg.MP; g.NP = hg.NP; g.LP = hg.LP;
    for (int q = 0; q < 2; ++q) g.BVF[q] = hg.bvf[q];
    for (int q = 0; q < 6; ++q) g.BAF[q] = hg.baf[q];
    g.HALF = hg.half;
    g.HX = hg.MP / 2 + 1; g.HY = hg.NP / 2 + 1; g.HZ = hg.LP / 2 + 1;
    g.PX = ((g.HX + 15) / 16) * 16;
    g.CB = (long long)g.PX * g.HY * g.HZ;
    g.PXH = ((g.HX + 1) / 2 + 15) / 16 * 16;
    g.CBH = g.PXH * g.HY * g.HZ;
    h->CB = g.CB;
    h->NS = 8 * g.CB;
    if (h->NS >= (1LL << 31) || 2LL * ((g.HX + 1) / 2 + 16) * g.HY * g.HZ >= (1LL << 31)) {
        h->err = "grid too large for 32-bit field offsets";
        return GFM_E_UNSUPPORTED;
    }
    if (g.HY > 256 || g.HZ > 256) { h->err = "line solver: more than 256 points on a y- or z-line"; return GFM_E_UNSUPPORTED; }
    {
        std::vector<int8_t> ibs((size_t)h->NS, 1);
        for (int K = 1; K <= hg.LP; ++K)
            for (int J = 1; J <= hg.NP; ++J)
                for (int I = 1; I <= hg.MP; ++I) ibs[(size_t)pidx(g, I, J, K)] = (int8_t)hg.at(I, J, K);
        int8_t* d = nullptr;
        int rc = dupload(h, &d, ibs);
        if (rc) return rc;
        g.ib = d;
    }
    std::vector<int> wall_list, ft_start, cp_start, cp_list;
    std::vector<ExtrRec> io, walls, ft;
    std::vector<ExtrvRec> ev;
    std::vector<Patch> patches;
    std::vector<int8_t> intp_mode;
    int nev[3] = {0, 0, 0};
    int rc = build_tables(h, gr, wall_list, io, walls, ft, ft_start, ev, nev, patches, cp_start, cp_list, intp_mode);
    if (rc) return rc;
    Ctx<double>& c = h->cd;
    // tables shared by both precisions (kept in the double context)
    std::vector<double> rt(gr->rtim, gr->rtim + gr->nr0), dr(gr->delrt, gr->delrt + gr->nr0),
        dl(gr->delr, gr->delr + gr->nr0), tm(gr->timed, gr->timed + gr->nr0);
    double *p1, *p2, *p3, *p4;
    if ((rc = dupload(h, &p1, rt)) || (rc = dupload(h, &p2, dr)) || (rc = dupload(h, &p3, dl)) || (rc = dupload(h, &p4, tm))) return rc;
    c.rtim = p1; c.delrt = p2; c.delr = p3; c.timed = p4; c.nr0 = gr->nr0;
    ExtrRec *e1, *e2, *e3;
    ExtrvRec* e4;
    Patch* pp;
    int *i1, *i2, *i3;
    int8_t* im;
    if ((rc = dupload(h, &e1, io)) || (rc = dupload(h, &e2, walls)) || (rc = dupload(h, &e3, ft)) || (rc = dupload(h, &e4, ev)) ||
        (rc = dupload(h, &pp, patches)) || (rc = dupload(h, &i1, ft_start)) || (rc = dupload(h, &i2, cp_start)) ||
        (rc = dupload(h, &i3, cp_list)) || (rc = dupload(h, &im, intp_mode)) || (rc = dupload(h, &h->d_wall, wall_list)))
        return rc;
    h->n_wall = (int)wall_list.size() / 3;
    c.extr_io = e1; c.extr_wall = e2; c.extr_ft = e3; c.n_extr_io = (int)io.size(); c.n_extr_wall = (int)walls.size();
    c.n_extr_ft = (int)ft.size(); c.ft_col_start = i1; c.n_ft_cols = (int)ft_start.size() - 1;
    c.extrv = e4;
    for (int d = 0; d < 3; ++d) c.n_extrv[d] = nev[d];
    c.patch = pp; c.cell_patch_start = i2; c.cell_patch_list = i3; c.n_patch = (int)patches.size();
    h->d_patches = pp;
    h->bp_typ.assign(gr->b_typ, gr->b_typ + gr->b_cnt); h->bp_i.assign(gr->b_i, gr->b_i + gr->b_cnt);
    h->bp_j.assign(gr->b_j, gr->b_j + gr->b_cnt); h->bp_k.assign(gr->b_k, gr->b_k + gr->b_cnt);
    h->bp_ori.assign(gr->b_orient, gr->b_orient + gr->b_cnt); h->bp_dir.assign(gr->b_direct, gr->b_direct + gr->b_cnt);
    c.intp_mode = im;
    if ((rc = dalloc(h, &c.scal, S_NUM + 128)) || (rc = dalloc(h, &c.partials, (long long)kRedSlots * kRedBlocks)) ||
        (rc = dalloc(h, &h->d_stage, h->N)) || (rc = dalloc(h, &h->d_bad, 1)))
        return rc;
    {
        Nist* dn = nullptr;
        std::vector<Nist> v(1, nist_host());
        if ((rc = dupload(h, &dn, v))) return rc;
        c.nist = dn;
    }
    if (cudaMallocHost(&h->h_scal, sizeof(double) * (S_NUM + 128)) != cudaSuccess) return GFM_E_NOMEM;
    if (cudaMallocHost(&h->h_flags, sizeof(double) * 4) != cudaSuccess) return GFM_E_NOMEM;
    for (int q = 0; q < 16; ++q) cudaEventCreate(&h->ev[q]);
    cudaEventCreate(&h->ev_g0);
    cudaEventCreate(&h->ev_g1);
    {
        const char* ng = std::getenv("GFM_NO_GRAPH");
        h->use_graph = !(ng && ng[0] == '1');
    }
    std::memset(h->h_scal, 0, sizeof(double) * (S_NUM + 128));
    // constants
    Prm& p = c.p;
    p.t0 = prm->t0; p.h_0 = prm->h_0; p.dnst0 = prm->dnst0; p.ug0 = prm->ug0; p.gmfr = prm->gmfr; p.pg0 = prm->pg0; p.r0 = prm->r0;
    p.reyg = prm->reyg; p.reyg2 = prm->reyg2; p.epsr = prm->epsr; p.taur = prm->taur; p.eun = prm->eun; p.qr0 = prm->qr0;
    p.q0 = prm->q0; p.tk0 = prm->tk0;
    for (int i = 0; i < 3; ++i) p.gra[i] = prm->gra[i];
    p.amu = prm->amu; p.trdg = prm->trdg; p.wt0 = prm->wt0; p.stoich = prm->stoich;
    p.cmu = prm->cmu; p.ct1 = prm->ct1; p.ct2 = prm->ct2;
    p.p_mx = prm->p_mx; p.p_mn = prm->p_mn; p.t_mx = prm->t_mx; p.t_mn = prm->t_mn; p.u_mx = prm->u_mx; p.u_mn = prm->u_mn;
    p.f_mx = prm->f_mx; p.f_mn = prm->f_mn;
    for (int i = 0; i < 21; ++i) { p.rf[i] = prm->rf[i]; p.rfc[i] = 1.0 - prm->rf[i]; p.rfl[i] = prm->rfl[i]; p.rflc[i] = 1.0 - prm->rfl[i]; }
    for (int i = 0; i < 12; ++i) p.sigma[i] = prm->sigma[i];
    p.rf_hsource = prm->rf_hsource; p.h_g = prm->h_g;
    p.sig = prm->sig; p.ri = prm->ri; p.hck = prm->hck;
    p.rt20 = p.reyg2 * std::sqrt(p.epsr) * std::pow(p.cmu, 0.25);
    p.cbl0 = 2.5 * std::sqrt(p.epsr) / p.taur * std::pow(p.cmu, 0.75);
    p.react = prm->react; p.wall_sink = prm->wall_sink;
    c.nwl = gr->nwl;
    for (int l = 0; l < gr->nwl; ++l) { c.wl[l] = gr->wl[l]; c.akl0[l] = gr->akl0[l]; }
    c.i_ref = gr->i_ref; c.j_ref = gr->j_ref; c.k_ref = gr->k_ref; c.p_ref = gr->p_ref;
    // coefficient sets by sigma: equations with equal sigma share one set
    {
        double sv[3];
        int ns = 0;
        for (int L = 1; L <= 7; ++L) {
            int s = -1;
            for (int q = 0; q < ns; ++q) if (sv[q] == prm->sigma[L - 1]) s = q;
            if (s < 0) { if (ns == 3) { h->err = "more than three distinct sigma values"; return GFM_E_UNSUPPORTED; } sv[ns] = prm->sigma[L - 1]; s = ns++; }
            c.as_set[L - 1] = s;
        }
    }
    if (h->prec == GFM_PREC_FP64) {
        if ((rc = setup_ctx<double>(h, c, h->gd, h->scr_d, gr))) return rc;
    } else {
        fill_ctx_common(h, h->cf, c);
        NistT<float>* dnf = nullptr;
        std::vector<NistT<float>> vf(1, nist_cast<float>(nist_host()));
        if ((rc = dupload(h, &dnf, vf))) return rc;
        h->cf.nist = dnf;
        h->gfl.ib = g.ib;
        if ((rc = setup_ctx<float>(h, h->cf, h->gfl, h->scr_f, gr))) return rc;
    }
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return GFM_E_CUDA; }
    return GFM_OK;
}
}  // namespace

extern "C" int gfm_gpu_upload(gfm_handle* h, const gfm_fields* f) {
    if (!h || !f) return GFM_E_ARG;
    h->itr_gas = f->itr_gas;
    h->cnt_qe = f->do_rad_qe_only_cnt;
    h->rad_active = f->i1st_rad_qe_done;
    h->q_h_in = f->q_h_in;
    h->h_scal[S_FACTOR] = f->factor;
    h->h_scal[S_FADJ] = f->fadj;
    h->h_scal[S_GFIN0] = f->gfin0;
    double* scal = h->prec == GFM_PREC_FP64 ? h->cd.scal : h->cf.scal;
    cudaError_t e = cudaMemcpy(scal, h->h_scal, sizeof(double) * (S_NUM + 128), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return GFM_E_CUDA; }
    return h->prec == GFM_PREC_FP64 ? upload_fields(h, h->cd, f) : upload_fields(h, h->cf, f);
}

extern "C" int gfm_gpu_initsv(gfm_handle* h) {
    if (!h) return GFM_E_ARG;
    int rc = h->prec == GFM_PREC_FP64 ? initsv_dev(h, h->cd) : initsv_dev(h, h->cf);
    if (rc) return rc;
    double* scal = h->prec == GFM_PREC_FP64 ? h->cd.scal : h->cf.scal;
    cudaError_t e = cudaMemcpyAsync(h->h_scal, scal, sizeof(double) * (S_NUM + 128), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return GFM_E_CUDA; }
    return GFM_OK;
}

namespace {
int capture_iteration(gfm_handle* h) {
    if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; }
    if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
    cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) { h->err = std::string("capture: ") + cudaGetErrorString(e); return GFM_E_CUDA; }
    int rc = h->prec == GFM_PREC_FP64 ? gflow_once(h, h->cd, h->scr_d) : gflow_once(h, h->cf, h->scr_f);
    e = cudaStreamEndCapture(h->stream, &h->graph);
    if (rc) return rc;
    if (e != cudaSuccess) { h->err = std::string("capture end: ") + cudaGetErrorString(e); return GFM_E_CUDA; }
    size_t n = 0;
    cudaGraphGetNodes(h->graph, nullptr, &n);
    std::vector<cudaGraphNode_t> nodes(n);
    cudaGraphGetNodes(h->graph, nodes.data(), &n);
    long long k = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        cudaGraphNodeGetType(nd, &t);
        if (t == cudaGraphNodeTypeKernel) ++k;
    }
    h->kernels_per_iter = k;
    e = cudaGraphInstantiate(&h->graph_exec, h->graph, 0);
    if (e != cudaSuccess) { h->err = std::string("instantiate: ") + cudaGetErrorString(e); return GFM_E_CUDA; }
    return GFM_OK;
}
}  // namespace

namespace {
int gas_band(gfm_handle* h);
int gas_check(gfm_handle* h);
int minor_initsvm(gfm_handle* h, int restart);
int msflow_run(gfm_handle* h, int maxms, gfm_msflow_stats* out);
// the emission-only source (rad_qe_only, Rad_emis.f90:411-466) on the
// handle's stream, on the band model's coefficients when the case asks for it
int rad_emission_launch(gfm_handle* h) {
    if (h->params.gas_model) {
        if (h->gas.err) CK(cudaMemsetAsync(h->gas.err, 0, sizeof(int), h->stream));
        int rc = gas_band(h);
        if (rc) return rc;
    }
    const double* ag = h->params.gas_model ? h->gas.aklg : nullptr;
    const double* as = h->params.gas_model ? h->gas.akls : nullptr;
    if (h->prec == GFM_PREC_FP64) launch_rad_emission(h->cd, h->stream, ag, as);
    else launch_rad_emission(h->cf, h->stream, ag, as);
    return GFM_OK;
}

// One SPHASE pass split in two, so that several handles can have an
// iteration in flight at once: iter_launch queues GFLOW and the read-back of
// the statistics on the handle's stream; iter_finish waits for them and
// applies the convergence test and the emission cadence (Sphase.f90:37-235).
int iter_launch(gfm_handle* h) {
    h->itr_gas += 1;
    h->as_minor_current = false;   // GSLV3G leaves the last gas equation's coefficients
    h->h_flags[0] = (double)h->itr_gas;
    h->h_flags[1] = (double)h->rad_active;
    if (h->use_graph) {
        cudaError_t e = cudaGraphLaunch(h->graph_exec, h->stream);
        if (e != cudaSuccess) { h->err = std::string("graph launch: ") + cudaGetErrorString(e); return GFM_E_CUDA; }
        h->launches += h->kernels_per_iter;
    } else {
        int rc = h->prec == GFM_PREC_FP64 ? gflow_once(h, h->cd, h->scr_d) : gflow_once(h, h->cf, h->scr_f);
        if (rc) return rc;
    }
    double* scal = h->prec == GFM_PREC_FP64 ? h->cd.scal : h->cf.scal;
    cudaError_t e = cudaMemcpyAsync(h->h_scal, scal, sizeof(double) * (S_NUM + 128), cudaMemcpyDeviceToHost, h->stream);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return GFM_E_CUDA; }
    return GFM_OK;
}
// *conv = 1 when res_mass < BGCON
int iter_finish(gfm_handle* h, int* conv) {
    *conv = 0;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return GFM_E_CUDA; }
    if (int rc = gas_check(h)) return rc;   // the band model of the last emission update
    for (int q = 0; q + 1 < h->n_ev; q += 2) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, h->ev[q], h->ev[q + 1]) == cudaSuccess) h->adi_ms += ms;
    }
    if (!std::isfinite(h->h_scal[S_RES_MASS])) { h->err = "res_mass is not finite"; return GFM_E_NAN; }
    if (h->h_scal[S_RES_MASS] < h->params.bgcon) { *conv = 1; return GFM_OK; }
    if (h->params.rad_emission) {
        h->cnt_qe += 1;
        if (h->cnt_qe >= h->params.rad_qe_frequency && h->itr_gas > 50) {
            int rc;
            if (h->params.gas_model && !h->rad_active) {
                // the first emission update runs INITSVM and MSFLOW(300) before it (Sphase.f90:210-224)
                if ((rc = minor_initsvm(h, h->params.irstypm != 0 && h->minor_from_host)) || (rc = msflow_run(h, 300, nullptr)))
                    return rc;
            }
            rc = rad_emission_launch(h);
            if (rc) return rc;
            h->rad_active = 1;
            h->cnt_qe = 0;
        }
    }
    return GFM_OK;
}
__global__ void k_tune_fill(float* p, long long n, float v) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = v;
}
__global__ void k_tune_fill(double* p, long long n, double v) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = v;
}

// Times every call site of the iteration in the three red-black forms --
// segmented colour passes, plane visits (small planes on 256-thread CTAs),
// plane visits on 768-thread CTAs only -- on stand-in systems with the
// site's ranges and sweep counts (diagonally dominant, AP = 1, AS = 0.1,
// BS = 0.1), three timed calls after one untimed, and keeps the fastest
// form's flags for the site.  The stand-in arrays live only for the tuning.
// Choices already made in this process, by call shape (precision, systems,
// ranges, sweeps): a shape is timed once, so every handle of the process
// that meets it runs the same form and gives the same bits.
std::mutex g_tune_mu;
std::map<std::vector<int>, std::pair<int, std::array<float, 3>>> g_tune_cache;

template <typename R>
int tune_sites(gfm_handle* h, Ctx<R>& c, AdiScratch<R>* scr) {
    const GeoT<R>& g = c.g;
    cudaStream_t st = h->stream;
    int max_sys = 1;
    for (const auto& s : h->sites) max_sys = std::max(max_sys, s.nsys);
    const long long NS = 8LL * g.CB;
    const int narr = 8 + max_sys;   // AP, AS x6, BS shared; one XT per system
    R* pool = nullptr;
    if (cudaMalloc(&pool, sizeof(R) * NS * narr) != cudaSuccess) {
        cudaGetLastError();
        return GFM_OK;   // no room to tune: the default forms stay
    }
    R* ap = pool;
    R* as6[6];
    for (int q = 0; q < 6; ++q) as6[q] = pool + NS * (1 + q);
    R* bs = pool + NS * 7;
    k_tune_fill<<<1024, 256, 0, st>>>(ap, NS, R(1));
    k_tune_fill<<<1024, 256, 0, st>>>(as6[0], 6 * NS, R(0.1));
    k_tune_fill<<<1024, 256, 0, st>>>(bs, NS, R(0.1));
    k_tune_fill<<<1024, 256, 0, st>>>(pool + NS * 8, NS * max_sys, R(0));
    const int forms[3] = {h->rb_flags & ~kRbPlane, h->rb_flags | kRbPlane | kRbSmallF64,
                          h->rb_flags | kRbPlane | kRbNoSmall};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    h->site_flags.assign(h->sites.size(), h->rb_flags);
    h->site_ms.assign(h->sites.size(), {0.f, 0.f, 0.f});
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (size_t k = 0; k < h->sites.size(); ++k) {
        const auto& site = h->sites[k];
        std::vector<int> key = {(int)sizeof(R), h->rb_flags, site.nsys};
        for (int e = 0; e < site.nsys; ++e) key.insert(key.end(), site.rng[e], site.rng[e] + 7);
        const auto hit = g_tune_cache.find(key);
        if (hit != g_tune_cache.end()) {
            h->site_flags[k] = hit->second.first;
            h->site_ms[k] = hit->second.second;
            continue;
        }
        Sys<R> sys[8];
        for (int e = 0; e < site.nsys; ++e) {
            const int* r = site.rng[e];
            sys[e] = sys_of<R>(pool + NS * (8 + e), ap, as6, bs, r[0], r[1], r[2], r[3], r[4], r[5], r[6]);
        }
        float best = 0.f;
        for (int f = 0; f < 3; ++f) {
            launch_adlbl3_scr(g, sys, scr, site.nsys, h->adi_mode, st, forms[f]);
            float ms = 1e30f;
            for (int rep = 0; rep < 3; ++rep) {
                cudaEventRecord(e0, st);
                launch_adlbl3_scr(g, sys, scr, site.nsys, h->adi_mode, st, forms[f]);
                cudaEventRecord(e1, st);
                float t = 0.f;
                if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess)
                    ms = std::min(ms, t);
            }
            h->site_ms[k][f] = ms;
            if (f == 0 || ms < best) {
                best = ms;
                h->site_flags[k] = forms[f];
            }
        }
        g_tune_cache[key] = {h->site_flags[k], h->site_ms[k]};
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(pool);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return GFM_E_CUDA; }
    if (const char* lg = std::getenv("GFM_TUNE_LOG"); lg && lg[0] == '1')
        for (size_t k = 0; k < h->sites.size(); ++k)
            std::fprintf(stderr, "gfm line-solver site %zu: %d system(s), %dx%dx%d, nim %d: segmented %.3f ms, plane %.3f ms, "
                         "plane-768 %.3f ms -> flags %d\n", k, h->sites[k].nsys,
                         (h->sites[k].rng[0][1] - h->sites[k].rng[0][0]) / 2 + 1,
                         (h->sites[k].rng[0][3] - h->sites[k].rng[0][2]) / 2 + 1,
                         (h->sites[k].rng[0][5] - h->sites[k].rng[0][4]) / 2 + 1, h->sites[k].rng[0][6],
                         h->site_ms[k][0], h->site_ms[k][1], h->site_ms[k][2], h->site_flags[k]);
    return GFM_OK;
}

int ensure_graph(gfm_handle* h) {
    if (!h->use_graph || h->graph_exec) return GFM_OK;
    // (GFM_RB_PLANE=0 forces the segmented passes: nothing to choose then)
    const bool tune = h->tune && !h->tuned && h->adi_mode == GFM_ADI_REDBLACK && (h->rb_flags & kRbPlane);
    h->record_sites = tune;
    h->sites.clear();
    int rc = capture_iteration(h);
    h->record_sites = false;
    if (rc || !tune) return rc;
    rc = h->prec == GFM_PREC_FP64 ? tune_sites(h, h->cd, h->scr_d) : tune_sites(h, h->cf, h->scr_f);
    if (rc) return rc;
    h->tuned = true;
    return capture_iteration(h);
}
void close_timing(gfm_handle* h) {
    cudaEventRecord(h->ev_g1, h->stream);
    if (cudaEventSynchronize(h->ev_g1) == cudaSuccess) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, h->ev_g0, h->ev_g1) == cudaSuccess) h->asm_ms += ms;
    }
}
}  // namespace

extern "C" int gfm_gpu_gflow(gfm_handle* h, int n_iter, gfm_iter_stats* out, int* n_done) {
    if (!h || n_iter < 0) return GFM_E_ARG;
    int done = 0, conv = 0;
    int rc = ensure_graph(h);
    if (rc) return rc;
    cudaEventRecord(h->ev_g0, h->stream);
    for (int it = 0; it < n_iter; ++it) {
        if ((rc = iter_launch(h))) return rc;
        rc = iter_finish(h, &conv);
        ++done;
        if (rc) { if (n_done) *n_done = done; fill_stats(h, out, 0); return rc; }
        if (conv) break;
    }
    close_timing(h);
    fill_stats(h, out, conv);
    if (n_done) *n_done = done;
    return GFM_OK;
}

extern "C" int gfm_gpu_gflow_batch(gfm_handle* const* hs, int n, int n_iter, gfm_iter_stats* out, int* n_done) {
    if (!hs || n <= 0 || n_iter < 0) return GFM_E_ARG;
    for (int i = 0; i < n; ++i) if (!hs[i]) return GFM_E_ARG;
    std::vector<int> done(n, 0), conv(n, 0);
    for (int i = 0; i < n; ++i) {
        int rc = ensure_graph(hs[i]);
        if (rc) return rc;
        cudaEventRecord(hs[i]->ev_g0, hs[i]->stream);
    }
    int status = GFM_OK;
    for (int it = 0; it < n_iter && status == GFM_OK; ++it) {
        int active = 0;
        for (int i = 0; i < n; ++i) {
            if (conv[i]) continue;
            int rc = iter_launch(hs[i]);
            if (rc) { status = rc; break; }
            ++active;
        }
        if (status != GFM_OK || active == 0) break;
        for (int i = 0; i < n; ++i) {
            if (conv[i]) continue;
            int rc = iter_finish(hs[i], &conv[i]);
            ++done[i];
            if (rc) { status = rc; break; }
        }
    }
    for (int i = 0; i < n; ++i) {
        close_timing(hs[i]);
        if (out) fill_stats(hs[i], out + i, conv[i]);
        if (n_done) n_done[i] = done[i];
    }
    return status;
}

extern "C" int gfm_gpu_download(gfm_handle* h, gfm_fields* f) {
    if (!h || !f) return GFM_E_ARG;
    return h->prec == GFM_PREC_FP64 ? download_fields(h, h->cd, f) : download_fields(h, h->cf, f);
}

namespace {
// The radiation code works in FP64: in mixed mode the handle's FP64 geometry
// holds only IBCELL until this uploads its coordinates (once per handle)
int ensure_double_coords(gfm_handle* h) {
    if (h->gd.X) return GFM_OK;
    const HostGrid& hg = h->hg;
    double *x, *dx, *r, *dr, *rs, *z, *dz;
    int rc;
    if ((rc = dupload(h, &x, hg.X)) || (rc = dupload(h, &dx, hg.DX)) || (rc = dupload(h, &r, hg.R)) ||
        (rc = dupload(h, &dr, hg.DR)) || (rc = dupload(h, &rs, hg.RS)) || (rc = dupload(h, &z, hg.Z)) ||
        (rc = dupload(h, &dz, hg.DZ)))
        return rc;
    h->gd.X = x; h->gd.DX = dx; h->gd.Rr = r; h->gd.DR = dr; h->gd.RS = rs; h->gd.Z = z; h->gd.DZ = dz;
    return GFM_OK;
}

// buffers, streams and the launch plan of the volume transfer, once per handle
int rad_prepare(gfm_handle* h, const RadArgs& in) {
    if (h->rad_ready) return GFM_OK;
    RadArgs a = in;
    const long long nc = (long long)a.MZ * a.NZ * a.LZ;
    if (int rc = ensure_double_coords(h)) return rc;
    a.g.X = h->gd.X; a.g.DX = h->gd.DX; a.g.Rr = h->gd.Rr; a.g.DR = h->gd.DR; a.g.RS = h->gd.RS;
    a.g.Z = h->gd.Z; a.g.DZ = h->gd.DZ;
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    {
        // GFM_RAD_GLOBAL_SLAB=1 (read at the first transfer): the slab arrays
        // in global scratch even where they fit in shared memory
        const char* gs = std::getenv("GFM_RAD_GLOBAL_SLAB");
        a.slab_global = gs && gs[0] == '1';
    }
    int rc = rad_plan(a, sms > 0 ? sms : 1);
    if (rc) { h->err = "radiation transfer: launch plan"; return rc; }
    a.akl_blocks = (int)std::min<long long>((nc + 255) / 256, 1024);
    const long long parts = a.part_base[3];
    if ((rc = dalloc(h, &a.ibr, nc)) || (rc = dalloc(h, &a.akl, nc * a.NWL)) || (rc = dalloc(h, &a.qel0, nc * a.NWL)) ||
        (rc = dalloc(h, &a.tcell, nc)) || (rc = dalloc(h, &a.qal_part, nc * a.NWL * parts)) ||
        (rc = dalloc(h, &a.qe, nc)) || (rc = dalloc(h, &a.qa, nc)) || (rc = dalloc(h, &a.tot_part, 8 * parts)) ||
        (rc = dalloc(h, &a.akl_part, 2LL * a.akl_blocks)) || (rc = dalloc(h, &a.qe_part, 2LL * a.akl_blocks)) ||
        (rc = dalloc(h, &a.err, 1)))
        return rc;
    for (int d = 0; d < 3; ++d) {
        a.scratch[d] = nullptr;
        a.fscratch[d] = nullptr;
        if (a.slab_in_smem[d]) continue;
        const long long A = d == 0 ? (a.NP / 2) * (a.LP / 2) : (d == 1 ? (a.MP / 2) * (a.LP / 2) : (a.MP / 2) * (a.NP / 2));
        if ((rc = dalloc(h, &a.scratch[d], 3 * A * a.NWL * a.grid[d])) || (rc = dalloc(h, &a.fscratch[d], 3 * A * a.grid[d])))
            return rc;
    }
    // corner-split lists: per CTA and part-2 column up to min(Dv, 64) entries
    // (a column splits at most once per source row and spread direction)
    for (int d = 0; d < 3; ++d) {
        const int Du = d == 0 ? a.NP : a.MP, Dv = d == 2 ? a.NP : a.LP;
        const long long cols = (long long)(Du / 2) * a.grid[d];
        a.split_capc[d] = std::min(Dv, 64);
        if ((rc = dalloc(h, &a.split_cnt[d], cols)) || (rc = dalloc(h, &a.split_meta[d], 3 * cols * a.split_capc[d])) ||
            (rc = dalloc(h, &a.split_q[d], cols * a.split_capc[d] * a.NWL)))
            return rc;
    }
    for (int s = 0; s < 2; ++s) CK(cudaStreamCreateWithFlags(&h->rad_stream[s], cudaStreamNonBlocking));
    for (int e = 0; e < 3; ++e) CK(cudaEventCreateWithFlags(&h->rad_ev[e], cudaEventDisableTiming));
    h->rad = a;
    h->rad_ready = true;
    return GFM_OK;
}
}  // namespace

namespace {

// the sum of one slot of the exchange's block partials, in block order
double wall_slot(const std::vector<double>& part, int slot) {
    double s = 0.0;
    for (int b = 0; b < kWallBlocks; ++b) s += part[(size_t)slot * kWallBlocks + b];
    return s;
}
int wall_read(gfm_handle* h, std::vector<double>& part) {
    part.resize((size_t)kWallSlots * kWallBlocks);
    CK(cudaMemcpyAsync(part.data(), h->wall.part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return GFM_OK;
}

// The exchange after a volume transfer: RAD_EMIS's patch temperatures
// (Rad_emis.f90:186-273), wall_q_amb, then wallq's loops (Qwall.f90:990-
// 1245), with T normalised throughout (T*T0 is formed where the reference
// reads T in K).  The loop control runs on the host from sums read back after
// each sweep.
template <typename R>
int wall_exchange(gfm_handle* h, Ctx<R>& c, gfm_wall_totals* tot) {
    WallArgs& a = h->wall;
    const gfm_wall_spec& w = h->wspec;
    cudaStream_t st = h->stream;
    std::vector<double> part;
    int rc;
    launch_wall_start<R>(a, c.T, h->wall_first, st);
    launch_wall_init<R>(a, c.QA, c.QE, st);
    launch_wall_qamb(a, st);
    if ((rc = wall_read(h, part))) return rc;
    gfm_wall_totals t{};
    t.q_incident_total = wall_slot(part, W_INC_TOTAL); t.q_incident_wall = wall_slot(part, W_INC_WALL);
    t.q_incident_inlet = wall_slot(part, W_INC_INLET); t.q_incident_exit = wall_slot(part, W_INC_EXIT);
    t.q_incident_melt = wall_slot(part, W_INC_MELT);
    const double tol = 1.0e-10;   // wall_radiosity_tolerance, radiation_boundary_tolerance
    int nn = 1, nnextra = w.maxri1, outer = 0;
    double rel_mean = 0.0;
    while (nn <= w.maxri1 && nn <= nnextra) {
        const int minradi = w.minri2;
        // calc_q_conv_wall: the wall sink's kernel on the exchange's temperatures
        launch_wall_to_sink(a, h->d_patches, st);
        launch_qconv(c, st);
        launch_wall_from_sink<R>(a, c.qconv, st);
        int n = 1, nextra = w.maxri2;
        while (n <= w.maxri2 && n <= nextra) {
            launch_wall_sweep(a, st);
            std::swap(a.J, a.Jn);
            ++h->iterw;
            double rel = 0.0;
            CK(cudaMemcpyAsync(part.data() + (size_t)W_REL * kWallBlocks, a.part + (size_t)W_REL * kWallBlocks,
                               kWallBlocks * sizeof(double), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            rel = wall_slot(part, W_REL);
            rel_mean = rel / a.nb;
            if (rel_mean < tol && n > minradi && nextra == w.maxri2) nextra = n + 3;
            ++n;
        }
        const double prev_q_melt = h->q_melt;
        launch_wall_rad(a, 1 << 4, st);
        launch_wall_temps(a, st);
        launch_wall_qamb(a, st);
        if ((rc = wall_read(h, part))) return rc;
        h->q_melt = wall_slot(part, W_Q_MELT);
        t.q_wall_loss = wall_slot(part, W_Q_LOSS);
        t.qconv_total = wall_slot(part, W_QCONV);
        const double chg = std::fabs((prev_q_melt - h->q_melt) / (h->q_melt + 1.0e-16));
        if (chg < tol && nnextra == w.maxri1) nnextra = nn + 1;
        ++outer;
        ++nn;
    }
    // after the loops: wall T into the field, inlet, outlet and melt totals
    launch_wall_rad(a, (1 << 2) | (1 << 3) | (1 << 4), st);
    launch_wall_post<R>(a, c.T, st);
    if ((rc = wall_read(h, part))) return rc;
    h->avg_wall_T = wall_slot(part, W_T_AREA) / h->wall_area_total;
    if (h->wall_frac_exits) launch_wall_exits(a, h->d_frac_exit, h->d_frac, h->avg_wall_T, st);
    launch_wall_to_sink(a, h->d_patches, st);   // the gas solve's wall sink reads the new b_T
    const double one = 1.0;
    CK(cudaMemcpyAsync(c.scal + S_RAD_DONE, &one, sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    h->wall_first = 0;
    t.b_cnt = a.nb;
    t.sweeps = h->iterw;
    t.outer = outer;
    t.avg_wall_T = h->avg_wall_T;
    t.q_melt = h->q_melt;
    t.q_rad_inlet = wall_slot(part, W_Q_RAD_IN);
    t.q_rad_outlet = wall_slot(part, W_Q_RAD_OUT);
    t.qm_flame = wall_slot(part, W_QM_FLAME);
    t.qm_bnds = wall_slot(part, W_QM_BNDS);
    t.qm_conv = wall_slot(part, W_QM_CONV);
    t.rel_rad_chg_mean = rel_mean;
    if (tot) *tot = t;
    return GFM_OK;
}

}  // namespace

// Boundary-patch data of the exchange (prepare_for_wall_radiation_calculation
// steps 5-8, Qwall.f90:395-736) from the case's patch list, and the view
// factors on the device.
extern "C" int gfm_gpu_wall_setup(gfm_handle* h, const gfm_wall_spec* spec) {
    if (!h || !spec) return GFM_E_ARG;
    if (h->wall_on) { h->err = "wall exchange: already set up"; return GFM_E_ARG; }
    if (spec->nex < 0 || spec->nex > GFM_MAX_EXHAUSTS || spec->maxri1 < 1 || spec->maxri2 < 1 || spec->eps_w <= 0.0 ||
        spec->eps_c <= 0.0 || spec->eps_m <= 0.0) {
        h->err = "wall exchange: inputs out of range";
        return GFM_E_ARG;
    }
    const int nb = (int)h->bp_typ.size();
    if (nb < 2) { h->err = "wall exchange: fewer than two boundary patches"; return GFM_E_ARG; }
    const HostGrid& g = h->hg;
    std::vector<int> typ(nb), bi(nb), bj(nb), bk(nb), ori(nb), dir(nb), o_bc(nb), o_b(nb), sink(nb), exh(nb, 0),
        frac_exit(nb, 0);
    std::vector<int> bci(nb), bcj(nb), bck(nb);
    std::vector<double> px(nb), py(nb), pz(nb), emis(nb), area(nb), face(nb), bt_exit(nb, 0.0), frac(nb, 0.0);
    int ns = 0;
    h->wall_area_total = 0.0;
    for (int n = 0; n < nb; ++n) {
        typ[n] = h->bp_typ[n]; bi[n] = h->bp_i[n]; bj[n] = h->bp_j[n]; bk[n] = h->bp_k[n];
        ori[n] = h->bp_ori[n]; dir[n] = h->bp_dir[n];
        const int s = dir[n] == 0 ? -1 : 1;   // the closed cell is behind the face
        bci[n] = bi[n] + (ori[n] == 1 ? s : 0);
        bcj[n] = bj[n] + (ori[n] == 2 ? s : 0);
        bck[n] = bk[n] + (ori[n] == 3 ? s : 0);
        o_bc[n] = (int)pidx(h->gd, bci[n], bcj[n], bck[n]);
        o_b[n] = (int)pidx(h->gd, bi[n], bj[n], bk[n]);
        px[n] = g.X[bi[n]]; py[n] = g.R[bj[n]]; pz[n] = g.Z[bk[n]];
        area[n] = ori[n] == 1 ? g.DR[bj[n]] * g.DZ[bk[n]] : ori[n] == 2 ? g.DX[bi[n]] * g.DZ[bk[n]] : g.DX[bi[n]] * g.DR[bj[n]];
        if (typ[n] == 1) {
            const int ktop = ori[n] == 3 ? g.LP - 1 : g.LP;
            emis[n] = (g.Z[bk[n]] >= spec->height_to_ceiling || (bk[n] == ktop && spec->have_crown == 0)) ? spec->eps_c
                                                                                                              : spec->eps_w;
            h->wall_area_total += area[n];
        } else {
            emis[n] = typ[n] == 4 && ori[n] == 3 ? spec->eps_m : 1.0;
        }
        sink[n] = (typ[n] == 1 || typ[n] == 4) ? ns++ : -1;
        if (typ[n] == 3) {
            // the exhaust the patch belongs to (step 6, Qwall.f90:534-557)
            for (int m = 0; m < spec->nex && !exh[n]; ++m) {
                if (ori[n] != spec->exh_orient[m] || dir[n] != spec->exh_direct[m]) continue;
                const bool in = ori[n] == 1 ? (bcj[n] >= spec->exh_j1[m] && bcj[n] <= spec->exh_j2[m] && bck[n] >= spec->exh_k1[m] && bck[n] <= spec->exh_k2[m])
                              : ori[n] == 2 ? (bci[n] >= spec->exh_i1[m] && bci[n] <= spec->exh_i2[m] && bck[n] >= spec->exh_k1[m] && bck[n] <= spec->exh_k2[m])
                                            : (bci[n] >= spec->exh_i1[m] && bci[n] <= spec->exh_i2[m] && bcj[n] >= spec->exh_j1[m] && bcj[n] <= spec->exh_j2[m]);
                if (in) exh[n] = m + 1;
            }
            if (!exh[n]) { h->err = "wall exchange: an exit patch outside every exhaust"; return GFM_E_ARG; }
            const int m = exh[n] - 1;
            bt_exit[n] = spec->exh_type[m] == 0 ? spec->exh_frac[m] * h->avg_wall_T : spec->exh_fixed[m];
            frac_exit[n] = spec->exh_type[m] == 0;
            frac[n] = spec->exh_frac[m];
            if (frac_exit[n]) h->wall_frac_exits = 1;
        }
    }
    if (ns != h->cd.n_patch) { h->err = "wall exchange: patch list differs from the wall sink's"; return GFM_E_ARG; }
    if (h->wall_area_total <= 0.0) { h->err = "wall exchange: no wall patches"; return GFM_E_ARG; }
    // step 8: the face area of the patches on one cell, with the reference's
    // chain of same-cell links as it is written (Qwall.f90:684-736)
    {
        std::vector<int> c1(nb + 1, 0), c2(nb + 1, 0), c3(nb + 1, 0), c4(nb + 1, 0);   // 1-based, 0 = none
        auto same = [&](int n, int m) { return bci[n - 1] == bci[m - 1] && bcj[n - 1] == bcj[m - 1] && bck[n - 1] == bck[m - 1]; };
        for (int n = 1; n <= nb; ++n)
            for (int m = n + 1; m <= nb; ++m) {
                if (!same(n, m)) continue;
                if (c1[n] == 0) { c1[n] = m; c1[m] = n; }
                else if (c2[n] == 0) {
                    if (c1[n] == m) continue;
                    c2[n] = m; c1[m] = n; c2[m] = c1[n]; c2[c1[n]] = m;
                } else if (c3[n] == 0) {
                    if (c1[n] == m || c2[n] == m) continue;
                    c3[n] = m; c1[m] = n; c2[m] = c1[n]; c3[c2[n]] = m; c3[m] = c2[n];
                } else if (c4[n] == 0) {
                    if (c1[n] == m || c2[n] == m || c3[n] == m) continue;
                    c4[n] = m; c1[m] = n; c2[m] = c1[n]; c4[c2[n]] = m; c3[m] = c2[n]; c4[c3[n]] = m; c4[m] = c3[n];
                }
            }
        for (int n = 1; n <= nb; ++n) {
            double f = area[n - 1];
            const int links[4] = {c1[n], c2[n], c3[n], c4[n]};
            for (int q = 0; q < 4 && links[q]; ++q) f = f + area[links[q] - 1];
            face[n - 1] = f;
        }
    }
    WallArgs a{};
    a.nb = nb;
    int* ip[10];
    const std::vector<int>* iv[10] = {&typ, &bi, &bj, &bk, &ori, &dir, &o_bc, &o_b, &sink, &frac_exit};
    double* dp[7];
    const std::vector<double>* dv[7] = {&px, &py, &pz, &emis, &area, &face, &bt_exit};
    int rc;
    for (int q = 0; q < 10; ++q) if ((rc = dupload(h, &ip[q], *iv[q]))) return rc;
    for (int q = 0; q < 7; ++q) if ((rc = dupload(h, &dp[q], *dv[q]))) return rc;
    a.typ = ip[0]; a.bi = ip[1]; a.bj = ip[2]; a.bk = ip[3]; a.ori = ip[4]; a.dir = ip[5];
    a.o_bc = ip[6]; a.o_b = ip[7]; a.sink = ip[8]; h->d_frac_exit = ip[9];
    a.px = dp[0]; a.py = dp[1]; a.pz = dp[2]; a.emis = dp[3]; a.area = dp[4]; a.face_area = dp[5]; a.bT_exit = dp[6];
    if ((rc = dupload(h, &h->d_frac, frac))) return rc;
    double* work[10];
    for (int q = 0; q < 10; ++q) if ((rc = dalloc(h, &work[q], nb))) return rc;
    a.bT = work[0]; a.J = work[1]; a.Jn = work[2]; a.qc = work[3]; a.qeb = work[4]; a.qconv = work[5];
    a.qamb = work[6]; a.rad = work[7]; a.rel = work[8]; a.vfsum = work[9];
    if ((rc = dalloc(h, &a.part, (long long)kWallSlots * kWallBlocks))) return rc;
    // the view factors: FP64 on the FP64 path, FP32 on the mixed one
    const size_t vf_bytes = (size_t)nb * nb * (h->prec == GFM_PREC_FP64 ? 8 : 4);
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    if (vf_bytes + ((size_t)1 << 30) > free_b) { h->err = "wall exchange: view factors exceed device memory"; return GFM_E_NOMEM; }
    if (h->prec == GFM_PREC_FP64) { if ((rc = dalloc(h, &a.vf64, (long long)nb * nb))) return rc; }
    else if ((rc = dalloc(h, &a.vf32, (long long)nb * nb))) return rc;
    a.sig = h->params.sig;
    const double t2 = spec->t_mnk * spec->t_mnk;
    a.radi_min = h->params.sig * (t2 * t2);   // Setup.f90:214
    a.t0 = h->params.t0;
    a.u_a0 = (spec->w_k < 1.0e-20 || spec->h_a < 1.0e-20) ? 0.0 : 1.0 / (spec->w_d / spec->w_k + 1.0 / spec->h_a);
    a.t_a = spec->t_a;
    a.t_mnk = spec->t_mnk;
    if ((rc = launch_wall_vf(a, h->stream))) { h->err = "wall exchange: view-factor launch"; return rc; }
    CK(cudaStreamSynchronize(h->stream));
    h->wall = a;
    h->wspec = *spec;
    h->wall_typ = typ;
    h->wall_exh = exh;
    h->wall_on = true;
    return GFM_OK;
}

extern "C" int gfm_gpu_wall_totals(gfm_handle* h, gfm_wall_totals* out) {
    if (!h || !out || !h->wall_on) return GFM_E_ARG;
    *out = h->wall_last;
    return GFM_OK;
}

extern "C" int gfm_gpu_wall_get(gfm_handle* h, const char* name, double* out, int cap) {
    if (!h || !name || !out || !h->wall_on) return GFM_E_ARG;
    const WallArgs& a = h->wall;
    if (cap < a.nb) return GFM_E_ARG;
    const std::string s(name);
    if (s == "qrs") {
        // the melt-surface heat flux of the melt patches, qc + q_conv + the
        // radiation from the boundaries - the radiosity (Qwall.f90:1166), 0 elsewhere
        std::vector<double> qc(a.nb), qv(a.nb), rad(a.nb), J(a.nb);
        CK(cudaMemcpy(qc.data(), a.qc, (size_t)a.nb * sizeof(double), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(qv.data(), a.qconv, (size_t)a.nb * sizeof(double), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(rad.data(), a.rad, (size_t)a.nb * sizeof(double), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(J.data(), a.J, (size_t)a.nb * sizeof(double), cudaMemcpyDeviceToHost));
        for (int i = 0; i < a.nb; ++i) out[i] = h->wall_typ[i] == 4 ? qc[i] + qv[i] + rad[i] - J[i] : 0.0;
        return a.nb;
    }
    // the patch list and the closed cell behind each patch (the face's
    // neighbour on the side its direction points away from)
    const std::vector<int16_t>* list = s == "b_typ" ? &h->bp_typ : s == "b_i" ? &h->bp_i : s == "b_j" ? &h->bp_j
                                     : s == "b_k" ? &h->bp_k : s == "b_orient" ? &h->bp_ori
                                     : s == "b_direct" ? &h->bp_dir : nullptr;
    if (list) {
        for (int n = 0; n < a.nb; ++n) out[n] = (*list)[n];
        return a.nb;
    }
    if (s == "bc_i" || s == "bc_j" || s == "bc_k") {
        const int axis = s == "bc_i" ? 1 : s == "bc_j" ? 2 : 3;
        const std::vector<int16_t>& pos = axis == 1 ? h->bp_i : axis == 2 ? h->bp_j : h->bp_k;
        for (int n = 0; n < a.nb; ++n)
            out[n] = pos[n] + (h->bp_ori[n] == axis ? (h->bp_dir[n] == 0 ? -1 : 1) : 0);
        return a.nb;
    }
    if (s == "b_exh") {
        for (int n = 0; n < a.nb; ++n) out[n] = h->wall_exh[n];
        return a.nb;
    }
    const double* src = s == "b_t" ? a.bT : s == "radiosity" ? a.J : s == "q_amb" ? a.qamb : s == "q_conv" ? a.qconv
                      : s == "qc" ? a.qc : s == "qeb" ? a.qeb : s == "emis" ? a.emis : s == "b_face_area" ? a.face_area
                      : s == "patch_area" ? a.area : s == "rad" ? a.rad : s == "vf_sum" ? a.vfsum : nullptr;
    if (!src) return GFM_E_ARG;
    CK(cudaMemcpy(out, src, (size_t)a.nb * sizeof(double), cudaMemcpyDeviceToHost));
    return a.nb;
}

extern "C" long long gfm_gpu_wall_vf(gfm_handle* h, double* out, long long cap) {
    if (!h || !out || !h->wall_on) return GFM_E_ARG;
    const WallArgs& a = h->wall;
    const long long nn = (long long)a.nb * a.nb;
    if (cap < nn) return GFM_E_ARG;
    if (a.vf64) {
        CK(cudaMemcpy(out, a.vf64, (size_t)nn * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
        // FP32 on the mixed path: whole rows at a time, about 64 MB a copy
        const size_t rows = std::max<size_t>(1, ((size_t)64 << 20) / ((size_t)a.nb * sizeof(float)));
        std::vector<float> buf(rows * (size_t)a.nb);
        for (size_t n0 = 0; n0 < (size_t)a.nb; n0 += rows) {
            const size_t cnt = std::min(rows, (size_t)a.nb - n0) * (size_t)a.nb;
            CK(cudaMemcpy(buf.data(), a.vf32 + n0 * a.nb, cnt * sizeof(float), cudaMemcpyDeviceToHost));
            for (size_t q = 0; q < cnt; ++q) out[n0 * a.nb + q] = buf[q];
        }
    }
    return nn;
}

extern "C" int gfm_gpu_wall_put(gfm_handle* h, const char* name, const double* src, int n) {
    if (!h || !name || !src || !h->wall_on) return GFM_E_ARG;
    const WallArgs& a = h->wall;
    const std::string s(name);
    if (s == "radiosity" || s == "b_t") {
        if (n != a.nb) return GFM_E_ARG;
        for (int q = 0; q < n; ++q) if (!std::isfinite(src[q])) return GFM_E_NAN;
        CK(cudaMemcpy(s == "b_t" ? a.bT : a.J, src, (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
        if (s == "b_t") {
            // the given wall temperatures stand at the next exchange, and the
            // gas solve's wall sink reads them too
            h->wall_first = 0;
            launch_wall_to_sink(a, h->d_patches, h->stream);
            CK(cudaStreamSynchronize(h->stream));
        }
        return GFM_OK;
    }
    if (n != 1 || !std::isfinite(src[0])) return GFM_E_ARG;
    if (s == "iterw") h->iterw = (int)src[0];
    else if (s == "q_melt") h->q_melt = src[0];
    else if (s == "avg_wall_T") h->avg_wall_T = src[0];
    else return GFM_E_ARG;
    return GFM_OK;
}

namespace {
__global__ void k_cast_d2f(const double* __restrict__ s, float* __restrict__ d, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = (float)s[i];
}
__global__ void k_cast_f2d(const float* __restrict__ s, double* __restrict__ d, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = (double)s[i];
}
int cast_grid(long long n) { return (int)std::min<long long>((n + 255) / 256, 4096); }

template <typename R>
int minor_alloc(gfm_handle* h, MinorDev<R>& m) {
    if (m.smf) return GFM_OK;
    const long long ncl = (long long)(h->hg.MP / 2) * (h->hg.NP / 2) * (h->hg.LP / 2);
    int rc;
    for (int l = 0; l < 7; ++l)
        if ((rc = dalloc(h, &m.gfm[l], h->NS))) return rc;
    if ((rc = dalloc(h, &m.smf, h->NS)) || (rc = dalloc(h, &m.bsp, h->NS)) || (rc = dalloc(h, &m.sfpp, h->NS)) ||
        (rc = dalloc(h, &m.rrms, 5 * ncl)))
        return rc;
    return GFM_OK;
}

template <typename R>
int minor_put(gfm_handle* h, const GeoT<R>& g, MinorDev<R>& m, const gfm_minor* src) {
    int rc;
    if ((rc = minor_alloc(h, m))) return rc;
    cudaStream_t st = h->stream;
    const long long N = h->N;
    const long long ncl = (long long)(h->hg.MP / 2) * (h->hg.NP / 2) * (h->hg.LP / 2);
    auto put = [&](const double* a, R* dst) -> int {
        CK(cudaMemcpyAsync(h->d_stage, a, N * sizeof(double), cudaMemcpyHostToDevice, st));
        launch_to_split(g, h->d_stage, dst, st);
        return GFM_OK;
    };
    for (int l = 0; l < 7; ++l)
        if ((rc = put(src->gfm + (long long)l * N, m.gfm[l]))) return rc;
    if ((rc = put(src->smf, m.smf)) || (rc = put(src->bs_soot_prev, m.bsp)) || (rc = put(src->sfp_soot_prev, m.sfpp)))
        return rc;
    // RRMS keeps the cell layout; 5 x ncell <= N, so it fits the staging buffer
    CK(cudaMemcpyAsync(h->d_stage, src->rrms, 5 * ncl * sizeof(double), cudaMemcpyHostToDevice, st));
    if constexpr (std::is_same<R, double>::value) {
        CK(cudaMemcpyAsync(m.rrms, h->d_stage, 5 * ncl * sizeof(double), cudaMemcpyDeviceToDevice, st));
    } else {
        k_cast_d2f<<<cast_grid(5 * ncl), 256, 0, st>>>(h->d_stage, m.rrms, 5 * ncl);
    }
    CK(cudaStreamSynchronize(st));
    return GFM_OK;
}

template <typename R>
int minor_get(gfm_handle* h, const GeoT<R>& g, const MinorDev<R>& m, gfm_minor* out) {
    cudaStream_t st = h->stream;
    const long long N = h->N;
    const long long ncl = (long long)(h->hg.MP / 2) * (h->hg.NP / 2) * (h->hg.LP / 2);
    auto get = [&](const R* src, double* a) -> int {
        launch_from_split(g, src, h->d_stage, st);
        CK(cudaMemcpyAsync(a, h->d_stage, N * sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        return GFM_OK;
    };
    int rc;
    for (int l = 0; l < 7; ++l)
        if ((rc = get(m.gfm[l], out->gfm + (long long)l * N))) return rc;
    if ((rc = get(m.smf, out->smf)) || (rc = get(m.bsp, out->bs_soot_prev)) || (rc = get(m.sfpp, out->sfp_soot_prev)))
        return rc;
    if constexpr (std::is_same<R, double>::value) {
        CK(cudaMemcpyAsync(h->d_stage, m.rrms, 5 * ncl * sizeof(double), cudaMemcpyDeviceToDevice, st));
    } else {
        k_cast_f2d<<<cast_grid(5 * ncl), 256, 0, st>>>(m.rrms, h->d_stage, 5 * ncl);
    }
    CK(cudaMemcpyAsync(out->rrms, h->d_stage, 5 * ncl * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return GFM_OK;
}

// the band model's AKLG and AKLS on the current state (gas.cu), when the
// case asks for it; a no-op for the gray bands
int gas_band(gfm_handle* h) {
    if (!h->params.gas_model) return GFM_OK;
    if (!h->minor_on) { h->err = "band model: no minor species state (gfm_gpu_minor_upload)"; return GFM_E_ARG; }
    const int ncl = (h->hg.MP / 2) * (h->hg.NP / 2) * (h->hg.LP / 2);
    const int nwl = h->cd.nwl;
    int rc;
    if (!h->gas.aklg) {
        if ((rc = dalloc(h, &h->gas.aklg, (long long)ncl * nwl)) || (rc = dalloc(h, &h->gas.akls, (long long)ncl * nwl)) ||
            (rc = dalloc(h, &h->gas.fvs, ncl)) || (rc = dalloc(h, &h->gas.setter, ncl)) ||
            (rc = dalloc(h, &h->gas.blockmax, gas_scan_blocks(ncl))) || (rc = dalloc(h, &h->gas.err, 1)))
            return rc;
        std::vector<double> t((size_t)gas_sqper_size());
        gas_sqper_fill(t.data());
        double* d = nullptr;
        if ((rc = dupload(h, &d, t))) return rc;
        h->gas.sqper = d;
        std::vector<float> tf(t.begin(), t.end());
        float* df = nullptr;
        if ((rc = dupload(h, &df, tf))) return rc;
        h->gas.sqperf = df;
    }
    if ((rc = ensure_double_coords(h))) return rc;
    const gfm_params& P = h->params;
    if (h->prec == GFM_PREC_FP64) {
        const Ctx<double>& c = h->cd;
        rc = launch_gas_band<double>(h->gas, h->gd, c.T, c.P, c.DNST, h->mnd.gfm, h->mnd.smf, P.t0, P.pg0, P.dnst0, nwl,
                                     c.wl, h->stream);
    } else {
        const Ctx<float>& c = h->cf;
        rc = launch_gas_band<float>(h->gas, h->gd, c.T, c.P, c.DNST, h->mnf.gfm, h->mnf.smf, P.t0, P.pg0, P.dnst0, nwl,
                                    h->cd.wl, h->stream);
    }
    if (rc) h->err = "band model launch";
    return rc;
}
// the band model's error bits, read after the stream has finished
int gas_check(gfm_handle* h) {
    if (!h->params.gas_model || !h->gas.err) return GFM_OK;
    int e = 0;
    CK(cudaMemcpy(&e, h->gas.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        h->err = (e & 2) ? "band model: BANDA argument < 0 (Rad_gas.f90:368-371)"
                         : "band model: W_R <= 0 with CO2 present (Rad_gas.f90:233)";
        return GFM_E_NAN;
    }
    return GFM_OK;
}
}  // namespace

namespace {
template <typename R>
int ms_alloc(gfm_handle* h, MsScratch<R>& s) {
    if (s.ap1) return GFM_OK;
    const int ni = (h->hg.MP - 2 - 4) / 2 + 1, nj = (h->hg.NP - 2 - 4) / 2 + 1, nk = (h->hg.LP - 2 - 4) / 2 + 1;
    s.nq = ni > 0 && nj > 0 && nk > 0 ? ni * nj * nk : 0;
    int rc;
    for (int q = 0; q < 6; ++q)
        if ((rc = dalloc(h, &s.as[q], h->NS))) return rc;
    for (int l = 0; l < 7; ++l)
        if ((rc = dalloc(h, &s.fz[l], h->NS)) || (rc = dalloc(h, &s.bs[l], h->NS))) return rc;
    if ((rc = dalloc(h, &s.ap1, h->NS)) || (rc = dalloc(h, &s.ap, h->NS)) ||
        (rc = dalloc(h, &s.r4, std::max(s.nq, 1))) || (rc = dalloc(h, &s.setter, std::max(s.nq, 1))) ||
        (rc = dalloc(h, &s.blockmax, std::max(gas_scan_blocks(s.nq), 1))) || (rc = dalloc(h, &s.carry, 1)) ||
        (rc = dalloc(h, &s.stats, 8)))
        return rc;
    const gfm_params& P = h->params;
    s.rfm = P.rfm; s.rfm_soot = P.rfm_soot; s.rf_sf = P.rf_soot_form; s.rf_so = P.rf_soot_oxid;
    s.soot_cap = P.soot_cap; s.t0_sf = P.t0_sf; s.t0_so = P.t0_so; s.aform = P.aform; s.aoxid = P.aoxid;
    s.esf_r = P.esf_r; s.eso_r = P.eso_r;
    s.snorm = P.r0 / (P.dnst0 * P.ug0);   // Sourcem.f90:81
    s.react = P.react;
    // the open volume (Grid3.f90:286-294), in the reference's loop order
    double v = 0.0;
    const HostGrid& hg = h->hg;
    for (int i = 2; i <= hg.MP; i += 2)
        for (int j = 2; j <= hg.NP; j += 2)
            for (int k = 2; k <= hg.LP; k += 2)
                if (hg.at(i, j, k) == 0) v = v + hg.DX[i] * hg.DR[j] * hg.RS[j] * hg.DZ[k] * 1.0;
    h->vol_tot = v;
    return GFM_OK;
}

// INITSVM (Initsv.f90:329-378) on the device
template <typename R>
int initsvm_dev(gfm_handle* h, Ctx<R>& c, MinorDev<R>& m, int restart) {
    int rc;
    if ((rc = minor_alloc(h, m))) return rc;
    launch_initsvm(c, m, restart, h->stream);
    if (restart) launch_extrm(c, m, h->stream);
    launch_intpm(c, m, h->stream);
    h->igs0 = 0;
    CK(cudaStreamSynchronize(h->stream));
    return GFM_OK;
}
int minor_initsvm(gfm_handle* h, int restart) {
    if (restart && !h->minor_on) { h->err = "INITSVM restart: no minor species state"; return GFM_E_ARG; }
    int rc = h->prec == GFM_PREC_FP64 ? initsvm_dev(h, h->cd, h->mnd, restart) : initsvm_dev(h, h->cf, h->mnf, restart);
    if (rc) return rc;
    if (!h->minor_on) for (int l = 0; l < 8; ++l) { h->resid_ms[l] = 1.0e-16; h->resid_ms_pre[l] = 1.0e-16; }
    h->minor_on = true;
    return GFM_OK;
}

// MSFLOW (Msflow.f90:29-165): GSLV3M, the report sums, the convergence test
// after iteration 10, EXTRM and INTPM, up to maxms iterations
template <typename R>
int msflow_dev(gfm_handle* h, Ctx<R>& c, MinorDev<R>& m, MsScratch<R>& s, AdiScratch<R>* scr, int maxms,
               gfm_msflow_stats* out) {
    int rc;
    if ((rc = ms_alloc(h, s))) return rc;
    cudaStream_t st = h->stream;
    const GeoT<R>& g = c.g;
    const gfm_params& P = h->params;
    h->igs0 = 0;
    int done = 0;
    for (int it = 0; it < maxms; ++it) {
        h->itr_ms += 1;
        ++done;
        CK(cudaMemsetAsync(c.partials, 0, sizeof(double) * kRedSlots * kRedBlocks, st));
        // reaction rates, with the coefficients the reference's AS array holds now
        R* const* as_spin = h->as_minor_current ? s.as : c.ASs[c.as_set[6]];
        launch_ms_rates(c, m, s, as_spin, st);
        if (h->igs0 == 0) {   // GSLV3G0(...,0) of the first species after INITSVM / MSFLOW's start
            launch_scalar_faces_into(c, s.as, P.ssigma, st);
            h->as_minor_current = true;
            h->igs0 = 1;
        }
        launch_ms_ap(c, s, st);
        for (int l = 0; l < 7; ++l) CK(cudaMemcpyAsync(s.fz[l], m.gfm[l], sizeof(R) * h->NS, cudaMemcpyDeviceToDevice, st));
        launch_ms_species(c, m, s, st);
        Sys<R> ss[7];
        for (int l = 0; l < 7; ++l) {
            ss[l] = sys_of<R>(s.fz[l], s.ap, s.as, s.bs[l], 4, g.MPM2, g.NJY1, g.NJY2, g.LKZ1, g.LKZ2, P.ntimesm);
            launch_residual(c, ss[l], kSlMsPre + l, st);
        }
        launch_adlbl3_scr(g, ss, scr, 7, h->adi_mode, st, h->rb_flags);   // returns the kernels it launched
        for (int l = 0; l < 7; ++l) launch_residual(c, ss[l], kSlMsPost + l, st);
        launch_ms_update(c, m, s, st);
        if (P.react) {   // soot (Gslv3m.f90:225-284)
            CK(cudaMemcpyAsync(s.fz[0], m.smf, sizeof(R) * h->NS, cudaMemcpyDeviceToDevice, st));
            launch_soot_system(c, m, s, h->itr_ms, st);
            Sys<R> so = sys_of<R>(s.fz[0], s.ap, s.as, s.bs[0], 4, g.MPM2, g.NJY1, g.NJY2, g.LKZ1, g.LKZ2, P.ntimesm);
            launch_residual(c, so, kSlMsPre + 7, st);
            launch_adlbl3_scr(g, &so, scr, 1, h->adi_mode, st, h->rb_flags);
            launch_residual(c, so, kSlMsPost + 7, st);
            launch_soot_update(c, m, s, st);
        }
        launch_ms_stats(c, m, s, st);
        FinishSpec f{};
        auto add = [&](int slot, int dst, int op) { f.slot[f.n] = slot; f.dst[f.n] = dst; f.op[f.n] = op; ++f.n; };
        const int nsys = P.react ? 8 : 7;
        for (int l = 0; l < nsys; ++l) { add(kSlMsPre + l, S_MS_RPRE + l, 2); add(kSlMsPost + l, S_MS_RES + l, 2); }
        add(kSlMsBal, S_MS_BAL, 0);
        if (P.react) { add(kSlMsSoot, S_MS_SOOT, 0); add(kSlMsSmfMax, S_MS_SMFMAX, 1); add(kSlMsSmfMaxNc, S_MS_SMFMAXNC, 1); }
        launch_finish(c.partials, c.scal, f, (double)h->ncells, st);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(h->h_scal, c.scal, sizeof(double) * (S_NUM + 128), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int l = 0; l < nsys; ++l) { h->resid_ms_pre[l] = h->h_scal[S_MS_RPRE + l]; h->resid_ms[l] = h->h_scal[S_MS_RES + l]; }
        h->imscon = 0;
        if (h->itr_ms > 10) {
            h->imscon = 1;
            for (int l = 0; l < 8; ++l) if (h->resid_ms[l] > P.bmcon) h->imscon = 0;
        }
        if (h->imscon == 1) break;
        launch_extrm(c, m, st);
        launch_intpm(c, m, st);
    }
    double stats[8] = {0};
    CK(cudaMemcpyAsync(stats, s.stats, sizeof stats, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (out) {
        std::memset(out, 0, sizeof *out);
        out->itr_ms = h->itr_ms;
        out->iterations = done;
        out->converged = h->imscon;
        for (int l = 0; l < 8; ++l) { out->resid_ms_pre[l] = h->resid_ms_pre[l]; out->resid_ms[l] = h->resid_ms[l]; }
        out->bal_ms = h->h_scal[S_MS_BAL] * 1.0 / h->vol_tot;
        out->soot_tot = h->h_scal[S_MS_SOOT];
        out->smf_max = h->h_scal[S_MS_SMFMAX];
        out->smf_max_noclip = h->h_scal[S_MS_SMFMAXNC];
        for (int l = 0; l < 7; ++l) out->gfm_out[l] = stats[l];
        out->svf_r = stats[7];
    }
    return GFM_OK;
}
int msflow_run(gfm_handle* h, int maxms, gfm_msflow_stats* out) {
    if (!h->minor_on) { h->err = "MSFLOW: no minor species state (gfm_gpu_initsvm or gfm_gpu_minor_upload)"; return GFM_E_ARG; }
    return h->prec == GFM_PREC_FP64 ? msflow_dev(h, h->cd, h->mnd, h->msd, h->scr_d, maxms, out)
                                    : msflow_dev(h, h->cf, h->mnf, h->msf, h->scr_f, maxms, out);
}
}  // namespace

extern "C" int gfm_gpu_initsvm(gfm_handle* h, int restart) {
    if (!h) return GFM_E_ARG;
    return minor_initsvm(h, restart);
}

extern "C" int gfm_gpu_msflow(gfm_handle* h, int maxms, gfm_msflow_stats* out) {
    if (!h || maxms < 0) return GFM_E_ARG;
    return msflow_run(h, maxms, out);
}

extern "C" int gfm_gpu_minor_upload(gfm_handle* h, const gfm_minor* m) {
    if (!h || !m || !m->gfm || !m->smf || !m->bs_soot_prev || !m->sfp_soot_prev || !m->rrms) return GFM_E_ARG;
    int rc = h->prec == GFM_PREC_FP64 ? minor_put(h, h->gd, h->mnd, m) : minor_put(h, h->gfl, h->mnf, m);
    if (rc) return rc;
    if (!h->minor_on) for (int l = 0; l < 8; ++l) { h->resid_ms[l] = 1.0e-16; h->resid_ms_pre[l] = 1.0e-16; }
    h->minor_on = true;
    h->minor_from_host = true;
    h->itr_ms = m->itr_ms;
    h->imscon = m->imscon;
    return GFM_OK;
}

extern "C" int gfm_gpu_minor_download(gfm_handle* h, gfm_minor* m) {
    if (!h || !m || !m->gfm || !m->smf || !m->bs_soot_prev || !m->sfp_soot_prev || !m->rrms) return GFM_E_ARG;
    if (!h->minor_on) { h->err = "no minor species state"; return GFM_E_ARG; }
    int rc = h->prec == GFM_PREC_FP64 ? minor_get(h, h->gd, h->mnd, m) : minor_get(h, h->gfl, h->mnf, m);
    if (rc) return rc;
    m->itr_ms = h->itr_ms;
    m->imscon = h->imscon;
    return GFM_OK;
}

extern "C" int gfm_gpu_rad_transfer(gfm_handle* h, gfm_rad_totals* out) {
    if (!h) return GFM_E_ARG;
    const Ctx<double>& cdb = h->cd;
    if (cdb.nwl < 1 || cdb.nwl > kRadMaxBands) { h->err = "radiation transfer: 1 to 16 bands"; return GFM_E_UNSUPPORTED; }
    if (!h->rad_ready) {
        RadArgs a{};
        a.g = h->gd;
        a.MP = h->gd.MP; a.NP = h->gd.NP; a.LP = h->gd.LP;
        a.MZ = a.MP / 2; a.NZ = a.NP / 2; a.LZ = a.LP / 2;
        a.NWL = cdb.nwl;
        a.t0 = h->params.t0;
        a.sgn = h->params.sig * h->params.ri * h->params.ri;                      // SGN (Rad0.f90:33)
        for (int l = 0; l < a.NWL; ++l) {
            a.akl0[l] = cdb.akl0[l];
            a.deb0[l] = h->params.hck / h->params.ri / cdb.wl[l];                  // DEB0 (Rad0.f90:34)
        }
        int rc = rad_prepare(h, a);
        if (rc) return rc;
    }
    cudaStream_t st = h->stream;
    int rc;
    if (h->params.gas_model) {
        if (h->gas.err) CK(cudaMemsetAsync(h->gas.err, 0, sizeof(int), st));
        if ((rc = gas_band(h))) return rc;
        h->rad.gas_aklg = h->gas.aklg;
        h->rad.gas_akls = h->gas.akls;
    } else {
        h->rad.gas_aklg = h->rad.gas_akls = nullptr;
    }
    const RadArgs& a = h->rad;
    const cudaStream_t streams[3] = {st, h->rad_stream[0], h->rad_stream[1]};
    CK(cudaMemsetAsync(a.err, 0, sizeof(int), st));
    const long long nT = 8 * h->gd.CB;
    if (h->prec == GFM_PREC_FP64) {
        if ((rc = launch_rad_transfer<double>(a, h->cd.T, nT, streams, h->rad_ev))) { h->err = "radiation transfer launch"; return rc; }
        launch_cells_to_split(h->gd, a.qe, h->cd.QE, st);
        launch_cells_to_split(h->gd, a.qa, h->cd.QA, st);
    } else {
        if ((rc = launch_rad_transfer<float>(a, h->cf.T, nT, streams, h->rad_ev))) { h->err = "radiation transfer launch"; return rc; }
        launch_cells_to_split(h->gfl, a.qe, h->cf.QE, st);
        launch_cells_to_split(h->gfl, a.qa, h->cf.QA, st);
    }
    const int parts = a.part_base[3];
    std::vector<double> tot(8 * (size_t)parts), akp(2 * (size_t)a.akl_blocks), qep(2 * (size_t)a.akl_blocks);
    int err = 0;
    CK(cudaMemcpyAsync(tot.data(), a.tot_part, tot.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(akp.data(), a.akl_part, akp.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(qep.data(), a.qe_part, qep.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&err, a.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (err) {
        h->err = "radiation transfer: a wall-corner split inside the box (geometry outside the supported set)";
        return GFM_E_UNSUPPORTED;
    }
    if ((rc = gas_check(h))) return rc;
    h->rad_active = 1;
    if (h->wall_on) {
        // the wall exchange of QRNF (Qrn.f90:209-211)
        rc = h->prec == GFM_PREC_FP64 ? wall_exchange<double>(h, h->cd, &h->wall_last)
                                      : wall_exchange<float>(h, h->cf, &h->wall_last);
        if (rc) return rc;
    }
    if (out) {
        std::memset(out, 0, sizeof *out);
        for (int b = 0; b < parts; ++b) {   // x-, y-, z-direction CTAs, each in CTA order
            out->qa_sum_to_melt += tot[8 * b + 0];
            out->qa_sum_to_exit += tot[8 * b + 1];
            out->qa_sum_to_inlet += tot[8 * b + 2];
            out->qa_sum_to_wall += tot[8 * b + 3];
            out->qa_sum_to_open += tot[8 * b + 4];
        }
        double ne = 0.0;
        for (int b = 0; b < a.akl_blocks; ++b) {
            out->tot_qe_h2o_co2 += akp[2 * b];
            out->tot_qe_soot += akp[2 * b + 1];
            out->qe_sum_from_open += qep[2 * b];
            ne += qep[2 * b + 1];
        }
        out->n_emitters = (int)ne;
    }
    return GFM_OK;
}

extern "C" int gfm_gpu_rad_emission(gfm_handle* h) {
    if (!h) return GFM_E_ARG;
    int rc = rad_emission_launch(h);
    if (rc) return rc;
    h->rad_active = 1;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return GFM_E_CUDA; }
    return gas_check(h);
}

namespace {
template <typename R>
int adlbl3_user(gfm_handle* h, Ctx<R>& c, AdiScratch<R>* scr, double* xt, const double* ap, const double* const as[6],
                const double* bs, int ib, int ie, int jb, int je, int kb, int ke, int nim) {
    const GeoT<R>& g = c.g;
    cudaStream_t st = h->stream;
    const long long N = h->N;
    // the user system lives in the momentum coefficient arrays and FZ
    auto put = [&](const double* src, R* dst) -> int {
        CK(cudaMemcpyAsync(h->d_stage, src, N * sizeof(double), cudaMemcpyHostToDevice, st));
        launch_to_split(g, h->d_stage, dst, st);
        return GFM_OK;
    };
    int rc;
    if ((rc = put(xt, c.FZ)) || (rc = put(ap, c.APm)) || (rc = put(bs, c.BSm))) return rc;
    for (int q = 0; q < 6; ++q) if ((rc = put(as[q], c.ASm[q]))) return rc;
    Sys<R> s = sys_of<R>(c.FZ, c.APm, c.ASm, c.BSm, ib, ie, jb, je, kb, ke, nim);
    launch_adlbl3_scr(g, &s, scr, 1, h->adi_mode, st, h->rb_flags);
    launch_from_split(g, c.FZ, h->d_stage, st);
    CK(cudaMemcpyAsync(xt, h->d_stage, N * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return GFM_OK;
}
}  // namespace

extern "C" int gfm_gpu_adlbl3(gfm_handle* h, double* xt, const double* ap, const double* const as[6], const double* bs,
                              int ib, int ie, int jb, int je, int kb, int ke, int nim) {
    if (!h || !xt || !ap || !as || !bs || nim < 0) return GFM_E_ARG;
    for (int q = 0; q < 6; ++q) if (!as[q]) return GFM_E_ARG;
    const HostGrid& g = h->hg;
    if (((ib ^ ie) & 1) || ((jb ^ je) & 1) || ((kb ^ ke) & 1) || ib < 3 || jb < 3 || kb < 3 || ie > g.MP - 2 || je > g.NP - 2 ||
        ke > g.LP - 2 || ie < ib || je < jb || ke < kb)
        return GFM_E_ARG;
    return h->prec == GFM_PREC_FP64 ? adlbl3_user(h, h->cd, h->scr_d, xt, ap, as, bs, ib, ie, jb, je, kb, ke, nim)
                                    : adlbl3_user(h, h->cf, h->scr_f, xt, ap, as, bs, ib, ie, jb, je, kb, ke, nim);
}

namespace {
template <typename R>
int pcorr_sample(gfm_handle* h, Ctx<R>& c, AdiScratch<R>* scr, int nsweeps, void* feats, float* target) {
    const GeoT<R>& g = c.g;
    cudaStream_t st = h->stream;
    const int nx = g.MP / 2 - 2, ny = g.NP / 2 - 2, nz = g.LP / 2 - 2;
    launch_lp_features(c, feats, nx, ny, nz, st);
    CK(cudaMemsetAsync(c.DPc, 0, sizeof(R) * h->CB, st));
    R* asc[6];
    for (int q = 0; q < 6; ++q) asc[q] = c.ASc[q];
    Sys<R> s = sys_of<R>(c.DPc, c.APc, asc, c.BSq, 4, g.MPM2, g.NJY1, g.NJY2, g.LKZ1, g.LKZ2, nsweeps);
    launch_adlbl3_scr(g, &s, scr, 1, h->adi_mode, st, h->rb_flags);
    launch_lp_target(c, c.DPc, target, nx, ny, nz, st);
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    return GFM_OK;
}
bool on_this_device(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    int dev = -1;
    cudaGetDevice(&dev);
    return a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev);
}
}  // namespace

extern "C" int gfm_gpu_pcorr_sample(gfm_handle* h, int nsweeps, void* feats, float* target, int* dims) {
    if (!h || !feats || !target || nsweeps < 0) return GFM_E_ARG;
    const HostGrid& g = h->hg;
    const int nx = g.MP / 2 - 2, ny = g.NP / 2 - 2, nz = g.LP / 2 - 2;
    if (dims) { dims[0] = nx; dims[1] = ny; dims[2] = nz; }
    if (!on_this_device(feats) || !on_this_device(target)) { h->err = "pcorr_sample: buffers must be device memory"; return GFM_E_ARG; }
    return h->prec == GFM_PREC_FP64 ? pcorr_sample(h, h->cd, h->scr_d, nsweeps, feats, target)
                                    : pcorr_sample(h, h->cf, h->scr_f, nsweeps, feats, target);
}

extern "C" int gfm_gpu_set_lp(gfm_handle* h, gfm_lp* lp) {
    if (!h) return GFM_E_ARG;
    gfm::lp::Net* n = reinterpret_cast<gfm::lp::Net*>(lp);
    const int nx = h->hg.MP / 2 - 2, ny = h->hg.NP / 2 - 2, nz = h->hg.LP / 2 - 2;
    if (n) {
        int rc = n->check_dims(nx, ny, nz);
        if (rc != GFM_OK) { h->err = "set_lp: the network's grid is smaller than the p' solve range, or an extent is odd"; return rc; }
        if (!h->lp_feats || (long long)h->lp_nx * h->lp_ny * h->lp_nz < (long long)nx * ny * nz) {
            uint16_t* f = nullptr;
            int r2 = dalloc(h, &f, (long long)nx * ny * nz * 16);
            if (r2) return r2;
            h->lp_feats = f;
        }
        h->lp_nx = nx; h->lp_ny = ny; h->lp_nz = nz;
    }
    h->lp = n;
    // the captured iteration changes: capture again at the next gfm_gpu_gflow
    if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; }
    if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
    return GFM_OK;
}

extern "C" int gfm_gpu_kernel_times(gfm_handle* h, double* adi_ms, double* assemble_ms, double* other_ms, long long* launches) {
    if (!h) return GFM_E_ARG;
    if (adi_ms) *adi_ms = h->adi_ms;
    if (assemble_ms) *assemble_ms = h->asm_ms;
    if (other_ms) *other_ms = h->other_ms;
    if (launches) *launches = h->launches;
    return GFM_OK;
}
extern "C" int gfm_gpu_reset_kernel_times(gfm_handle* h) {
    if (!h) return GFM_E_ARG;
    h->adi_ms = h->asm_ms = h->other_ms = 0;
    h->launches = 0;
    return GFM_OK;
}
extern "C" int gfm_gpu_iteration_profile(gfm_handle* h, long long* kernels_per_iter, long long* adi_kernels_per_iter,
                                         double* adi_cell_visits_per_iter) {
    if (!h) return GFM_E_ARG;
    if (kernels_per_iter) *kernels_per_iter = h->kernels_per_iter;
    if (adi_kernels_per_iter) *adi_kernels_per_iter = h->adi_kernels_per_iter;
    if (adi_cell_visits_per_iter) *adi_cell_visits_per_iter = h->adi_cells_visits;
    return GFM_OK;
}
extern "C" const char* gfm_gpu_last_error(gfm_handle* h) { return h ? h->err.c_str() : g_create_err.c_str(); }

extern "C" void gfm_gpu_destroy(gfm_handle* h);
extern "C" void gfm_gpu_destroy(gfm_handle* h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (void* p : h->allocs) cudaFree(p);
    if (h->h_scal) cudaFreeHost(h->h_scal);
    if (h->h_flags) cudaFreeHost(h->h_flags);
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    for (int q = 0; q < 16; ++q) if (h->ev[q]) cudaEventDestroy(h->ev[q]);
    if (h->ev_g0) cudaEventDestroy(h->ev_g0);
    if (h->ev_g1) cudaEventDestroy(h->ev_g1);
    if (h->ev_adi0) cudaEventDestroy(h->ev_adi0);
    if (h->ev_adi1) cudaEventDestroy(h->ev_adi1);
    for (int i = 0; i <= kXferSlots; ++i) if (h->ev_xfer[i]) cudaEventDestroy(h->ev_xfer[i]);
    for (int e = 0; e < 3; ++e) if (h->rad_ev[e]) cudaEventDestroy(h->rad_ev[e]);
    for (int q = 0; q < 2; ++q) if (h->rad_stream[q]) { cudaStreamSynchronize(h->rad_stream[q]); cudaStreamDestroy(h->rad_stream[q]); }
    for (int s = 0; s < kXferStreams; ++s)
        if (h->copy_stream[s]) { cudaStreamSynchronize(h->copy_stream[s]); cudaStreamDestroy(h->copy_stream[s]); }
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}
