// rad.cu -- volume radiation transfer on the device: the volume part of
// RAD_EMIS (combustion/Code/Rad_emis.f90:120-377).
//
//   k_rad_mark    wall markers: IBCELL 1 -> 101..311 where a neighbour is open
//                 (Rad_emis.f90:144-178), on a cell map of its own
//   k_rad_akl     RAD0 with ID_RAD=10 (Rad0.f90:112-166): AKL = EMF(AKL0, OPL)
//                 of the hot open cells, band-emission totals, and QREF's
//                 per-area band emission QEL0 of every emitter
//   k_rad_qe      QE of every emitter (QREF's six face powers and band sum)
//   k_rad_trace   the QRNF emitter loop (Qrn.f90:58-154) with the x-, y- or
//                 z-flux of QREF (Qre.f90:31-515) and QRTX/QRTY/QRTZ
//                 (Qrtx.f90:15-209, Qrty.f90:9-224, Qrtz.f90:15-234): one
//                 launch per direction, the three on three streams at once
//   k_rad_reduce  QAL summed over the CTAs, QA = sum over bands (QRN1,
//                 Qrn.f90:250-259)
//
// A CTA of direction d traces that direction for one emitter at a time (cells
// in the reference's loop order, a grid-stride over the emitters); emitters
// and directions are independent, so many are in flight at once, each
// direction's CTAs sized by its own slab.  Within one emitter and direction
// the reference is sequential; the CTA keeps its order where it matters:
//   * the slab arrays QTX1, QTX2, Q2M and their flags live in shared memory
//     (global scratch when they do not fit);
//   * the far-face angles of a slab (SANG2), the reference's outward scan
//     with its early exit, are run by one thread per transverse axis;
//   * the spread across the first transverse axis (part 1 of QRTX/Y/Z) touches
//     only its own row of the slab arrays: one thread per row, the reference's
//     order inside the row;
//   * the spread across the second transverse axis (part 2) touches only its
//     own column, except for the wall-corner split, which also adds into the
//     neighbouring column toward the emitter (on the emitter's own column,
//     into the column the spread's loop variable last held: two past the last
//     column below the emitter that split, else where the slab's last part-1
//     spread ended).  The first column runs alone, then the interior columns
//     in parallel, then the last column.  The interior columns' splits into
//     other columns are listed and added after the interior phase, in the
//     reference's column order; in a box only the first and the last column
//     split, so every slab-array element receives its additions in the
//     reference's order, and with obstacles (ports, a stepped crown) the
//     listed additions are associated differently by a few roundings.  A
//     list that overflows or a target outside the slab is reported as
//     unsupported;
//   * absorption into the slab's cells is per cell.
// QAL is accumulated per CTA in its own copy (fixed emitter order) and the
// copies are summed in a fixed order (x-direction CTAs, then y, then z), so
// the result is deterministic; it differs from the reference's single running
// sum only by the association of the additions.
//
// Angles come from rad_atand, the same operations as the oracle's ATAND; this
// translation unit is compiled with --fmad=false so that no multiply-add is
// fused where the reference rounds twice, and angle ties break the same way.
#include "state.cuh"

namespace gfm {
namespace {

constexpr double kSmall16 = 1.0e-16;

// A double's IEEE bit pattern as a signed 64-bit integer.  Two non-negative
// doubles, or any double and a positive one, compare the same way as these
// integers (no NaN occurs here), so the frequent comparisons of angles and of
// powers against SMALL16 run on the integer pipe, GB300's FP64 pipe being
// narrow; the results are those of the floating-point comparisons.
__device__ __forceinline__ long long rb(double x) { return __double_as_longlong(x); }
constexpr double kTgMn = 300.0;     // TG_MN (Rad0.f90:42)
constexpr int kRadThreads = 128;

// atan(x) in degrees: reduction to [0,1] by atan(x) = pi/2 - atan(1/x), to
// [0, tan(pi/12)] by atan(a) = pi/6 + atan((a*sqrt(3)-1)/(a+sqrt(3)))
// (Abramowitz & Stegun 4.4.34), Maclaurin series to t^29 (A&S 4.4.42) by
// Horner's rule in t^2 with fused multiply-adds.
__device__ double rad_atand(double x) {
    const double PI = 3.14159265358979323846;
    const double SQRT3 = 1.73205080756887729353;
    const double TAN_PI_12 = 0.26794919243112270647;
    double a = fabs(x);
    const bool inv = a > 1.0;
    if (inv) a = 1.0 / a;
    const bool sh = a > TAN_PI_12;
    if (sh) a = (a * SQRT3 - 1.0) / (a + SQRT3);
    const double z = a * a;
    double p = 1.0 / 29.0;
#pragma unroll
    for (int n = 13; n >= 0; --n) p = fma(p, z, ((n & 1) ? -1.0 : 1.0) / (double)(2 * n + 1));
    double r = a * p;
    if (sh) r = PI / 6.0 + r;
    if (inv) r = PI / 2.0 - r;
    const double d = r * (180.0 / PI);
    return x < 0.0 ? -d : d;
}

__global__ void k_rad_mark(RadArgs a) {
    const int n = a.MZ * a.NZ * a.LZ;
    GFM_FOR(c, n) {
        const int I = 2 * (c % a.MZ + 1), J = 2 * ((c / a.MZ) % a.NZ + 1), K = 2 * (c / (a.MZ * a.NZ) + 1);
        auto ibc = [&](int i, int j, int k) { return (int)a.g.ib[pidx(a.g, i, j, k)]; };
        int v = ibc(I, J, K);
        if (v == 1) {
            const int KM2 = max(K - 2, 2), KP2 = min(K + 2, a.LP);
            const int JM2 = max(J - 2, 2), JP2 = min(J + 2, a.NP);
            const int IM2 = max(I - 2, 2), IP2 = min(I + 2, a.MP);
            if (ibc(I, J, KM2) <= 0) v = 301;
            else if (ibc(I, J, KP2) <= 0) v = 311;
            else if (ibc(I, JM2, K) <= 0) v = 201;
            else if (ibc(I, JP2, K) <= 0) v = 211;
            else if (ibc(IM2, J, K) <= 0) v = 101;
            else if (ibc(IP2, J, K) <= 0) v = 111;
        }
        a.ibr[c] = (int16_t)v;
    }
}

__device__ void rad_debx(const RadArgs& a, double t, double* deb) {   // DEBX, Rad_fun.f90:83-101
    double eb0 = 0.0;
    for (int l = 1; l <= a.NWL - 1; ++l) {
        const double x1 = a.deb0[l - 1] / t;
        const double eb1 = rif3(x1);
        deb[l - 1] = eb1 - eb0;
        if (deb[l - 1] <= 1.0e-3) deb[l - 1] = 0.0; else eb0 = eb1;
    }
    deb[a.NWL - 1] = 1.0 - eb0;
}

// RAD0 (ID_RAD=10): AKL = EMF(AKLG + AKLS) from the band model (gas.cu), or
// from the gray bands (AKLG = AKL0, AKLS = 0).  Also the cell
// temperature in kelvin (T*T0), the one the transfer reads, and for every
// emitter (open, T > TG_MN) QREF's emission per unit area of each band,
// QEL0 = DEB*AKL*SGN*T^4 (Qre.f90:80-86), with the same DEB.  Block partials
// of the two band-emission totals are summed on the host in block order.
template <typename R>
__global__ void __launch_bounds__(256) k_rad_akl(RadArgs a, const R* __restrict__ T) {
    __shared__ double sh[2][256];
    const int n = a.MZ * a.NZ * a.LZ;
    double sg_tot = 0.0, ss_tot = 0.0;
    GFM_FOR(c, n) {
        const int I = 2 * (c % a.MZ + 1), J = 2 * ((c / a.MZ) % a.NZ + 1), K = 2 * (c / (a.MZ * a.NZ) + 1);
        const double t = (double)T[pidx(a.g, I, J, K)] * a.t0;
        a.tcell[c] = t;
        for (int l = 0; l < a.NWL; ++l) { a.akl[c + (long long)l * n] = 0.0; a.qel0[c + (long long)l * n] = 0.0; }
        if (!(a.ibr[c] <= 0 && t >= kTgMn)) continue;
        const double dx = a.g.DX[I], dr = a.g.DR[J], dz = a.g.DZ[K];
        double vol = dx * dr * a.g.RS[J] * dz;                        // VOL_C at a cell centre (VOL_C0)
        if (a.g.HALF && a.ibr[c] <= -1) vol = vol * a.g.BVF[-a.ibr[c] - 1];
        const double sa = ((dx * dr) + (dr * dz) + (dx * dz)) * 2.0;
        if (sa <= kSmall16) continue;
        const double opl = 6.0 * vol / sa;
        if (opl <= 1.0e-10) continue;
        double deb[kRadMaxBands];
        rad_debx(a, t, deb);
        const double t2 = t * t;
        const double area_sgn_t4 = sa * a.sgn * (t2 * t2);
        double sg = 0.0, ss = 0.0;
        const bool emitter = t > kTgMn;
        const double g0 = a.sgn * (t2 * t2);
        for (int l = 0; l < a.NWL; ++l) {
            const long long cl = c + (long long)l * n;
            const double ag = a.gas_aklg ? a.gas_aklg[cl] : a.akl0[l];
            const double as = a.gas_aklg ? a.gas_akls[cl] : 0.0;
            const double akl = emf(a.gas_aklg ? ag + as : a.akl0[l], opl);
            a.akl[cl] = akl;
            if (emitter) a.qel0[cl] = deb[l] * akl * g0;
            sg = sg + deb[l] * emf(ag, opl);
            ss = ss + deb[l] * emf(as, opl);
        }
        sg_tot += area_sgn_t4 * sg;
        ss_tot += area_sgn_t4 * ss;
    }
    sh[0][threadIdx.x] = sg_tot;
    sh[1][threadIdx.x] = ss_tot;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) { sh[0][threadIdx.x] += sh[0][threadIdx.x + s]; sh[1][threadIdx.x] += sh[1][threadIdx.x + s]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { a.akl_part[2 * blockIdx.x] = sh[0][0]; a.akl_part[2 * blockIdx.x + 1] = sh[1][0]; }
}

// One march direction of QREF: d = slab axis, u = first transverse axis (the
// part-1 spread, the part-2 columns), v = second (the part-1 rows, the part-2
// spread).  x-flux: u = y, v = z (QRTX); y-flux: u = x, v = z (QRTY); z-flux:
// u = x, v = y (QRTZ).  Slab arrays are indexed e = (v/2-1)*DA + (u/2-1).
struct Dir {
    int d, u, v;
    int Dd, Du, Dv, DA, DB, A;
    int d0, u0, v0;
    int sd, su, sv;              // cell-index strides of the three axes
    const double *cd, *cu, *cv;  // coordinates (shared-memory copies, 1-based)
    double *angU1, *angU2, *angV1, *angV2;   // ANG(.,1), ANG(.,2) of u and v (1-based)
    int direct1, direct2;        // IBCELL codes deposited whole in part 2 (and 4)
};

struct Slab {   // scratch of one CTA
    double *q1, *q2, *qm;        // QTX1, QTX2, Q2M: [l*A + e]
    unsigned char *f1, *f2, *fm; // IQT1, IQT2, IQTM
    int16_t* ib;                 // IBCELL (with wall markers) of the current slab's cells: [e]
    double *tU, *tV;             // far-face angle candidates of the current slab (1-based positions)
};

// Corner-split additions of the interior columns into other columns,
// gathered during the parallel part 2 of one slab: capc entries per column in
// the CTA's global scratch, in the column's own order; and, in shared
// memory, the two values that decide the emitter column's target.
struct SplitList {
    int* any;                    // an interior column listed a split in this slab
    int* maxbelow;               // largest column below the emitter that split (0: none)
    unsigned long long* last1;   // (row << 32) | (u2 + 8) of the slab's last part-1 spread
    int* cnt;                    // [column]: entries used (zero between slabs)
    int* meta;                   // [column][entry][3]: target row, target column (-1: emitter's), band mask
    double* q;                   // [column][entry][band]
    int capc, nw;
};

__device__ __forceinline__ bool rad_corner(int d, int ibc1) {
    return d == 0 ? ibc1 > 100 : (d == 1 ? ibc1 >= 100 : ibc1 > 1);
}

template <int NW>
__device__ void part1_row(const RadArgs& a, const Dir& D, const Slab& S, int slab, int v1, double ang0u,
                          const SplitList& SL) {
    const int NWL = NW > 0 ? NW : a.NWL;
    double Q11[NW > 0 ? NW : kRadMaxBands], Q12[NW > 0 ? NW : kRadMaxBands];
    const int bb = v1 / 2;
    int last_u2 = 0;
    bool spread = false;
    for (int UPM = -2; UPM <= 2; UPM += 4) {
        double A11 = 0.0, A12 = 0.0;
        const int uend = UPM < 0 ? 2 : D.Du;
        for (int u1 = D.u0; UPM > 0 ? u1 <= uend - UPM : u1 >= uend - UPM; u1 += UPM) {
            if (rb(A11) >= rb(ang0u)) break;
            const int u12 = u1 + UPM / 2;
            A12 = D.angU1[u12];
            const double DANG = A12 - A11;
            if (DANG <= 1.0e-10) { A11 = A12; continue; }
            double A21 = A11;
            const int e = (bb - 1) * D.DA + (u1 / 2 - 1);
            if (S.f1[e]) { A11 = A12; continue; }
            if (u1 == D.u0) {
                for (int l = 0; l < NWL; ++l) Q11[l] = S.q1[l * D.A + e] * 0.5;
                if (UPM > 0) for (int l = 0; l < NWL; ++l) S.q1[l * D.A + e] = 0.0;
            } else {
                for (int l = 0; l < NWL; ++l) { Q11[l] = S.q1[l * D.A + e]; S.q1[l * D.A + e] = 0.0; }
            }
            if (u1 != D.u0 || UPM > 0) S.f1[e] = 1;
            for (int l = 0; l < NWL; ++l) Q12[l] = Q11[l];
            int u2 = u1;
            for (; UPM > 0 ? u2 <= uend : u2 >= uend; u2 += UPM) {
                const int e2 = (bb - 1) * D.DA + (u2 / 2 - 1);
                if (S.ib[e2] < 1) {
                    const double A22 = D.angU2[u2 + UPM / 2];
                    if (rb(A22) <= rb(A21)) continue;
                    if (rb(A22) < rb(A12)) {
                        const double FIJ = (A22 - A21) / DANG;
                        for (int l = 0; l < NWL; ++l) {
                            if (rb(Q11[l]) < rb(kSmall16)) continue;
                            const double Q21 = Q11[l] * FIJ;
                            S.qm[l * D.A + e2] = S.qm[l * D.A + e2] + Q21;
                            Q12[l] = Q12[l] - Q21;
                        }
                        S.fm[e2] = 0;
                        A21 = A22;
                        continue;
                    }
                }
                for (int l = 0; l < NWL; ++l) S.qm[l * D.A + e2] = S.qm[l * D.A + e2] + Q12[l];
                S.fm[e2] = 0;
                break;
            }
            last_u2 = u2;   // the loop variable as the loop leaves it
            spread = true;
            A11 = A12;
        }
    }
    // rows run in parallel: the reference's last spread is the highest row's
    if (spread) atomicMax(SL.last1, ((unsigned long long)v1 << 32) | (unsigned)(last_u2 + 8));
}

template <int NW>
__device__ void part2_col(const RadArgs& a, const Dir& D, const Slab& S, int slab, int u1, double ang0v, int* err,
                          const SplitList& SL) {
    const int NWL = NW > 0 ? NW : a.NWL;
    double Q11[NW > 0 ? NW : kRadMaxBands], Q12[NW > 0 ? NW : kRadMaxBands];
    const int aa = u1 / 2;
    const bool edge = u1 == 2 || u1 == D.Du;
    for (int KM = -2; KM <= 2; KM += 4) {
        double A11 = 0.0, A12 = 0.0;
        const int vend = KM < 0 ? 2 : D.Dv;
        for (int v1 = D.v0; KM > 0 ? v1 <= vend - KM : v1 >= vend - KM; v1 += KM) {
            if (rb(A11) >= rb(ang0v)) break;
            const int v12 = v1 + KM / 2;
            A12 = D.angV1[v12];
            const double DANG = A12 - A11;
            if (DANG <= 1.0e-10) { A11 = A12; continue; }
            double A21 = A11;
            const int e = (v1 / 2 - 1) * D.DA + (aa - 1);
            if (S.fm[e]) { A11 = A12; continue; }
            if (v1 == D.v0) {
                for (int l = 0; l < NWL; ++l) Q11[l] = S.qm[l * D.A + e] * 0.5;
                if (KM > 0) for (int l = 0; l < NWL; ++l) S.qm[l * D.A + e] = 0.0;
            } else {
                for (int l = 0; l < NWL; ++l) { Q11[l] = S.qm[l * D.A + e]; S.qm[l * D.A + e] = 0.0; }
            }
            if (v1 != D.v0 || KM > 0) S.fm[e] = 1;
            const int ibc1 = S.ib[e];
            if (ibc1 == D.direct1 || ibc1 == D.direct2 || ibc1 == 4) {
                for (int l = 0; l < NWL; ++l) S.q2[l * D.A + e] = S.q2[l * D.A + e] + Q11[l];
                S.f2[e] = 0;
                A11 = A12;
                continue;
            }
            for (int l = 0; l < NWL; ++l) Q12[l] = Q11[l];
            for (int v2 = v1; KM > 0 ? v2 <= vend : v2 >= vend; v2 += KM) {
                const int v2m = v2 + KM / 2;
                const int e2 = (v2 / 2 - 1) * D.DA + (aa - 1);
                const int ibc2 = S.ib[e2];
                bool to330 = ibc1 <= 0 && ibc2 >= 1;
                if (!to330) {
                    if (rad_corner(D.d, ibc1) && ibc2 == 1) {
                        // half into the neighbouring column toward the emitter
                        // (the emitter's own column: resolved after the
                        // interior phase), half into this column's previous row
                        const int ut = u1 < D.u0 ? u1 + 2 : (u1 > D.u0 ? u1 - 2 : -1);
                        if (u1 < D.u0) atomicMax(SL.maxbelow, u1);
                        const int e2m = (v2 / 2 - KM / 2 - 1) * D.DA + (aa - 1);
                        if (edge) {
                            const int et = (v2 / 2 - 1) * D.DA + (ut / 2 - 1);
                            for (int l = 0; l < NWL; ++l) {
                                if (rb(Q12[l]) < rb(kSmall16)) continue;
                                const double Q21 = Q12[l] * 0.5;
                                S.q2[l * D.A + et] = S.q2[l * D.A + et] + Q21;
                                S.q2[l * D.A + e2m] = S.q2[l * D.A + e2m] + Q21;
                            }
                            S.f2[et] = 0;
                        } else {
                            // only this column's thread writes its entries
                            const int k = SL.cnt[aa - 1];
                            const long long ent = (long long)(aa - 1) * SL.capc + k;
                            unsigned msk = 0;
                            for (int l = 0; l < NWL; ++l) {
                                if (rb(Q12[l]) < rb(kSmall16)) continue;
                                const double Q21 = Q12[l] * 0.5;
                                if (k < SL.capc) SL.q[ent * SL.nw + l] = Q21;
                                msk |= 1u << l;
                                S.q2[l * D.A + e2m] = S.q2[l * D.A + e2m] + Q21;
                            }
                            *SL.any = 1;
                            if (k < SL.capc) {
                                SL.meta[3 * ent] = v2;
                                SL.meta[3 * ent + 1] = ut;
                                SL.meta[3 * ent + 2] = (int)msk;
                                SL.cnt[aa - 1] = k + 1;
                            } else {
                                atomicOr(err, 1);   // more splits in one column than the list holds
                            }
                        }
                        S.f2[e2m] = 0;
                        break;
                    }
                    if (v2m > D.Dv || v2m < 2) {
                        to330 = true;
                    } else {
                        const double A22 = D.angV2[v2m];
                        if ((A22 - A21) <= 1.0e-10) continue;
                        if (rb(A22) < rb(A12)) {
                            const double FIJ = (A22 - A21) / DANG;
                            for (int l = 0; l < NWL; ++l) {
                                if (rb(Q11[l]) < rb(kSmall16)) continue;
                                const double Q21 = Q11[l] * FIJ;
                                S.q2[l * D.A + e2] = S.q2[l * D.A + e2] + Q21;
                                Q12[l] = Q12[l] - Q21;
                            }
                            S.f2[e2] = 0;
                            A21 = A22;
                            continue;
                        }
                    }
                }
                for (int l = 0; l < NWL; ++l) S.q2[l * D.A + e2] = S.q2[l * D.A + e2] + Q12[l];
                S.f2[e2] = 0;
                break;
            }
            A11 = A12;
        }
    }
}

// The listed splits of the interior columns, in the reference's column order
// (and, within a column, its order); the emitter column's target is two past
// the last column below the emitter that split, else where the slab's last
// part-1 spread ended.  One thread.
__device__ void rad_apply_splits(const RadArgs& a, const Dir& D, const Slab& S, const SplitList& SL, int* err) {
    const int NWL = a.NWL;
    int tgt_emitter = -1;
    if (*SL.maxbelow >= 2) tgt_emitter = *SL.maxbelow + 2;
    else if (*SL.last1 != 0ull) tgt_emitter = (int)(unsigned)(*SL.last1 & 0xffffffffull) - 8;
    for (int c = 1; c <= D.DA; ++c) {   // source columns 2, 4, .. in the reference's order
        const int m = SL.cnt[c - 1];
        if (m == 0) continue;
        SL.cnt[c - 1] = 0;
        for (int k = 0; k < (m < SL.capc ? m : SL.capc); ++k) {
            const long long ent = (long long)(c - 1) * SL.capc + k;
            const int row = SL.meta[3 * ent];
            const int col = SL.meta[3 * ent + 1] >= 0 ? SL.meta[3 * ent + 1] : tgt_emitter;
            const unsigned msk = (unsigned)SL.meta[3 * ent + 2];
            if (col < 2 || col > D.Du || (col & 1) || row < 2 || row > D.Dv) { atomicOr(err, 1); continue; }
            const int et = (row / 2 - 1) * D.DA + (col / 2 - 1);
            for (int l = 0; l < NWL; ++l)
                if (msk & (1u << l)) S.q2[l * D.A + et] = S.q2[l * D.A + et] + SL.q[ent * SL.nw + l];
            S.f2[et] = 0;
        }
    }
}

// Is row v1 (part 1) / column u1 (part 2) visited?  The reference skips the
// rows before the emitter whose near angle is outside the cone and stops at
// the first row after it whose near angle is; `exit` is that row (or beyond
// the range), found once per slab.
__device__ __forceinline__ bool rad_visit(const double* ang2, int p, int p0, double ang0, int exit) {
    if (p < p0) return rb(ang2[p + 1]) < rb(ang0);
    return p < exit;
}
__device__ int rad_exit(const double* ang2, int p0, int last, double ang0) {
    for (int q = p0 + 2; q <= last; q += 2)
        if (rb(ang2[q - 1]) >= rb(ang0)) return q;
    return last + 2;
}

struct RadAcc {   // per-thread sums of the deposits by destination
    double melt, exit, inlet, wall, open;
};

template <int NW>
__device__ void rad_direction(const RadArgs& a, Dir& D, const Slab& S, double* qalp, const double* qel1,
                              double* ang0, RadAcc& acc, int* err, const SplitList& SL) {
    const int NWL = NW > 0 ? NW : a.NWL;
    const int n = a.MZ * a.NZ * a.LZ;
    const int tid = threadIdx.x, nth = blockDim.x;
    // ALLOCATE and initialise the slab arrays of this direction
    for (int i = tid; i < D.A * NWL; i += nth) { S.q1[i] = 0.0; S.q2[i] = 0.0; S.qm[i] = 0.0; }
    for (int i = tid; i < D.A; i += nth) { S.f1[i] = 1; S.f2[i] = 1; S.fm[i] = 1; }
    __syncthreads();
    const int e0 = (D.v0 / 2 - 1) * D.DA + (D.u0 / 2 - 1);
    __shared__ int exits[2];
    for (int s = -1; s <= 1; s += 2) {
        if (tid == 0) {
            for (int l = 0; l < NWL; ++l) S.q1[l * D.A + e0] = qel1[l];
            S.f1[e0] = 0;
            // SANG1 for an open cell
            const double b = fabs(D.cd[D.d0 + s] - D.cd[D.d0]);
            if (b < kSmall16) { ang0[0] = 90.0; ang0[1] = 90.0; }
            else {
                ang0[0] = rad_atand(fabs(D.cu[D.u0 + s] - D.cu[D.u0]) / b);
                ang0[1] = rad_atand(fabs(D.cv[D.v0 + s] - D.cv[D.v0]) / b);
            }
        }
        __syncthreads();
        const double ang0u = ang0[0], ang0v = ang0[1];
        for (int p = 1 + tid; p <= D.Du; p += nth) { D.angU1[p] = ang0u; D.angU2[p] = ang0u; }
        for (int p = 1 + tid; p <= D.Dv; p += nth) { D.angV1[p] = ang0v; D.angV2[p] = ang0v; }
        __syncthreads();
        if (tid == 0) { D.angU1[D.u0] = 0.0; D.angU2[D.u0] = 0.0; D.angV1[D.v0] = 0.0; D.angV2[D.v0] = 0.0; }
        __syncthreads();
        const int dend = s < 0 ? 2 : D.Dd;
        for (int slab = D.d0 + 2 * s; s > 0 ? slab <= dend : slab >= dend; slab += 2 * s) {
            // the slab's IBCELL codes, and SANG2: the far-face angles of every
            // transverse face in parallel, then the reference's outward scan
            // with its early exit, one thread per transverse axis
            int far = slab + s;
            far = min(far, D.Dd);
            const double b = fabs(D.cd[far] - D.cd[D.d0]);
            for (int e = tid; e < D.A; e += nth)
                S.ib[e] = a.ibr[(slab / 2 - 1) * D.sd + (e % D.DA) * D.su + (e / D.DA) * D.sv];
            {
                const int nu = D.Du / 2, nv = D.Dv / 2;   // odd positions 1 .. Du-1 and 1 .. Dv-1
                for (int i = tid; i < nu + nv; i += nth) {
                    const bool isu = i < nu;
                    const int pp = 2 * (isu ? i : i - nu) + 1;
                    const double* c = isu ? D.cu : D.cv;
                    const int p0 = isu ? D.u0 : D.v0;
                    (isu ? S.tU : S.tV)[pp] = b < kSmall16 ? 90.0 : rad_atand(fabs(c[pp] - c[p0]) / b);
                }
            }
            __syncthreads();
            if (tid == 0) { *SL.any = 0; *SL.maxbelow = 0; *SL.last1 = 0ull; }
            if (tid == 0 || tid == 32) {
                const bool isu = tid == 0;
                const int P = isu ? D.Du : D.Dv, p0 = isu ? D.u0 : D.v0;
                const double* cand = isu ? S.tU : S.tV;
                double* out = isu ? D.angU2 : D.angV2;
                const double lim = isu ? ang0u : ang0v;
                for (int M = -1; M <= 1; M += 2) {
                    const int pend = M < 0 ? 2 : P;
                    for (int pp = p0 + M; M > 0 ? pp <= pend : pp >= pend; pp += 2 * M) {
                        const double aa = cand[pp];
                        if (rb(aa) >= rb(lim)) break;
                        out[pp] = aa;
                    }
                }
                // the first part-2 column (u) / part-1 row (v) after the emitter that ends its loop
                exits[isu ? 0 : 1] = isu ? rad_exit(out, p0, P, lim) : rad_exit(out, p0, P - 2, lim);
            }
            __syncthreads();
            // part 1: one thread per row
            {
                const int nrows = (D.Dv - 4) / 2;   // rows 4 .. Dv-2
                for (int r = tid; r < nrows; r += nth) {
                    const int v1 = 4 + 2 * r;
                    if (rad_visit(D.angV2, v1, D.v0, ang0v, exits[1])) part1_row<NW>(a, D, S, slab, v1, ang0u, SL);
                }
            }
            __syncthreads();
            // part 2: first column, interior columns, last column
            if (tid == 0 && rad_visit(D.angU2, 2, D.u0, ang0u, exits[0])) part2_col<NW>(a, D, S, slab, 2, ang0v, err, SL);
            __syncthreads();
            {
                const int ncols = (D.Du - 4) / 2;   // columns 4 .. Du-2
                for (int r = tid; r < ncols; r += nth) {
                    const int u1 = 4 + 2 * r;
                    if (rad_visit(D.angU2, u1, D.u0, ang0u, exits[0])) part2_col<NW>(a, D, S, slab, u1, ang0v, err, SL);
                }
            }
            __syncthreads();
            if (tid == 0) {
                if (*SL.any) rad_apply_splits(a, D, S, SL, err);
                if (rad_visit(D.angU2, D.Du, D.u0, ang0u, exits[0])) part2_col<NW>(a, D, S, slab, D.Du, ang0v, err, SL);
            }
            __syncthreads();
            // absorption in the slab's cells
            const bool end = slab == dend;
            for (int e = tid; e < D.A; e += nth) {
                if (S.f2[e]) continue;
                const int ua = e % D.DA + 1, vb = e / D.DA + 1;
                const int c = (slab / 2 - 1) * D.sd + (ua - 1) * D.su + (vb - 1) * D.sv;
                const int ib = S.ib[e];
                for (int l = 0; l < NWL; ++l) {
                    const double q = S.q2[l * D.A + e];
                    if (rb(q) < rb(kSmall16)) continue;
                    double* qa = qalp + c + (long long)l * n;
                    if (ib >= 1 || end) {
                        *qa = *qa + q;
                        if (ib == 4) acc.melt += q;
                        else if (ib == 3) acc.exit += q;
                        else if (ib == 2) acc.inlet += q;
                        else acc.wall += q;
                    } else {
                        const double qa0 = q * a.akl[c + (long long)l * n];
                        *qa = *qa + qa0;
                        S.q1[l * D.A + e] = q - qa0;
                        S.f1[e] = 0;
                        acc.open += qa0;
                    }
                    S.q2[l * D.A + e] = 0.0;
                    S.f2[e] = 1;
                }
            }
            __syncthreads();
            for (int p = 1 + tid; p <= D.Du; p += nth) D.angU1[p] = D.angU2[p];
            for (int p = 1 + tid; p <= D.Dv; p += nth) D.angV1[p] = D.angV2[p];
            __syncthreads();
        }
    }
}

// One march direction d of QREF for every emitter of the grid-stride: the
// three directions are independent apart from the order of their QAL
// additions, so they run as three launches at once, each with the shared
// memory of its own slab.
template <int NW>
__global__ void __launch_bounds__(kRadThreads) k_rad_trace(RadArgs a, int d) {
    extern __shared__ __align__(16) unsigned char rad_smem[];
    __shared__ double s_qel1[kRadMaxBands];
    __shared__ double s_ang0[2];
    __shared__ double s_red[kRadThreads];
    __shared__ int s_any, s_maxbelow;
    __shared__ unsigned long long s_last1;
    const int NWL = NW > 0 ? NW : a.NWL;
    const int n = a.MZ * a.NZ * a.LZ;
    const int tid = threadIdx.x;
    Dir D;
    D.d = d;
    D.u = d == 0 ? 1 : 0;
    D.v = d == 2 ? 1 : 2;
    const int dims[3] = {a.MP, a.NP, a.LP};
    D.Dd = dims[d]; D.Du = dims[D.u]; D.Dv = dims[D.v];
    D.DA = D.Du / 2; D.DB = D.Dv / 2; D.A = D.DA * D.DB;
    const int strides[3] = {1, a.MZ, a.MZ * a.NZ};
    D.sd = strides[d]; D.su = strides[D.u]; D.sv = strides[D.v];
    D.direct1 = 100 * (d + 1) + 1; D.direct2 = 100 * (d + 1) + 11;
    // shared layout: coordinates X(1..MP), R(1..NP), Z(1..LP); ANG1/2/3 (two
    // columns each); angle candidates; the slab's IBCELL; then the slab arrays
    // (here or in global scratch)
    double* sx = reinterpret_cast<double*>(rad_smem);
    double* sr = sx + (a.MP + 2);
    double* sz = sr + (a.NP + 2);
    double* ang1 = sz + (a.LP + 2);              // ANG1(.,1), ANG1(.,2)
    double* ang2 = ang1 + 2 * (a.MP + 2);
    double* ang3 = ang2 + 2 * (a.NP + 2);
    double* tmp = ang3 + 2 * (a.LP + 2);         // angle candidates: (MP+2) + (NP+2) + (LP+2)
    int16_t* sib = reinterpret_cast<int16_t*>(tmp + (a.MP + 2) + (a.NP + 2) + (a.LP + 2));
    double* arr = reinterpret_cast<double*>(sib + ((D.A + 7) / 8) * 8);
    {
        const double* crd[3] = {sx, sr, sz};
        double* angs[3] = {ang1, ang2, ang3};
        const int angw[3] = {a.MP + 2, a.NP + 2, a.LP + 2};
        double* tmps[3] = {tmp, tmp + (a.MP + 2), tmp + (a.MP + 2) + (a.NP + 2)};
        D.cd = crd[d]; D.cu = crd[D.u]; D.cv = crd[D.v];
        D.angU1 = angs[D.u]; D.angU2 = angs[D.u] + angw[D.u];
        D.angV1 = angs[D.v]; D.angV2 = angs[D.v] + angw[D.v];
        D.d0 = D.u0 = D.v0 = 0;
        (void)tmps;
    }
    Slab S;
    S.ib = sib;
    {
        double* tmps[3] = {tmp, tmp + (a.MP + 2), tmp + (a.MP + 2) + (a.NP + 2)};
        S.tU = tmps[D.u];
        S.tV = tmps[D.v];
    }
    S.q1 = a.slab_in_smem[d] ? arr : a.scratch[d] + (long long)blockIdx.x * 3 * D.A * NWL;
    S.q2 = S.q1 + (long long)D.A * NWL;
    S.qm = S.q2 + (long long)D.A * NWL;
    unsigned char* flags = a.slab_in_smem[d] ? reinterpret_cast<unsigned char*>(S.qm + (long long)D.A * NWL)
                                             : a.fscratch[d] + (long long)blockIdx.x * 3 * D.A;
    S.f1 = flags;
    S.f2 = flags + D.A;
    S.fm = flags + 2 * D.A;
    const long long cta_cols = (long long)blockIdx.x * D.DA;
    const SplitList SL{&s_any, &s_maxbelow, &s_last1, a.split_cnt[d] + cta_cols,
                       a.split_meta[d] + 3 * cta_cols * a.split_capc[d],
                       a.split_q[d] + cta_cols * a.split_capc[d] * a.NWL, a.split_capc[d], a.NWL};
    for (int e = tid; e < D.DA; e += blockDim.x) SL.cnt[e] = 0;
    for (int i = 1 + tid; i <= a.MP; i += blockDim.x) sx[i] = a.g.X[i];
    for (int i = 1 + tid; i <= a.NP; i += blockDim.x) sr[i] = a.g.Rr[i];
    for (int i = 1 + tid; i <= a.LP; i += blockDim.x) sz[i] = a.g.Z[i];
    const long long part = a.part_base[d] + blockIdx.x;
    double* qalp = a.qal_part + part * n * NWL;
    for (long long i = tid; i < (long long)n * NWL; i += blockDim.x) qalp[i] = 0.0;
    const double* dface[3] = {a.g.DX, a.g.DR, a.g.DZ};
    RadAcc acc{0.0, 0.0, 0.0, 0.0, 0.0};
    __syncthreads();

    for (int c = blockIdx.x; c < n; c += gridDim.x) {
        // emitters in the reference's loop order: I outer, K inner
        const int KD2 = c % a.LZ + 1, JD2 = (c / a.LZ) % a.NZ + 1, ID2 = c / (a.LZ * a.NZ) + 1;
        const int cc = (ID2 - 1) + a.MZ * ((JD2 - 1) + a.NZ * (KD2 - 1));
        if (a.ibr[cc] >= 1 || a.tcell[cc] <= kTgMn) continue;
        const int pos[3] = {2 * ID2, 2 * JD2, 2 * KD2};
        D.d0 = pos[d]; D.u0 = pos[D.u]; D.v0 = pos[D.v];
        if (tid == 0)   // power through one face of the emitter (QEL1, Qre.f90:118/241/384)
            for (int l = 0; l < NWL; ++l)
                s_qel1[l] = a.qel0[cc + (long long)l * n] * dface[D.u][D.u0] * dface[D.v][D.v0];
        __syncthreads();
        rad_direction<NW>(a, D, S, qalp, s_qel1, s_ang0, acc, a.err, SL);
        __syncthreads();
    }
    // block totals in a fixed order
    double vals[5] = {acc.melt, acc.exit, acc.inlet, acc.wall, acc.open};
    for (int k = 0; k < 5; ++k) {
        s_red[tid] = vals[k];
        __syncthreads();
        for (int st = kRadThreads / 2; st > 0; st >>= 1) {
            if (tid < st) s_red[tid] += s_red[tid + st];
            __syncthreads();
        }
        if (tid == 0) a.tot_part[8 * part + k] = s_red[0];
        __syncthreads();
    }
}

// QE of every emitter (QREF's QEL accumulation, Qre.f90:121/244/387, and the
// band sum, Qre.f90:503-507): the six faces' powers in the order x-, x+, y-,
// y+, z-, z+; block totals of the emission and of the emitter count.
__global__ void __launch_bounds__(256) k_rad_qe(RadArgs a) {
    __shared__ double sh[2][256];
    const int n = a.MZ * a.NZ * a.LZ;
    double qs = 0.0, cnt = 0.0;
    GFM_FOR(c, n) {
        a.qe[c] = 0.0;
        if (a.ibr[c] >= 1 || a.tcell[c] <= kTgMn) continue;
        const int I = 2 * (c % a.MZ + 1), J = 2 * ((c / a.MZ) % a.NZ + 1), K = 2 * (c / (a.MZ * a.NZ) + 1);
        double qe = 0.0;
        for (int l = 0; l < a.NWL; ++l) {
            const double q0 = a.qel0[c + (long long)l * n];
            const double fx = q0 * a.g.DR[J] * a.g.DZ[K], fy = q0 * a.g.DX[I] * a.g.DZ[K], fz = q0 * a.g.DX[I] * a.g.DR[J];
            double q = 0.0;
            q = q + fx; q = q + fx; q = q + fy; q = q + fy; q = q + fz; q = q + fz;
            qe = l == 0 ? q : qe + q;
        }
        a.qe[c] = qe;
        qs += qe;
        cnt += 1.0;
    }
    sh[0][threadIdx.x] = qs;
    sh[1][threadIdx.x] = cnt;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) { sh[0][threadIdx.x] += sh[0][threadIdx.x + s]; sh[1][threadIdx.x] += sh[1][threadIdx.x + s]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { a.qe_part[2 * blockIdx.x] = sh[0][0]; a.qe_part[2 * blockIdx.x + 1] = sh[1][0]; }
}

// QAL = sum of the CTA copies in CTA order; QA = sum over bands (QRN1)
__global__ void k_rad_reduce(RadArgs a) {
    const int nparts = a.part_base[3];
    const int n = a.MZ * a.NZ * a.LZ;
    GFM_FOR(c, n) {
        double g0 = 0.0;
        for (int l = 0; l < a.NWL; ++l) {
            double s = 0.0;
            for (int b = 0; b < nparts; ++b) s += a.qal_part[(long long)b * n * a.NWL + (long long)l * n + c];
            g0 = g0 + s;
        }
        a.qa[c] = g0;
    }
}

template <typename R>
__global__ void k_rad_t_roundtrip(R* T, long long n, double t0) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        T[t] = R(((double)T[t] * t0) / t0);
}

size_t rad_smem_fixed(const RadArgs& a, int A) {   // coordinates, ANG1/2/3, angle candidates, slab IBCELL
    return sizeof(double) * (4 * ((size_t)(a.MP + 2) + (a.NP + 2) + (a.LP + 2))) + sizeof(int16_t) * (((size_t)A + 7) / 8 * 8);
}
size_t rad_smem_slab(const RadArgs& a, int A) { return (size_t)3 * A * a.NWL * sizeof(double) + (size_t)3 * A; }
int rad_slab_cells(const RadArgs& a, int d) {
    return d == 0 ? (a.NP / 2) * (a.LP / 2) : (d == 1 ? (a.MP / 2) * (a.LP / 2) : (a.MP / 2) * (a.NP / 2));
}
template <int NW>
int rad_plan_nw(RadArgs& a, int sms) {
    // dynamic shared memory available to one CTA: the device's opt-in
    // maximum less the kernel's static shared memory
    int dev = 0, optin = 0;
    cudaFuncAttributes fa{};
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, k_rad_trace<NW>) != cudaSuccess)
        return GFM_E_CUDA;
    const size_t limit = (size_t)optin - fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(k_rad_trace<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit) != cudaSuccess)
        return GFM_E_CUDA;
    int base = 0;
    for (int d = 0; d < 3; ++d) {
        const int A = rad_slab_cells(a, d);
        const size_t with = rad_smem_fixed(a, A) + rad_smem_slab(a, A);
        a.slab_in_smem[d] = with <= limit && !a.slab_global;
        a.smem[d] = a.slab_in_smem[d] ? with : rad_smem_fixed(a, A);
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_rad_trace<NW>, kRadThreads, a.smem[d]) != cudaSuccess)
            return GFM_E_CUDA;
        occ = occ < 1 ? 1 : (occ > 4 ? 4 : occ);
        a.grid[d] = sms * occ;
        a.part_base[d] = base;
        base += a.grid[d];
    }
    a.part_base[3] = base;
    return GFM_OK;
}

template <int NW>
void rad_trace_launch(const RadArgs& a, cudaStream_t const* st) {
    for (int d = 0; d < 3; ++d) k_rad_trace<NW><<<a.grid[d], kRadThreads, a.smem[d], st[d]>>>(a, d);
}

}  // namespace

int rad_plan(RadArgs& a, int sms) {
    switch (a.NWL) {
        case 4: return rad_plan_nw<4>(a, sms);
        case 10: return rad_plan_nw<10>(a, sms);
        default: return rad_plan_nw<0>(a, sms);
    }
}

// st[0] is the caller's stream; the x-, y- and z-directions run on st[0..2],
// forked after the per-cell kernels (ev[0]) and joined before the sums
// (ev[1], ev[2]).
template <typename R>
int launch_rad_transfer(RadArgs a, R* T, long long nT, cudaStream_t const* st, cudaEvent_t const* ev) {
    const int n = a.MZ * a.NZ * a.LZ;
    const int gb = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
    k_rad_mark<<<gb, 256, 0, st[0]>>>(a);
    k_rad_akl<R><<<a.akl_blocks, 256, 0, st[0]>>>(a, T);
    k_rad_qe<<<a.akl_blocks, 256, 0, st[0]>>>(a);
    if (cudaEventRecord(ev[0], st[0]) != cudaSuccess || cudaStreamWaitEvent(st[1], ev[0], 0) != cudaSuccess ||
        cudaStreamWaitEvent(st[2], ev[0], 0) != cudaSuccess)
        return GFM_E_CUDA;
    switch (a.NWL) {
        case 4: rad_trace_launch<4>(a, st); break;
        case 10: rad_trace_launch<10>(a, st); break;
        default: rad_trace_launch<0>(a, st); break;
    }
    if (cudaEventRecord(ev[1], st[1]) != cudaSuccess || cudaEventRecord(ev[2], st[2]) != cudaSuccess ||
        cudaStreamWaitEvent(st[0], ev[1], 0) != cudaSuccess || cudaStreamWaitEvent(st[0], ev[2], 0) != cudaSuccess)
        return GFM_E_CUDA;
    k_rad_reduce<<<gb, 256, 0, st[0]>>>(a);
    k_rad_t_roundtrip<R><<<1024, 256, 0, st[0]>>>(T, nT, a.t0);
    return cudaGetLastError() == cudaSuccess ? GFM_OK : GFM_E_CUDA;
}
template int launch_rad_transfer<double>(RadArgs, double*, long long, cudaStream_t const*, cudaEvent_t const*);
template int launch_rad_transfer<float>(RadArgs, float*, long long, cudaStream_t const*, cudaEvent_t const*);

}  // namespace gfm
