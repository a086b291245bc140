// adi.cu -- line-by-line ADI solver (ADLBL3, Adlbl3.f90:10-221) and the
// normalised equation residual (calc_residual, Adlbl3.f90:239-271).
//
// One plane update (ADLZ) solves, twice, every y-line and every z-line of the
// x-plane I with the Thomas algorithm and replaces the plane by the average of
// the two passes.  y- and z-lines of one pass only read the plane as it was
// before the pass, so all lines of both directions run concurrently inside one
// CTA; the average follows a barrier.
//
// Plane order:
//   GFM_ADI_MARCH    the reference's Gauss-Seidel march: planes IB..IE then
//                    IE..IB, NIM times, one CTA per equation walking the planes;
//                    PT and the pass results XT2/XT3 live in field-sized
//                    scratch (QT is stored in XT2/XT3 and back-substituted in
//                    place);
//   GFM_ADI_REDBLACK all planes of one colour at once, twice per sweep, NIM
//                    sweeps, on a colour-split copy of the system (below).
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "state.cuh"

namespace gfm {

#define A(arr, I, J, K) (arr)[pidx(g, (I), (J), (K))]

// One line of ADLZY (y-line, Adlbl3.f90:147-181) or ADLYZ (z-line,
// Adlbl3.f90:187-221): the Thomas forward sweep and back substitution over
// the n rows o0, o0+step, ..., writing PT and QT (then the solution) to pt/q.
// Within a class every neighbour of a row is a fixed offset: +-1 for I+-2,
// +-PX for J+-2, +-HY*PX for K+-2.  as[a_sub]/as[a_next] couple the line's
// previous/next row; as[1]/as[0] the planes I+2/I-2; as[a_p]/as[a_m] the
// in-plane neighbours across the line at +-d_pm.
// PT and QT of row r live at pt/q[l0 + r*lstep]: field-sized scratch
// indexed like the system (l0 = o0, lstep = step) or the plane's scratch in
// shared memory.
// The rows are taken NB at a time: their loads (coefficients, the right-hand
// side with its four neighbour terms, the copy test) are issued together
// before the pivot chain runs over them, so a step of the chain waits for
// arithmetic only.  Every value is formed by the same expression as in a
// row-by-row loop (NB = 1), so the results are the same bits; the right-hand
// side of a copied row is formed and not used.
template <typename R, int NB>
__device__ void adl_line(const GeoT<R>& g, const Sys<R>& s, R* __restrict__ pt, R* __restrict__ q, long long l0,
                         long long lstep, long long o0, int n, long long step, int a_sub, int a_next, int a_p, int a_m,
                         long long d_pm) {
    const R* __restrict__ xt = s.xt;
    const R* __restrict__ ap = s.ap;
    const R* __restrict__ bs = s.bs;
    const R* __restrict__ as_sub = s.as[a_sub];
    const R* __restrict__ as_next = s.as[a_next];
    const R* __restrict__ as_ip = s.as[1];
    const R* __restrict__ as_im = s.as[0];
    const R* __restrict__ as_p = s.as[a_p];
    const R* __restrict__ as_m = s.as[a_m];
    const int8_t* __restrict__ ib = g.ib;
    R pt_prev = R(0);
    R qt_prev = xt[o0 - step];   // QT of the row before the line: XT there
    long long ob = o0, lb = l0;   // first row of the batch
#pragma unroll 1
    for (int r0 = 0; r0 < n; r0 += NB, ob += NB * step, lb += NB * lstep) {
        R ap_[NB], sub_[NB], nxt_[NB], bsy_[NB], x_[NB];
        bool cp_[NB];
#pragma unroll
        for (int c = 0; c < NB; ++c) {
            if (r0 + c >= n) break;
            const long long o = ob + c * step;
            ap_[c] = ap[o];
            sub_[c] = as_sub[o];
            nxt_[c] = as_next[o];
            R bsy = bs[o];
            bsy = bsy + as_ip[o] * xt[o + 1] + as_im[o] * xt[o - 1];
            bsy = bsy + as_p[o] * xt[o + d_pm] + as_m[o] * xt[o - d_pm];
            bsy_[c] = bsy;
            x_[c] = xt[o];
            cp_[c] = ib[o] >= 1;
        }
#pragma unroll
        for (int c = 0; c < NB; ++c) {
            if (r0 + c >= n) break;
            R alp = ap_[c] - pt_prev * sub_[c];
            R p_, q_;
            if (fabs(alp) <= R(1.0e-20) || cp_[c]) {
                p_ = R(0);
                q_ = x_[c];
            } else {
                p_ = nxt_[c] / alp;
                q_ = (bsy_[c] + sub_[c] * qt_prev) / alp;
            }
            const long long l = lb + c * lstep;
            pt[l] = p_;
            q[l] = q_;
            pt_prev = p_;
            qt_prev = q_;
        }
    }
    // back substitution from the row after the line, whose value is XT there
    R nxt = xt[o0 + (long long)n * step];
    lb = l0 + (long long)(n - 1) * lstep;   // last row of the batch
#pragma unroll 1
    for (int r0 = n - 1; r0 >= 0; r0 -= NB, lb -= NB * lstep) {
        R pt_[NB], q_[NB];
#pragma unroll
        for (int c = 0; c < NB; ++c) {
            if (r0 - c < 0) break;
            pt_[c] = pt[lb - c * lstep];
            q_[c] = q[lb - c * lstep];
        }
#pragma unroll
        for (int c = 0; c < NB; ++c) {
            if (r0 - c < 0) break;
            R v = nxt * pt_[c] + q_[c];
            q[lb - c * lstep] = v;
            nxt = v;
        }
    }
}

// The pivots of a line: ALP = AP - PT(prev)*AS_sub and PT = AS_next/ALP,
// the expressions of ADLZY/ADLYZ, for every row; rows the reference copies
// (|ALP| <= 1e-20 or blocked) store ALP = 0 and PT = 0.  The coefficients are
// fixed during one ADLBL3 call, so these are the values every plane visit of
// the call would compute.
template <typename R>
__device__ void adl_pivots(const GeoT<R>& g, const Sys<R>& s, R* __restrict__ pt_out, R* __restrict__ alp_out,
                           long long o0, int n, long long step, int a_sub, int a_next) {
    const R* __restrict__ ap = s.ap;
    const R* __restrict__ as_sub = s.as[a_sub];
    const R* __restrict__ as_next = s.as[a_next];
    R pt_prev = R(0);
    for (int r = 0; r < n; ++r) {
        const long long o = o0 + (long long)r * step;
        R alp = ap[o] - pt_prev * as_sub[o];
        R p_;
        if (fabs(alp) <= R(1.0e-20) || g.ib[o] >= 1) {
            p_ = R(0);
            alp = R(0);
        } else {
            p_ = as_next[o] / alp;
        }
        pt_out[o] = p_;
        alp_out[o] = alp;
        pt_prev = p_;
    }
}

// One line as adl_line, with the pivots of the call (adl_pivots) loaded
// instead of formed: QT = (BSY + AS_sub*QT(prev))/ALP, the same expression,
// one division per row.  PT and QT go to the plane's shared-memory scratch.
template <typename R, int NB>
__device__ void adl_line_piv(const GeoT<R>& g, const Sys<R>& s, const R* __restrict__ piv_pt,
                             const R* __restrict__ piv_alp, R* __restrict__ pt, R* __restrict__ q, long long l0,
                             long long lstep, long long o0, int n, long long step, int a_sub, int a_p, int a_m,
                             long long d_pm) {
    const R* __restrict__ xt = s.xt;
    const R* __restrict__ bs = s.bs;
    const R* __restrict__ as_sub = s.as[a_sub];
    const R* __restrict__ as_ip = s.as[1];
    const R* __restrict__ as_im = s.as[0];
    const R* __restrict__ as_p = s.as[a_p];
    const R* __restrict__ as_m = s.as[a_m];
    R qt_prev = xt[o0 - step];
    long long ob = o0, lb = l0;
#pragma unroll 1
    for (int r0 = 0; r0 < n; r0 += NB, ob += NB * step, lb += NB * lstep) {
        R alp_[NB], sub_[NB], pt_[NB], bsy_[NB], x_[NB];
#pragma unroll
        for (int c = 0; c < NB; ++c) {
            if (r0 + c >= n) break;
            const long long o = ob + c * step;
            alp_[c] = piv_alp[o];
            pt_[c] = piv_pt[o];
            sub_[c] = as_sub[o];
            R bsy = bs[o];
            bsy = bsy + as_ip[o] * xt[o + 1] + as_im[o] * xt[o - 1];
            bsy = bsy + as_p[o] * xt[o + d_pm] + as_m[o] * xt[o - d_pm];
            bsy_[c] = bsy;
            x_[c] = xt[o];
        }
#pragma unroll
        for (int c = 0; c < NB; ++c) {
            if (r0 + c >= n) break;
            const R q_ = alp_[c] == R(0) ? x_[c] : (bsy_[c] + sub_[c] * qt_prev) / alp_[c];
            const long long l = lb + c * lstep;
            pt[l] = pt_[c];
            q[l] = q_;
            qt_prev = q_;
        }
    }
    R nxt = xt[o0 + (long long)n * step];
    lb = l0 + (long long)(n - 1) * lstep;
#pragma unroll 1
    for (int r0 = n - 1; r0 >= 0; r0 -= NB, lb -= NB * lstep) {
        R p_[NB], q_[NB];
#pragma unroll
        for (int c = 0; c < NB; ++c) {
            if (r0 - c < 0) break;
            p_[c] = pt[lb - c * lstep];
            q_[c] = q[lb - c * lstep];
        }
#pragma unroll
        for (int c = 0; c < NB; ++c) {
            if (r0 - c < 0) break;
            R v = nxt * p_[c] + q_[c];
            q[lb - c * lstep] = v;
            nxt = v;
        }
    }
}

// ADLZ (Adlbl3.f90:103-141) on plane I by the whole CTA.  With SM the lines'
// PT and QT live in the plane's scratch in shared memory (four arrays of
// nJ*nK, element (J,K) at ((K-kb)/2)*nJ + (J-jb)/2), else in the field-sized
// scratch; the values are the same either way.
template <typename R, int NB, bool SM, bool PIV = false>
__device__ void adlz(const GeoT<R>& g, const Sys<R>& s, const AdiScratch<R>& w, int I, R* sm, int wy) {
    const int LD = 2;
    const int nK = (s.ke - s.kb) / LD + 1, nJ = (s.je - s.jb) / LD + 1;
    const long long P = (long long)nJ * nK;
    R* pty = SM ? sm : w.pty;
    R* xt2 = SM ? sm + P : w.xt2;
    R* ptz = SM ? sm + 2 * P : w.ptz;
    R* xt3 = SM ? sm + 3 * P : w.xt3;
    for (int L = 1; L <= 2; ++L) {
        const long long dJ = g.PX, dK = (long long)g.HY * g.PX;
        // contiguous (wy == 0): thread t takes lines t, t + blockDim.x, .. of
        // the y-lines followed by the z-lines; split: warps [0, wy) take the
        // y-lines, the other warps the z-lines, each spread over its warps
        int v0 = threadIdx.x, vstep = blockDim.x, vend = nK + nJ, off = 0;
        if (wy > 0) {
            const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, nw = blockDim.x >> 5;
            if (wp < wy) { v0 = lane * wy + wp; vstep = 32 * wy; vend = nK; }
            else { v0 = lane * (nw - wy) + (wp - wy); vstep = 32 * (nw - wy); vend = nJ; off = nK; }
        }
        for (int v = v0; v < vend; v += vstep) {
            const int t = v + off;
            if (t < nK) {   // y-line (I,*,K): XT2, PT of y
                const long long o0 = pidx(g, I, s.jb, s.kb + LD * t);
                if (PIV) adl_line_piv<R, NB>(g, s, w.pty, w.xt2, pty, xt2, (long long)t * nJ, 1, o0, nJ, dJ, 2, 5, 4, dK);
                else adl_line<R, NB>(g, s, pty, xt2, SM ? (long long)t * nJ : o0, SM ? 1 : dJ, o0, nJ, dJ, 2, 3, 5, 4, dK);
            } else {        // z-line (I,J,*): XT3, PT of z
                const long long o0 = pidx(g, I, s.jb + LD * (t - nK), s.kb);
                if (PIV) adl_line_piv<R, NB>(g, s, w.ptz, w.xt3, ptz, xt3, (long long)(t - nK), nJ, o0, nK, dK, 4, 3, 2, dJ);
                else adl_line<R, NB>(g, s, ptz, xt3, SM ? (long long)(t - nK) : o0, SM ? nJ : dK, o0, nK, dK, 4, 5, 3, 2, dJ);
            }
        }
        __syncthreads();
        // a plane with one z-row (KB >= KE) takes the y-line pass alone and
        // is done after it (Adlbl3.f90:124-130); the z-lines solved
        // alongside are not used
        const bool one_row = s.kb >= s.ke;
        for (int t = threadIdx.x; t < nK * nJ; t += blockDim.x) {
            int K = s.kb + LD * (t / nJ), J = s.jb + LD * (t % nJ);
            long long o = pidx(g, I, J, K);
            const long long l = SM ? t : o;
            s.xt[o] = one_row ? xt2[l] : (xt2[l] + xt3[l]) / R(2);
        }
        __syncthreads();
        if (one_row) return;
    }
}

template <typename R>
struct AdiBatch {
    Sys<R> sys[8];
    AdiScratch<R> scr[8];
    int nsys;
    int wy[8];    // march layout of each system: 0 contiguous, else the warps of the y-lines
};

// Pivots of every y- and z-line of every plane of the batch's systems, one
// thread per line: y-line pivots into PTY/XT2, z-line pivots into PTZ/XT3 of
// the field-sized scratch, which the shared-memory march does not use.
template <typename R>
__global__ void k_march_pivots(GeoT<R> g, AdiBatch<R> b) {
    const Sys<R>& s = b.sys[blockIdx.y];
    const AdiScratch<R>& w = b.scr[blockIdx.y];
    const int npl = (s.ie - s.ib) / 2 + 1, nK = (s.ke - s.kb) / 2 + 1, nJ = (s.je - s.jb) / 2 + 1;
    const long long dJ = g.PX, dK = (long long)g.HY * g.PX;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < npl * (nK + nJ); t += gridDim.x * blockDim.x) {
        const int I = s.ib + 2 * (t % npl), u = t / npl;
        if (u < nK) adl_pivots<R>(g, s, w.pty, w.xt2, pidx(g, I, s.jb, s.kb + 2 * u), nJ, dJ, 2, 3);
        else adl_pivots<R>(g, s, w.ptz, w.xt3, pidx(g, I, s.jb + 2 * (u - nK), s.kb), nK, dK, 4, 5);
    }
}

// reference march: one CTA per equation; NB rows of a line per load batch;
// with SM the plane's line scratch in dynamic shared memory.
// At most kMarchThreads threads (a plane with more lines loops over them):
// the batched loads take up to 247 registers a thread.
constexpr int kMarchThreads = 256;
constexpr size_t kMarchMaxSmem = 227 * 1024;   // opt-in dynamic shared memory of one CTA
template <typename R, int NB, bool SM, bool PIV = false>
__global__ void __launch_bounds__(kMarchThreads) k_adlbl3_march(GeoT<R> g, AdiBatch<R> b) {
    extern __shared__ __align__(16) unsigned char march_smem[];
    R* sm = reinterpret_cast<R*>(march_smem);
    const Sys<R>& s = b.sys[blockIdx.x];
    const AdiScratch<R>& w = b.scr[blockIdx.x];
    for (int ns = 0; ns < s.nim; ++ns) {
        for (int I = s.ib; I <= s.ie; I += 2) adlz<R, NB, SM, PIV>(g, s, w, I, sm, b.wy[blockIdx.x]);
        for (int I = s.ie; I >= s.ib; I -= 2) adlz<R, NB, SM, PIV>(g, s, w, I, sm, b.wy[blockIdx.x]);
    }
}

// rows per load batch of the march: 4 (with the pivots of the call and the
// plane's scratch in shared memory where it fits), or 1 when GFM_MARCH_ROWS=1:
// the reference's row-by-row loop with field-sized scratch, kept to show that
// both give the same bits
static int march_rows() {
    static const int v = [] {
        const char* e = std::getenv("GFM_MARCH_ROWS");
        return (e && std::atoi(e) == 1) ? 1 : 4;
    }();
    return v;
}
// GFM_MARCH_LAYOUT=contiguous keeps thread t on lines t, t + blockDim.x, ..
// (kept to show that the split layout gives the same bits)
static bool march_contiguous() {
    static const bool v = [] {
        const char* e = std::getenv("GFM_MARCH_LAYOUT");
        return e && std::strcmp(e, "contiguous") == 0;
    }();
    return v;
}

// Rows of line recurrence a warp issues in one plane: a y-line is nJ rows, a
// z-line nK rows, and a warp whose lanes hold both kinds in one round runs
// both branches, one after the other.  The key of a layout is the largest
// warp's rows, then the rows of the busiest SM sub-partition (warp w on
// sub-partition w mod 4): a line's rows are a chain of dependent divisions,
// and the narrow FP64 pipe of a sub-partition costs the same per warp
// instruction whatever the number of active lanes.  Last, the most lanes a
// warp uses: a warp load over fewer lines touches fewer cache lines.
static long long march_layout_cost(int nJ, int nK, int warps, int wy) {
    long long smsp[4] = {0, 0, 0, 0}, wmax = 0;
    int lanes = 0;
    const int T = warps * 32;
    for (int w = 0; w < warps; ++w) {
        long long c = 0;
        if (wy == 0) {
            for (int r0 = 32 * w; r0 < nK + nJ; r0 += T) {
                const int e = std::min(r0 + 32, nK + nJ);
                c += (r0 < nK ? nJ : 0) + (e > nK ? nK : 0);
                lanes = std::max(lanes, e - r0);
            }
        } else if (w < wy) {
            for (int t = w; t < nK; t += 32 * wy) c += nJ;
            lanes = std::max(lanes, std::min(32, (nK - w + wy - 1) / wy));
        } else {
            for (int u = w - wy; u < nJ; u += 32 * (warps - wy)) c += nK;
            lanes = std::max(lanes, std::min(32, (nJ - (w - wy) + warps - wy - 1) / (warps - wy)));
        }
        smsp[w % 4] += c;
        wmax = std::max(wmax, c);
    }
    const long long sub = std::max(std::max(smsp[0], smsp[1]), std::max(smsp[2], smsp[3]));
    return (wmax << 40) + (sub << 8) + std::max(lanes, 0);
}

// ---------------------------------------------------------------------------
// Red-black order (GFM_ADI_REDBLACK) on a colour-split copy of the system.
//
// Planes of one colour are updated together; each plane update is still ADLZ
// (L = 1, 2: every y-line and z-line solved from the plane as it was before
// the pass, then averaged).  Three things make it fast on GB300:
//
//  * Colour split.  For the duration of one ADLBL3 call the unknown and the
//    factored rows live in arrays where the x-index xi = I>>1 of the class is
//    split by parity, element (xi,yj,zk) at (xi&1)*CBH + (zk*HY+yj)*PXH + xi>>1.
//    Planes of one colour are then unit-stride, so a warp whose lanes are
//    consecutive same-colour planes reads whole sectors; the x-neighbours
//    I+-2 are the other half at the same or the adjacent position.
//  * Factor once.  The tridiagonal matrix of every line is fixed during the
//    call, so its Thomas pivots are computed once and every row is stored
//    pre-scaled by IA = 1/ALP in two vector records per line direction:
//        A = (AS_op*IA, AS_om*IA, AS_sub*IA, PT),  B = (BS*IA, AS12*IA, AS11*IA, 0)
//    (op/om: the two in-plane neighbours across the line, sub: the previous
//    point of the line).  Rows the reference copies unchanged (|ALP| <= 1e-20
//    or a blocked cell) have zero coefficients and PT = -0.0, a value no other
//    row stores (a zero PT of any other row is +0.0).  A forward step
//    is then QT = B.x + B.y*XT(I+2) + B.z*XT(I-2) + A.x*XT(op) + A.y*XT(om)
//    + A.z*QT(prev), the reference's (BSY + AS_sub*QT(prev))/ALP with the
//    division applied to each term.  Within a pass the x-neighbour part is
//    constant: the first pass of a visit stores it (SBY/SBZ), the second
//    reads it.
//  * Segmented recurrences.  Each line is cut into S segments, one warp per
//    segment (lane = plane).  The forward and the back substitution are
//    affine recurrences: every thread runs its segment from a zero start,
//    keeping the values and the running product of the multipliers in
//    registers; a scan over the S segment maps in shared memory gives each
//    segment its true start, and the thread corrects its values in place.
//    The non-recurrent part of every row is computed before the recurrence
//    runs, so all loads of a segment are in flight together.
// ---------------------------------------------------------------------------
template <typename R>
struct RbBatch {
    Sys<R> sys[8];
    AdiScratch<R> scr[8];
    int nsys;
};

template <typename R>
__device__ __forceinline__ int sidx(const GeoT<R>& g, int xi, int yj, int zk) {
    return (xi & 1) * g.CBH + (zk * g.HY + yj) * g.PXH + (xi >> 1);
}
__device__ __forceinline__ int rb_nplanes(int ib, int ie) { return (ie - ib) / 2 + 1; }
// the copy-row marker PT = -0.0
__device__ __forceinline__ bool rb_copy(float pt) { return __float_as_uint(pt) == 0x80000000u; }
__device__ __forceinline__ bool rb_copy(double pt) {
    return (unsigned long long)__double_as_longlong(pt) == 0x8000000000000000ull;
}
__device__ __forceinline__ int rb_class(int ib, int jb, int kb) { return (ib & 1) | ((jb & 1) << 1) | ((kb & 1) << 2); }

// XT of the whole class -> split copy
template <typename R>
__global__ void k_rbs_in(GeoT<R> g, RbBatch<R> b) {
    pdl_wait();
    pdl_trigger();
    const Sys<R>& s = b.sys[blockIdx.y];
    const AdiScratch<R>& w = b.scr[blockIdx.y];
    const R* __restrict__ xt = s.xt + (long long)rb_class(s.ib, s.jb, s.kb) * g.CB;
    const int n = g.HX * g.HY * g.HZ;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int xi = t % g.HX, r = t / g.HX;
        const int yj = r % g.HY, zk = r / g.HY;
        w.xs[sidx(g, xi, yj, zk)] = xt[(zk * g.HY + yj) * g.PX + xi];
    }
}

// Factored, pre-scaled rows of every y-line and z-line of every plane (both
// colours), thread per line with the plane index fastest.  The pivot chain is
// ADLZY/ADLYZ's: ALP = AP - PT(prev)*AS_sub, PT = AS_next/ALP.  Rows are read
// C at a time before the chain runs over them, so a thread keeps C rows of
// loads in flight.
template <typename R>
__global__ void k_rbs_factor(GeoT<R> g, RbBatch<R> b) {
    pdl_wait();
    pdl_trigger();
    constexpr int C = 8;
    const Sys<R>& s = b.sys[blockIdx.y];
    const AdiScratch<R>& w = b.scr[blockIdx.y];
    const int npl = rb_nplanes(s.ib, s.ie), nK = (s.ke - s.kb) / 2 + 1, nJ = (s.je - s.jb) / 2 + 1;
    const int ny = npl * nK, nz = npl * nJ;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ny + nz; t += gridDim.x * blockDim.x) {
        const bool zl = t >= ny;
        const int u = zl ? t - ny : t;
        const int I = s.ib + 2 * (u % npl);
        // y-line (I,*,K): sub AS(J-2)=as[2], next AS(J+2)=as[3], across as[5]/as[4]
        // z-line (I,J,*): sub AS(K-2)=as[4], next AS(K+2)=as[5], across as[3]/as[2]
        const R* __restrict__ a_sub = s.as[zl ? 4 : 2];
        const R* __restrict__ a_next = s.as[zl ? 5 : 3];
        const R* __restrict__ a_op = s.as[zl ? 3 : 5];
        const R* __restrict__ a_om = s.as[zl ? 2 : 4];
        Quad<R>* __restrict__ qa = zl ? w.za : w.ya;
        Quad<R>* __restrict__ qb = zl ? w.zb : w.yb;
        const int n = zl ? nK : nJ;
        const int J0 = zl ? s.jb + 2 * (u / npl) : s.jb, K0 = zl ? s.kb : s.kb + 2 * (u / npl);
        const int o0 = (int)pidx(g, I, J0, K0), q0 = sidx(g, I >> 1, J0 >> 1, K0 >> 1);
        const int ostep = zl ? g.PX * g.HY : g.PX, qstep = zl ? g.HY * g.PXH : g.PXH;
        R pt_prev = R(0);
        for (int e0 = 0; e0 < n; e0 += C) {
            R vap[C], vsub[C], vnext[C], vop[C], vom[C], vbs[C], va1[C], va0[C];
            bool blk[C];
#pragma unroll
            for (int i = 0; i < C; ++i) {
                if (e0 + i < n) {
                    const int o = o0 + (e0 + i) * ostep;
                    vap[i] = s.ap[o]; vsub[i] = a_sub[o]; vnext[i] = a_next[o];
                    vop[i] = a_op[o]; vom[i] = a_om[o]; vbs[i] = s.bs[o];
                    va1[i] = s.as[1][o]; va0[i] = s.as[0][o];
                    blk[i] = g.ib[o] >= 1;
                }
            }
#pragma unroll
            for (int i = 0; i < C; ++i) {
                if (e0 + i < n) {
                    const int q = q0 + (e0 + i) * qstep;
                    const R alp = vap[i] - pt_prev * vsub[i];
                    Quad<R> A, B;
                    if (fabs(alp) <= R(1.0e-20) || blk[i]) {
                        A = Quad<R>{R(0), R(0), R(0), -R(0)};
                        B = Quad<R>{R(0), R(0), R(0), R(0)};
                        pt_prev = R(0);
                    } else {
                        const R ia = R(1) / alp;
                        const R pt = vnext[i] / alp;
                        A = Quad<R>{vop[i] * ia, vom[i] * ia, vsub[i] * ia, pt + R(0)};   // +0.0: no -0.0 here
                        B = Quad<R>{vbs[i] * ia, va1[i] * ia, va0[i] * ia, R(0)};
                        pt_prev = pt;
                    }
                    qa[q] = A;
                    qb[q] = B;
                }
            }
        }
    }
}

// at most M elements per segment, held in registers; S <= 32 segments per line
#ifndef GFM_RB_M
#define GFM_RB_M 8
#endif
template <typename R> struct RbSeg { static constexpr int M = GFM_RB_M; };
// minimum resident pass blocks per SM (blocks of up to 512 threads).  A
// 64-register cap (2) measured 7 % slower than the compiler's own choice.
#ifndef GFM_RB_MINB
#define GFM_RB_MINB 1
#endif

// One pass of all y- and z-lines of the planes of one colour.  Block = S warps
// x 32 lanes; lane = one line (32 consecutive line slots), warp = segment.
// Pass L=1 (FIRST) reads XT and writes X2/X3 and the scaled x-neighbour
// terms; pass L=2 writes X2B/X3B, which an averaging launch brings into XT.
// Pass L=2 reads XT too, or with AVG, for the cells of the solve range, the
// average (X2+X3)/2 of its colour's pass L=1 -- the value the averaging
// launch between the passes would have stored in XT, computed the same way,
// so that launch is left out.  (Averaging in pass L=1 as well, with X2B/X3B
// seeded from XT, removes the other launch but measured slower: pass L=1
// then needs ten neighbour loads a row.)
template <typename R, int S, bool FIRST, bool AVG>
__global__ void __launch_bounds__(32 * S, (32 * S <= 512 ? GFM_RB_MINB : 1))
    k_rbs_pass(GeoT<R> g, RbBatch<R> b, int colour, int sweep) {
    constexpr int M = RbSeg<R>::M;
    __shared__ R sA[S][32], sB[S][32];
    pdl_wait();
    pdl_trigger();
    const Sys<R>& s = b.sys[blockIdx.y];
    if (sweep >= s.nim) return;
    if (!FIRST && s.kb >= s.ke) return;            // one z-row: the y-line pass alone (Adlbl3.f90:124-130)
    const AdiScratch<R>& w = b.scr[blockIdx.y];
    const int npl = rb_nplanes(s.ib, s.ie);
    const int npc = (npl - colour + 1) / 2;
    const int nK = (s.ke - s.kb) / 2 + 1, nJ = (s.je - s.jb) / 2 + 1;
    const int ny = npc * nK, nz = npc * nJ;
    if ((int)blockIdx.x * 32 >= ny + nz) return;   // whole block
    const int lane = threadIdx.x & 31, seg = threadIdx.x >> 5;
    const int t = blockIdx.x * 32 + lane;
    const bool active = t < ny + nz;
    const int xh = (s.ib >> 1) + colour;           // xi of the first plane of this colour
    const int h = xh & 1;
    const int hb = h * g.CBH + (xh >> 1);
    const int SZ = g.HY * g.PXH;
    const int dxp = (1 - 2 * h) * g.CBH + h, dxm = dxp - 1;   // x-neighbours I+2, I-2 in the other half
    const bool zl = active && t >= ny;
    int base = 0, step = 0, ostep = 0, n = 0;
    bool up_in = false, dn_in = false;             // the neighbour lines at +-ostep lie in the solve range
    if (active) {
        if (!zl) {
            const int r = t % npc, kk = t / npc;
            base = hb + ((s.kb >> 1) + kk) * SZ + (s.jb >> 1) * g.PXH + r;
            step = g.PXH; ostep = SZ; n = nJ;
            up_in = kk + 1 < nK; dn_in = kk > 0;
        } else {
            const int u = t - ny, r = u % npc, jj = u / npc;
            base = hb + (s.kb >> 1) * SZ + ((s.jb >> 1) + jj) * g.PXH + r;
            step = SZ; ostep = g.PXH; n = nK;
            up_in = jj + 1 < nJ; dn_in = jj > 0;
        }
    }
    const R* __restrict__ x = w.xs;
    const R* __restrict__ x2 = w.x2;
    const R* __restrict__ x3 = w.x3;
    const Quad<R>* __restrict__ QA = zl ? w.za : w.ya;
    const Quad<R>* __restrict__ QB = zl ? w.zb : w.yb;
    R* __restrict__ sb = zl ? w.sbz : w.sby;
    R* __restrict__ out = FIRST ? (zl ? w.x3 : w.x2) : (zl ? w.x3b : w.x2b);
    const int m = (n + S - 1) / S;
    const int e0 = seg * m;
    int cnt = n - e0;
    cnt = cnt < 0 ? 0 : (cnt > m ? m : cnt);
    // XT one step below and one step above the line (JBML / KBML, JEPL / KEPL):
    // never updated by the pass, so loaded up front with the rows
    const R xlo = active ? x[base - step] : R(0);
    const R xhi = active ? x[base + n * step] : R(0);

    // non-recurrent part of every row of the segment
    R rr[M], al[M], pv[M];
#pragma unroll
    for (int i = 0; i < M; ++i) {
        if (i < cnt) {
            const int o = base + (e0 + i) * step;
            const Quad<R> A = QA[o];
            R v;
            const int ou = o + ostep, od = o - ostep;
            const R xu = AVG && up_in ? (x2[ou] + x3[ou]) / R(2) : x[ou];
            const R xd = AVG && dn_in ? (x2[od] + x3[od]) / R(2) : x[od];
            if (FIRST) {
                const Quad<R> B = QB[o];
                const R bx = B.x + B.y * x[o + dxp] + B.z * x[o + dxm];
                sb[o] = bx;
                v = bx + A.x * xu + A.y * xd;
            } else {
                v = sb[o] + A.x * xu + A.y * xd;
            }
            if (rb_copy(A.w)) v = AVG ? (x2[o] + x3[o]) / R(2) : x[o];
            rr[i] = v;
            al[i] = A.z;
            pv[i] = A.w;
        }
    }
    // forward recurrence of the segment from a zero start
    R q[M], P[M];
    R qc = R(0), Pc = R(1);
#pragma unroll
    for (int i = 0; i < M; ++i) {
        if (i < cnt) {
            qc = rr[i] + al[i] * qc;
            Pc = al[i] * Pc;
            q[i] = qc;
            P[i] = Pc;
        }
    }
    sA[seg][lane] = cnt > 0 ? Pc : R(1);
    sB[seg][lane] = cnt > 0 ? qc : R(0);
    __syncthreads();
    R qin = xlo;
    for (int k = 0; k < seg; ++k) qin = sA[k][lane] * qin + sB[k][lane];
#pragma unroll
    for (int i = 0; i < M; ++i)
        if (i < cnt) q[i] = q[i] + P[i] * qin;
    __syncthreads();

    // back substitution of the segment from a zero end value
    R xc = R(0), Rc = R(1);
#pragma unroll
    for (int i = M - 1; i >= 0; --i) {
        if (i < cnt) {
            xc = pv[i] * xc + q[i];
            Rc = pv[i] * Rc;
            q[i] = xc;
            P[i] = Rc;
        }
    }
    sA[seg][lane] = cnt > 0 ? Rc : R(1);
    sB[seg][lane] = cnt > 0 ? xc : R(0);
    __syncthreads();
    R xin = xhi;
    for (int k = S - 1; k > seg; --k) xin = sA[k][lane] * xin + sB[k][lane];
#pragma unroll
    for (int i = 0; i < M; ++i)
        if (i < cnt) out[base + (e0 + i) * step] = q[i] + P[i] * xin;
}

// XT = (XT2 + XT3)/2 on the planes of one colour (split copy).  Grid x runs
// over the planes of the colour (unit stride); each thread row handles
// kAvgRows (J,K) rows, kAvgRows*8 rows per block, loads issued together.
#ifndef GFM_AVG_ROWS
#define GFM_AVG_ROWS 8
#endif
constexpr int kAvgRows = GFM_AVG_ROWS;
// second: average the pass-2 results X2B/X3B (else the pass-1 results X2/X3)
template <typename R>
__global__ void k_rbs_avg(GeoT<R> g, RbBatch<R> b, int colour, int sweep, int second) {
    pdl_wait();
    pdl_trigger();
    const Sys<R>& s = b.sys[blockIdx.y];
    if (sweep >= s.nim) return;
    const AdiScratch<R>& w = b.scr[blockIdx.y];
    // one z-row (KB >= KE): the plane takes its pass L=1 y-line result and
    // nothing else (Adlbl3.f90:124-130); pass L=2 left it untouched
    const bool one_row = s.kb >= s.ke;
    const R* __restrict__ x2 = second && !one_row ? w.x2b : w.x2;
    const R* __restrict__ x3 = second && !one_row ? w.x3b : w.x3;
    const int npl = rb_nplanes(s.ib, s.ie);
    const int npc = (npl - colour + 1) / 2;
    const int nK = (s.ke - s.kb) / 2 + 1, nJ = (s.je - s.jb) / 2 + 1;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= npc) return;
    const int xh = (s.ib >> 1) + colour;
    const int hb = (xh & 1) * g.CBH + (xh >> 1) + r + ((s.kb >> 1) * g.HY + (s.jb >> 1)) * g.PXH;
    const int row0 = (blockIdx.z * blockDim.y + threadIdx.y) * kAvgRows;
    int o[kAvgRows];
    R a[kAvgRows], c[kAvgRows];
#pragma unroll
    for (int i = 0; i < kAvgRows; ++i) {
        const int row = row0 + i;
        const int jj = row % nJ, kk = row / nJ;
        o[i] = hb + (kk * g.HY + jj) * g.PXH;
        if (row < nJ * nK) { a[i] = x2[o[i]]; c[i] = x3[o[i]]; }
    }
#pragma unroll
    for (int i = 0; i < kAvgRows; ++i)
        if (row0 + i < nJ * nK) w.xs[o[i]] = one_row ? a[i] : (a[i] + c[i]) / R(2);
}

// split copy -> XT on the solve range
template <typename R>
__global__ void k_rbs_out(GeoT<R> g, RbBatch<R> b) {
    pdl_wait();
    pdl_trigger();
    const Sys<R>& s = b.sys[blockIdx.y];
    const AdiScratch<R>& w = b.scr[blockIdx.y];
    const int npl = rb_nplanes(s.ib, s.ie), nK = (s.ke - s.kb) / 2 + 1, nJ = (s.je - s.jb) / 2 + 1;
    const int n = npl * nJ * nK;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int p = t % npl, rest = t / npl;
        const int I = s.ib + 2 * p, J = s.jb + 2 * (rest % nJ), K = s.kb + 2 * (rest / nJ);
        s.xt[pidx(g, I, J, K)] = w.xs[sidx(g, I >> 1, J >> 1, K >> 1)];
    }
}

// ---------------------------------------------------------------------------
// calc_residual: per-cell |sum a_nb x_nb + b - a_p x| / max(terms), evaluated
// in the solver's arithmetic type (the FP64 path keeps the reference's FP64
// operation order); the per-thread sums and the block partials are FP64.
// Neighbours I+-2, J+-2, K+-2 of a class are +-1, +-PX, +-PX*HY apart.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_residual(GeoT<R> g, Sys<R> s, double* partials, int slot) {
    __shared__ double sh[32];
    const int ni = (s.ie - s.ib) / 2 + 1, nj = (s.je - s.jb) / 2 + 1, nk = (s.ke - s.kb) / 2 + 1;
    const int n = ni * nj * nk;
    const int sy = g.PX, sz = g.PX * g.HY;
    const R* __restrict__ xt = s.xt;
    double acc = 0.0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int i = s.ib + 2 * (t % ni);
        const int r = t / ni;
        const int j = s.jb + 2 * (r % nj), k = s.kb + 2 * (r / nj);
        const int o = (int)pidx(g, i, j, k);
        if (g.ib[o] > 0) continue;
        R t1 = s.as[0][o] * xt[o - 1], t2 = s.as[1][o] * xt[o + 1];
        R t3 = s.as[2][o] * xt[o - sy], t4 = s.as[3][o] * xt[o + sy];
        R t5 = s.as[4][o] * xt[o - sz], t6 = s.as[5][o] * xt[o + sz];
        R t7 = s.ap[o] * xt[o], t8 = s.bs[o];
        R em = fabs(t1);
        em = fabs(t2) > em ? fabs(t2) : em; em = fabs(t3) > em ? fabs(t3) : em; em = fabs(t4) > em ? fabs(t4) : em;
        em = fabs(t5) > em ? fabs(t5) : em; em = fabs(t6) > em ? fabs(t6) : em; em = fabs(t7) > em ? fabs(t7) : em;
        em = fabs(t8) > em ? fabs(t8) : em;
        acc += (double)(fabs(t1 + t2 + t3 + t4 + t5 + t6 + t8 - t7) / em);   // 0/0 -> NaN as in the reference
    }
    double v = block_sum(acc, sh);
    if (threadIdx.x == 0) partials[slot * kRedBlocks + blockIdx.x] = v;
}

// ---------------------------------------------------------------------------
// Iterative refinement of a line solve (mixed precision, p' equation): the
// right-hand side of the correction system, r = BS + sum AS*XT_nb - AP*XT,
// evaluated in FP64 from the stored coefficients and the current XT, and the
// update XT += DX on the solve range.  Rows the line solver copies unchanged
// (blocked cells) get r = 0.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_refine_rhs(GeoT<R> g, Sys<R> s, R* rhs) {
    const int ni = (s.ie - s.ib) / 2 + 1, nj = (s.je - s.jb) / 2 + 1, nk = (s.ke - s.kb) / 2 + 1;
    const int n = ni * nj * nk;
    const int sy = g.PX, sz = g.PX * g.HY;
    const R* __restrict__ xt = s.xt;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int i = s.ib + 2 * (t % ni);
        const int r = t / ni;
        const int j = s.jb + 2 * (r % nj), k = s.kb + 2 * (r / nj);
        const int o = (int)pidx(g, i, j, k);
        double v = 0.0;
        if (g.ib[o] < 1) {
            v = (double)s.bs[o] + (double)s.as[0][o] * (double)xt[o - 1] + (double)s.as[1][o] * (double)xt[o + 1] +
                (double)s.as[2][o] * (double)xt[o - sy] + (double)s.as[3][o] * (double)xt[o + sy] +
                (double)s.as[4][o] * (double)xt[o - sz] + (double)s.as[5][o] * (double)xt[o + sz] -
                (double)s.ap[o] * (double)xt[o];
        }
        rhs[o] = R(v);
    }
}
template <typename R>
__global__ void k_refine_add(GeoT<R> g, Sys<R> s, const R* __restrict__ dx) {
    const int ni = (s.ie - s.ib) / 2 + 1, nj = (s.je - s.jb) / 2 + 1, nk = (s.ke - s.kb) / 2 + 1;
    const int n = ni * nj * nk;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int i = s.ib + 2 * (t % ni);
        const int r = t / ni;
        const int j = s.jb + 2 * (r % nj), k = s.kb + 2 * (r / nj);
        const int o = (int)pidx(g, i, j, k);
        s.xt[o] = s.xt[o] + dx[o];
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <typename R>
void launch_residual(const Ctx<R>& c, const Sys<R>& s, int slot, cudaStream_t st) {
    const int ni = (s.ie - s.ib) / 2 + 1, nj = (s.je - s.jb) / 2 + 1, nk = (s.ke - s.kb) / 2 + 1;
    long long n = (long long)ni * nj * nk;
    long long nb = (n + 255) / 256;
    if (nb > kRedBlocks) nb = kRedBlocks;
    if (nb < 1) nb = 1;
    k_residual<R><<<(int)nb, 256, 0, st>>>(c.g, s, c.partials, slot);
}

// Segments per line: the smallest power of two that keeps a segment within
// the M registers of one thread (lines of up to 32*M points, checked at create).
#ifndef GFM_RB_MIN_SEGMENTS
#define GFM_RB_MIN_SEGMENTS 1
#endif
template <typename R>
int rb_segments(int n) {
    int S = 1;
    while (S < 32 && (S * RbSeg<R>::M < n || S < GFM_RB_MIN_SEGMENTS)) S *= 2;
    return S;
}
template <typename R, bool FIRST, bool AVG>
void rb_pass_s(bool pdl, int S, dim3 gp, const GeoT<R>& g, const RbBatch<R>& rb, int colour, int ns, cudaStream_t st) {
    switch (S) {
        case 1: launch_k(pdl, k_rbs_pass<R, 1, FIRST, AVG>, gp, 32, 0, st, g, rb, colour, ns); break;
        case 2: launch_k(pdl, k_rbs_pass<R, 2, FIRST, AVG>, gp, 64, 0, st, g, rb, colour, ns); break;
        case 4: launch_k(pdl, k_rbs_pass<R, 4, FIRST, AVG>, gp, 128, 0, st, g, rb, colour, ns); break;
        case 8: launch_k(pdl, k_rbs_pass<R, 8, FIRST, AVG>, gp, 256, 0, st, g, rb, colour, ns); break;
        case 16: launch_k(pdl, k_rbs_pass<R, 16, FIRST, AVG>, gp, 512, 0, st, g, rb, colour, ns); break;
        default: launch_k(pdl, k_rbs_pass<R, 32, FIRST, AVG>, gp, 1024, 0, st, g, rb, colour, ns); break;
    }
}
// pass L=1, or pass L=2 reading XT (avg false) or the pass L=1 average
template <typename R>
void rb_pass(bool pdl, int S, bool first, bool avg, dim3 gp, const GeoT<R>& g, const RbBatch<R>& rb, int colour, int ns,
             cudaStream_t st) {
    if (first) rb_pass_s<R, true, false>(pdl, S, gp, g, rb, colour, ns, st);
    else if (avg) rb_pass_s<R, false, true>(pdl, S, gp, g, rb, colour, ns, st);
    else rb_pass_s<R, false, false>(pdl, S, gp, g, rb, colour, ns, st);
}

// scratch buffers are passed through Sys-aligned array set by the host
template <typename R>
int launch_adlbl3_scr(const GeoT<R>& g, const Sys<R>* sys, const AdiScratch<R>* scr, int nsys, int mode, cudaStream_t st,
                      int rb_flags) {
    AdiBatch<R> b;
    b.nsys = nsys;
    for (int e = 0; e < 8; ++e) b.wy[e] = 0;
    int max_np = 1, max_lines = 1;
    for (int e = 0; e < nsys; ++e) {
        b.sys[e] = sys[e];
        b.scr[e] = scr[e];
        int np = (sys[e].ie - sys[e].ib) / 2 + 1;
        int nl = (sys[e].ke - sys[e].kb) / 2 + 1 + (sys[e].je - sys[e].jb) / 2 + 1;
        max_np = np > max_np ? np : max_np;
        max_lines = nl > max_lines ? nl : max_lines;
    }
    int threads = ((max_lines + 31) / 32) * 32;
    if (threads > 1024) threads = 1024;
    if (threads < 64) threads = 64;
    if (mode == GFM_ADI_MARCH) {
        if (threads > kMarchThreads) threads = kMarchThreads;
        if (march_rows() != 1 && !march_contiguous()) {
            // the CTA size and, per system, the layout of least cost
            // (march_layout_cost); the batch's systems run side by side
            long long best = -1;
            int best_warps = threads / 32, best_wy[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            for (int warps : {4, 8, threads / 32}) {   // on a tie, the first
                if (warps * 32 > kMarchThreads) continue;
                long long worst = 0;
                int wy[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                for (int e = 0; e < nsys; ++e) {
                    const int nJ = (sys[e].je - sys[e].jb) / 2 + 1, nK = (sys[e].ke - sys[e].kb) / 2 + 1;
                    long long c = march_layout_cost(nJ, nK, warps, 0);
                    for (int y = 1; y < warps; ++y) {
                        const long long cy = march_layout_cost(nJ, nK, warps, y);
                        if (cy < c) { c = cy; wy[e] = y; }
                    }
                    worst = std::max(worst, c);
                }
                if (best < 0 || worst < best) {
                    best = worst;
                    best_warps = warps;
                    for (int e = 0; e < 8; ++e) best_wy[e] = wy[e];
                }
            }
            threads = best_warps * 32;
            for (int e = 0; e < 8; ++e) b.wy[e] = best_wy[e];
        }
        size_t plane = 0;   // the largest plane of the batch
        for (int e = 0; e < nsys; ++e) {
            const size_t p = (size_t)((sys[e].je - sys[e].jb) / 2 + 1) * ((sys[e].ke - sys[e].kb) / 2 + 1);
            plane = p > plane ? p : plane;
        }
        const size_t smem = 4 * plane * sizeof(R);
        if (march_rows() == 1) k_adlbl3_march<R, 1, false><<<nsys, threads, 0, st>>>(g, b);
        else if (smem <= kMarchMaxSmem) {
            // pivots of the call first, then the march dividing once per row
            int lines = 1;
            for (int e = 0; e < nsys; ++e)
                lines = std::max(lines, ((sys[e].ie - sys[e].ib) / 2 + 1) *
                                            ((sys[e].ke - sys[e].kb) / 2 + 1 + (sys[e].je - sys[e].jb) / 2 + 1));
            k_march_pivots<R><<<dim3((lines + 127) / 128, nsys), 128, 0, st>>>(g, b);
            k_adlbl3_march<R, 4, true, true><<<nsys, threads, smem, st>>>(g, b);
            return 2;
        }
        else k_adlbl3_march<R, 4, false><<<nsys, threads, 0, st>>>(g, b);
        return 1;
    } else {
        RbBatch<R> rb;
        rb.nsys = nsys;
        long long max_lines = 0, max_cells = 0, max_slots = 0, max_np = 1, max_rows = 1;
        const long long max_class = (long long)g.HX * g.HY * g.HZ;
        int nim = 0, max_n = 1;
        for (int e = 0; e < nsys; ++e) {
            rb.sys[e] = sys[e];
            rb.scr[e] = scr[e];
            const Sys<R>& q = sys[e];
            long long np_ = (q.ie - q.ib) / 2 + 1, nK = (q.ke - q.kb) / 2 + 1, nJ = (q.je - q.jb) / 2 + 1;
            max_lines = np_ * (nK + nJ) > max_lines ? np_ * (nK + nJ) : max_lines;
            max_cells = np_ * nK * nJ > max_cells ? np_ * nK * nJ : max_cells;
            max_slots = (np_ + 1) / 2 * (nK + nJ) > max_slots ? (np_ + 1) / 2 * (nK + nJ) : max_slots;
            max_np = np_ > max_np ? np_ : max_np;
            max_rows = nK * nJ > max_rows ? nK * nJ : max_rows;
            max_n = (int)(nK > max_n ? nK : max_n);
            max_n = (int)(nJ > max_n ? nJ : max_n);
            nim = q.nim > nim ? q.nim : nim;
        }
        auto blocks = [](long long n, int t) { long long b = (n + t - 1) / t; return (unsigned)(b < 1 ? 1 : (b > 4096 ? 4096 : b)); };
        const bool pdl = (rb_flags & kRbPdl) != 0;
        if (rb_flags & kRbPlane) {
            const int n = launch_rbp(g, sys, scr, nsys, st, rb_flags);
            if (n > 0) return n;
        }
        const int S = rb_segments<R>(max_n);
        const bool avg2 = (rb_flags & kRbAvgInPass) != 0;            // pass L=2 averages pass L=1
        launch_k(pdl, k_rbs_in<R>, dim3(blocks(max_class, 256), nsys), 256, 0, st, g, rb);
        launch_k(pdl, k_rbs_factor<R>, dim3(blocks(max_lines, 128), nsys), 128, 0, st, g, rb);
        // line slots of one colour: ceil(planes/2) x (nK + nJ), 32 per block
        const dim3 gp((unsigned)((max_slots + 31) / 32), nsys);
        const dim3 ga((unsigned)((max_np + 1) / 2 + 31) / 32, nsys, (unsigned)((max_rows + 8 * kAvgRows - 1) / (8 * kAvgRows)));
        for (int ns = 0; ns < nim; ++ns)
            for (int half = 0; half < 2; ++half)
                for (int colour = 0; colour < 2; ++colour) {
                    rb_pass<R>(pdl, S, true, false, gp, g, rb, colour, ns, st);
                    if (!avg2) launch_k(pdl, k_rbs_avg<R>, ga, dim3(32, 8), 0, st, g, rb, colour, ns, 0);
                    rb_pass<R>(pdl, S, false, avg2, gp, g, rb, colour, ns, st);
                    launch_k(pdl, k_rbs_avg<R>, ga, dim3(32, 8), 0, st, g, rb, colour, ns, 1);
                }
        launch_k(pdl, k_rbs_out<R>, dim3(blocks(max_cells, 256), nsys), 256, 0, st, g, rb);
        return 3 + (avg2 ? 12 : 16) * nim;
    }
}

// raise the shared-memory limits of the line-solver kernels once, before any capture
int prepare_line_solver() {
    const bool ok = cudaFuncSetAttribute(k_adlbl3_march<float, 4, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kMarchMaxSmem) == cudaSuccess &&
                    cudaFuncSetAttribute(k_adlbl3_march<double, 4, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kMarchMaxSmem) == cudaSuccess;
    return ok ? prepare_rbp() : GFM_E_CUDA;
}

template <typename R>
void launch_refine_rhs(const GeoT<R>& g, const Sys<R>& s, R* rhs, cudaStream_t st) {
    const long long n = (long long)((s.ie - s.ib) / 2 + 1) * ((s.je - s.jb) / 2 + 1) * ((s.ke - s.kb) / 2 + 1);
    long long nb = (n + 255) / 256;
    k_refine_rhs<R><<<(int)(nb < 1 ? 1 : (nb > 4096 ? 4096 : nb)), 256, 0, st>>>(g, s, rhs);
}
template <typename R>
void launch_refine_add(const GeoT<R>& g, const Sys<R>& s, const R* dx, cudaStream_t st) {
    const long long n = (long long)((s.ie - s.ib) / 2 + 1) * ((s.je - s.jb) / 2 + 1) * ((s.ke - s.kb) / 2 + 1);
    long long nb = (n + 255) / 256;
    k_refine_add<R><<<(int)(nb < 1 ? 1 : (nb > 4096 ? 4096 : nb)), 256, 0, st>>>(g, s, dx);
}
template void launch_refine_rhs<float>(const GeoT<float>&, const Sys<float>&, float*, cudaStream_t);
template void launch_refine_rhs<double>(const GeoT<double>&, const Sys<double>&, double*, cudaStream_t);
template void launch_refine_add<float>(const GeoT<float>&, const Sys<float>&, const float*, cudaStream_t);
template void launch_refine_add<double>(const GeoT<double>&, const Sys<double>&, const double*, cudaStream_t);
template void launch_residual<double>(const Ctx<double>&, const Sys<double>&, int, cudaStream_t);
template void launch_residual<float>(const Ctx<float>&, const Sys<float>&, int, cudaStream_t);
template int launch_adlbl3_scr<double>(const GeoT<double>&, const Sys<double>*, const AdiScratch<double>*, int, int,
                                       cudaStream_t, int);
template int launch_adlbl3_scr<float>(const GeoT<float>&, const Sys<float>*, const AdiScratch<float>*, int, int, cudaStream_t,
                                      int);

}  // namespace gfm
