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
//   GFM_ADI_REDBLACK all even planes at once, then all odd planes (twice per
//                    sweep, NIM sweeps), one CTA per (equation, plane).
// Scratch: PT of the y-lines and of the z-lines, and the pass results XT2/XT3,
// live in per-equation class-sized device buffers (QT is stored in XT2/XT3 and
// back-substituted in place).
#include "state.cuh"

namespace gfm {

#define A(arr, I, J, K) (arr)[pidx(g, (I), (J), (K))]

// y-line Thomas (ADLZY, Adlbl3.f90:147-181): writes XT2 for line (I,*,K)
template <typename R, bool EXACT_DIV>
__device__ void adlzy(const GeoT<R>& g, const Sys<R>& s, const AdiScratch<R>& w, int I, int IPL, int IML, int K) {
    const int LD = 2;
    const int KPL = K + LD, KML = K - LD;
    const int JBML = s.jb - LD;
    R pt_prev = R(0);
    R qt_prev = A(s.xt, I, JBML, K);
    for (int J = s.jb; J <= s.je; J += LD) {
        const long long o = pidx(g, I, J, K);
        R alp = s.ap[o] - pt_prev * s.as[2][o];
        R bsy = s.bs[o];
        R pt, qt;
        if (fabs(alp) <= R(1.0e-20) || g.ib[o] >= 1) {
            pt = R(0);
            qt = s.xt[o];
        } else {
            bsy = bsy + s.as[1][o] * A(s.xt, IPL, J, K) + s.as[0][o] * A(s.xt, IML, J, K);
            bsy = bsy + s.as[5][o] * A(s.xt, I, J, KPL) + s.as[4][o] * A(s.xt, I, J, KML);
            if (EXACT_DIV) {
                pt = s.as[3][o] / alp;
                qt = (bsy + s.as[2][o] * qt_prev) / alp;
            } else {
                R ra = R(1) / alp;
                pt = s.as[3][o] * ra;
                qt = (bsy + s.as[2][o] * qt_prev) * ra;
            }
        }
        w.pty[o] = pt;
        w.xt2[o] = qt;
        pt_prev = pt;
        qt_prev = qt;
    }
    R nxt = A(s.xt, I, s.je + LD, K);   // XT2(JEPL) = XT(I,JEPL,K), never updated
    for (int J = s.je; J >= s.jb; J -= LD) {
        const long long o = pidx(g, I, J, K);
        R v = nxt * w.pty[o] + w.xt2[o];
        w.xt2[o] = v;
        nxt = v;
    }
}

// z-line Thomas (ADLYZ, Adlbl3.f90:187-221): writes XT3 for line (I,J,*)
template <typename R, bool EXACT_DIV>
__device__ void adlyz(const GeoT<R>& g, const Sys<R>& s, const AdiScratch<R>& w, int I, int IPL, int IML, int J) {
    const int LD = 2;
    const int JPL = J + LD, JML = J - LD;
    const int KBML = s.kb - LD;
    R pt_prev = R(0);
    R qt_prev = A(s.xt, I, J, KBML);
    for (int K = s.kb; K <= s.ke; K += LD) {
        const long long o = pidx(g, I, J, K);
        R alp = s.ap[o] - pt_prev * s.as[4][o];
        R bsy = s.bs[o];
        R pt, qt;
        if (fabs(alp) <= R(1.0e-20) || g.ib[o] >= 1) {
            pt = R(0);
            qt = s.xt[o];
        } else {
            bsy = bsy + s.as[1][o] * A(s.xt, IPL, J, K) + s.as[0][o] * A(s.xt, IML, J, K);
            bsy = bsy + s.as[3][o] * A(s.xt, I, JPL, K) + s.as[2][o] * A(s.xt, I, JML, K);
            if (EXACT_DIV) {
                pt = s.as[5][o] / alp;
                qt = (bsy + s.as[4][o] * qt_prev) / alp;
            } else {
                R ra = R(1) / alp;
                pt = s.as[5][o] * ra;
                qt = (bsy + s.as[4][o] * qt_prev) * ra;
            }
        }
        w.ptz[o] = pt;
        w.xt3[o] = qt;
        pt_prev = pt;
        qt_prev = qt;
    }
    R nxt = A(s.xt, I, J, s.ke + LD);   // XT3(KEPL) = XT(I,J,KEPL)
    for (int K = s.ke; K >= s.kb; K -= LD) {
        const long long o = pidx(g, I, J, K);
        R v = nxt * w.ptz[o] + w.xt3[o];
        w.xt3[o] = v;
        nxt = v;
    }
}

// ADLZ (Adlbl3.f90:103-141) on plane I by the whole CTA.
template <typename R, bool EXACT_DIV>
__device__ void adlz(const GeoT<R>& g, const Sys<R>& s, const AdiScratch<R>& w, int I) {
    const int LD = 2;
    const int IPL = I + LD, IML = I - LD;
    const int nK = (s.ke - s.kb) / LD + 1, nJ = (s.je - s.jb) / LD + 1;
    for (int L = 1; L <= 2; ++L) {
        for (int t = threadIdx.x; t < nK + nJ; t += blockDim.x) {
            if (t < nK) adlzy<R, EXACT_DIV>(g, s, w, I, IPL, IML, s.kb + LD * t);
            else adlyz<R, EXACT_DIV>(g, s, w, I, IPL, IML, s.jb + LD * (t - nK));
        }
        __syncthreads();
        for (int t = threadIdx.x; t < nK * nJ; t += blockDim.x) {
            int K = s.kb + LD * (t / nJ), J = s.jb + LD * (t % nJ);
            long long o = pidx(g, I, J, K);
            s.xt[o] = (w.xt2[o] + w.xt3[o]) / R(2);
        }
        __syncthreads();
    }
}

template <typename R>
struct AdiBatch {
    Sys<R> sys[8];
    AdiScratch<R> scr[8];
    int nsys;
};

// reference march: one CTA per equation
template <typename R>
__global__ void k_adlbl3_march(GeoT<R> g, AdiBatch<R> b) {
    const Sys<R>& s = b.sys[blockIdx.x];
    const AdiScratch<R>& w = b.scr[blockIdx.x];
    for (int ns = 0; ns < s.nim; ++ns) {
        for (int I = s.ib; I <= s.ie; I += 2) adlz<R, true>(g, s, w, I);
        for (int I = s.ie; I >= s.ib; I -= 2) adlz<R, true>(g, s, w, I);
    }
}

// red-black: one CTA per (equation, plane of the requested colour)
template <typename R>
__global__ void k_adlbl3_rb(GeoT<R> g, AdiBatch<R> b, int colour, int max_planes, int sweep) {
    int e = blockIdx.x / max_planes, pl = blockIdx.x % max_planes;
    if (e >= b.nsys) return;
    const Sys<R>& s = b.sys[e];
    if (sweep >= s.nim) return;
    int npl = (s.ie - s.ib) / 2 + 1;
    int p = 2 * pl + colour;
    if (p >= npl) return;
    adlz<R, false>(g, s, b.scr[e], s.ib + 2 * p);
}

// ---------------------------------------------------------------------------
// Red-black form.  The tridiagonal matrix of every y- and z-line is constant
// during one ADLBL3 call, so its Thomas pivots are factored once: PT (as in
// ADLZY/ADLYZ) and IA = 1/ALP, with IA = 0 marking the rows the reference
// copies unchanged (|ALP| <= 1e-20 or a blocked cell).  Within one plane visit
// the x-neighbour part of the right-hand side, BS + AS12*XT(I+2) +
// AS11*XT(I-2), is constant (neighbour planes have the other colour) and is
// summed first, as the reference does.  Threads map to (plane, line) with the
// plane index fastest, so each step of the sequential line recurrence reads
// consecutive same-colour planes: coalesced across the warp.
// ---------------------------------------------------------------------------
template <typename R>
struct RbBatch {
    Sys<R> sys[8];
    AdiScratch<R> scr[8];
    int nsys;
};

__device__ __forceinline__ int rb_nplanes(int ib, int ie) { return (ie - ib) / 2 + 1; }

// factor every y-line and z-line of every plane (both colours)
template <typename R>
__global__ void k_rb_factor(GeoT<R> g, RbBatch<R> b) {
    const Sys<R>& s = b.sys[blockIdx.y];
    const AdiScratch<R>& w = b.scr[blockIdx.y];
    const int npl = rb_nplanes(s.ib, s.ie), nK = (s.ke - s.kb) / 2 + 1, nJ = (s.je - s.jb) / 2 + 1;
    const long long ny = (long long)npl * nK, nz = (long long)npl * nJ;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ny + nz; t += (long long)gridDim.x * blockDim.x) {
        if (t < ny) {
            const int I = s.ib + 2 * (int)(t % npl), K = s.kb + 2 * (int)(t / npl);
            R pt_prev = R(0);
            for (int J = s.jb; J <= s.je; J += 2) {
                const long long o = pidx(g, I, J, K);
                R alp = s.ap[o] - pt_prev * s.as[2][o];
                R pt, ia;
                if (fabs(alp) <= R(1.0e-20) || g.ib[o] >= 1) { pt = R(0); ia = R(0); }
                else { pt = s.as[3][o] / alp; ia = R(1) / alp; }
                w.pty[o] = pt;
                w.iay[o] = ia;
                pt_prev = pt;
            }
        } else {
            const long long u = t - ny;
            const int I = s.ib + 2 * (int)(u % npl), J = s.jb + 2 * (int)(u / npl);
            R pt_prev = R(0);
            for (int K = s.kb; K <= s.ke; K += 2) {
                const long long o = pidx(g, I, J, K);
                R alp = s.ap[o] - pt_prev * s.as[4][o];
                R pt, ia;
                if (fabs(alp) <= R(1.0e-20) || g.ib[o] >= 1) { pt = R(0); ia = R(0); }
                else { pt = s.as[5][o] / alp; ia = R(1) / alp; }
                w.ptz[o] = pt;
                w.iaz[o] = ia;
                pt_prev = pt;
            }
        }
    }
}

// One line of one pass, software-pipelined: the inputs of D consecutive
// steps are loaded before the dependent recurrence runs over them, so a thread
// keeps ~D x 8 independent loads in flight.  Consecutive elements of a y-line
// are PX apart, of a z-line PX*HY apart; x-neighbours I+-2 are +-1.  Offsets
// are 32-bit (a parity-split field holds < 2^31 elements, checked at create).
template <typename R> struct Pipe { static constexpr int D = 8; };
template <> struct Pipe<double> { static constexpr int D = 4; };

template <typename R, bool FIRST, bool ZLINE>
__device__ __forceinline__ void rb_line(const R* __restrict__ xt, const R* __restrict__ bs, const R* __restrict__ a_xp,
                                        const R* __restrict__ a_xm, const R* __restrict__ a_op, const R* __restrict__ a_om,
                                        const R* __restrict__ a_sub, const R* __restrict__ ia, const R* __restrict__ pt,
                                        R* __restrict__ bsx, R* __restrict__ out, int o0, int step, int ostep, int n) {
    constexpr int D = Pipe<R>::D;
    R qt_prev = xt[o0 - step];
    int c = 0, o = o0;
    for (; c + D <= n; c += D, o += D * step) {
        R vb[D], vo1[D], vo2[D], vx1[D], vx2[D], vs[D], vi[D], vc[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const int q = o + d * step;
            if (FIRST) vb[d] = bs[q] + a_xp[q] * xt[q + 1] + a_xm[q] * xt[q - 1];
            else vb[d] = bsx[q];
            vo1[d] = a_op[q]; vo2[d] = a_om[q];
            vx1[d] = xt[q + ostep]; vx2[d] = xt[q - ostep];
            vs[d] = a_sub[q]; vi[d] = ia[q]; vc[d] = xt[q];
        }
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const int q = o + d * step;
            if (FIRST && !ZLINE) bsx[q] = vb[d];
            R qt = vi[d] == R(0) ? vc[d] : ((vb[d] + vo1[d] * vx1[d] + vo2[d] * vx2[d]) + vs[d] * qt_prev) * vi[d];
            out[q] = qt;
            qt_prev = qt;
        }
    }
    for (; c < n; ++c, o += step) {
        R b = FIRST ? bs[o] + a_xp[o] * xt[o + 1] + a_xm[o] * xt[o - 1] : bsx[o];
        if (FIRST && !ZLINE) bsx[o] = b;
        const R iv = ia[o];
        R qt = iv == R(0) ? xt[o] : ((b + a_op[o] * xt[o + ostep] + a_om[o] * xt[o - ostep]) + a_sub[o] * qt_prev) * iv;
        out[o] = qt;
        qt_prev = qt;
    }
    // back-substitution from the far boundary
    R nxt = xt[o0 + n * step];
    c = n - 1;
    o = o0 + c * step;
    for (; c + 1 >= D; c -= D, o -= D * step) {
        R vp[D], vq[D];
#pragma unroll
        for (int d = 0; d < D; ++d) { vp[d] = pt[o - d * step]; vq[d] = out[o - d * step]; }
#pragma unroll
        for (int d = 0; d < D; ++d) {
            R v = nxt * vp[d] + vq[d];
            out[o - d * step] = v;
            nxt = v;
        }
    }
    for (; c >= 0; --c, o -= step) {
        R v = nxt * pt[o] + out[o];
        out[o] = v;
        nxt = v;
    }
}

// one pass (both directions) over the planes of one colour; the first pass of a
// visit (L=1) computes BSX (y-lines store it), the second reads it
template <typename R, bool FIRST>
__global__ void k_rb_pass(GeoT<R> g, RbBatch<R> b, int colour, int sweep) {
    const Sys<R>& s = b.sys[blockIdx.y];
    if (sweep >= s.nim) return;
    const AdiScratch<R>& w = b.scr[blockIdx.y];
    const int npl = rb_nplanes(s.ib, s.ie);
    const int npc = (npl - colour + 1) / 2;   // planes of this colour
    const int nK = (s.ke - s.kb) / 2 + 1, nJ = (s.je - s.jb) / 2 + 1;
    const long long ny = (long long)npc * nK, nz = (long long)npc * nJ;
    const int sy = g.PX, sz = g.PX * g.HY;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ny + nz; t += (long long)gridDim.x * blockDim.x) {
        if (t < ny) {
            const int I = s.ib + 2 * (2 * (int)(t % npc) + colour), K = s.kb + 2 * (int)(t / npc);
            rb_line<R, FIRST, false>(s.xt, s.bs, s.as[1], s.as[0], s.as[5], s.as[4], s.as[2], w.iay, w.pty, w.bsx, w.xt2,
                                     (int)pidx(g, I, s.jb, K), sy, sz, nJ);
        } else {
            const long long u = t - ny;
            const int I = s.ib + 2 * (2 * (int)(u % npc) + colour), J = s.jb + 2 * (int)(u / npc);
            rb_line<R, FIRST, true>(s.xt, s.bs, s.as[1], s.as[0], s.as[3], s.as[2], s.as[4], w.iaz, w.ptz, w.bsx, w.xt3,
                                    (int)pidx(g, I, J, s.kb), sz, sy, nK);
        }
    }
}

// XT = (XT2 + XT3)/2 on the planes of one colour
template <typename R>
__global__ void k_rb_avg(GeoT<R> g, RbBatch<R> b, int colour, int sweep) {
    const Sys<R>& s = b.sys[blockIdx.y];
    if (sweep >= s.nim) return;
    const AdiScratch<R>& w = b.scr[blockIdx.y];
    const int npl = rb_nplanes(s.ib, s.ie);
    const int npc = (npl - colour + 1) / 2;
    const int nK = (s.ke - s.kb) / 2 + 1, nJ = (s.je - s.jb) / 2 + 1;
    const long long n = (long long)npc * nJ * nK;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int I = s.ib + 2 * (2 * (int)(t % npc) + colour);
        const long long r = t / npc;
        const int J = s.jb + 2 * (int)(r % nJ), K = s.kb + 2 * (int)(r / nJ);
        const long long o = pidx(g, I, J, K);
        s.xt[o] = (w.xt2[o] + w.xt3[o]) / R(2);
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

// scratch buffers are passed through Sys-aligned array set by the host
template <typename R>
void launch_adlbl3_scr(const GeoT<R>& g, const Sys<R>* sys, const AdiScratch<R>* scr, int nsys, int mode, cudaStream_t st) {
    AdiBatch<R> b;
    b.nsys = nsys;
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
        k_adlbl3_march<R><<<nsys, threads, 0, st>>>(g, b);
    } else {
        RbBatch<R> rb;
        rb.nsys = nsys;
        long long max_lines = 0, max_cells = 0;
        int nim = 0;
        for (int e = 0; e < nsys; ++e) {
            rb.sys[e] = sys[e];
            rb.scr[e] = scr[e];
            const Sys<R>& q = sys[e];
            long long np_ = (q.ie - q.ib) / 2 + 1, nK = (q.ke - q.kb) / 2 + 1, nJ = (q.je - q.jb) / 2 + 1;
            max_lines = np_ * (nK + nJ) > max_lines ? np_ * (nK + nJ) : max_lines;
            max_cells = np_ * nK * nJ > max_cells ? np_ * nK * nJ : max_cells;
            nim = q.nim > nim ? q.nim : nim;
        }
        const int T = 128;
        dim3 gf((unsigned)((max_lines + T - 1) / T), nsys);
        k_rb_factor<R><<<gf, T, 0, st>>>(g, rb);
        dim3 gp((unsigned)((max_lines / 2 + T) / T), nsys);
        dim3 ga((unsigned)((max_cells / 2 + 255) / 256 < 2048 ? (max_cells / 2 + 255) / 256 : 2048), nsys);
        for (int ns = 0; ns < nim; ++ns)
            for (int half = 0; half < 2; ++half)
                for (int colour = 0; colour < 2; ++colour) {
                    k_rb_pass<R, true><<<gp, T, 0, st>>>(g, rb, colour, ns);
                    k_rb_avg<R><<<ga, 256, 0, st>>>(g, rb, colour, ns);
                    k_rb_pass<R, false><<<gp, T, 0, st>>>(g, rb, colour, ns);
                    k_rb_avg<R><<<ga, 256, 0, st>>>(g, rb, colour, ns);
                }
    }
}

template void launch_residual<double>(const Ctx<double>&, const Sys<double>&, int, cudaStream_t);
template void launch_residual<float>(const Ctx<float>&, const Sys<float>&, int, cudaStream_t);
template void launch_adlbl3_scr<double>(const GeoT<double>&, const Sys<double>*, const AdiScratch<double>*, int, int, cudaStream_t);
template void launch_adlbl3_scr<float>(const GeoT<float>&, const Sys<float>*, const AdiScratch<float>*, int, int, cudaStream_t);

}  // namespace gfm
