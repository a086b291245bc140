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
// calc_residual: per-cell |sum a_nb x_nb + b - a_p x| / max(terms)
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_residual(GeoT<R> g, Sys<R> s, double* partials, int slot) {
    __shared__ double sh[32];
    const int ni = (s.ie - s.ib) / 2 + 1, nj = (s.je - s.jb) / 2 + 1, nk = (s.ke - s.kb) / 2 + 1;
    const long long n = (long long)ni * nj * nk;
    double acc = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int i = s.ib + 2 * (int)(t % ni);
        long long r = t / ni;
        int j = s.jb + 2 * (int)(r % nj), k = s.kb + 2 * (int)(r / nj);
        long long o = pidx(g, i, j, k);
        if (g.ib[o] > 0) continue;
        double t1 = (double)s.as[0][o] * (double)A(s.xt, i - 2, j, k), t2 = (double)s.as[1][o] * (double)A(s.xt, i + 2, j, k);
        double t3 = (double)s.as[2][o] * (double)A(s.xt, i, j - 2, k), t4 = (double)s.as[3][o] * (double)A(s.xt, i, j + 2, k);
        double t5 = (double)s.as[4][o] * (double)A(s.xt, i, j, k - 2), t6 = (double)s.as[5][o] * (double)A(s.xt, i, j, k + 2);
        double t7 = (double)s.ap[o] * (double)s.xt[o], t8 = (double)s.bs[o];
        double em = fabs(t1);
        em = fabs(t2) > em ? fabs(t2) : em; em = fabs(t3) > em ? fabs(t3) : em; em = fabs(t4) > em ? fabs(t4) : em;
        em = fabs(t5) > em ? fabs(t5) : em; em = fabs(t6) > em ? fabs(t6) : em; em = fabs(t7) > em ? fabs(t7) : em;
        em = fabs(t8) > em ? fabs(t8) : em;
        acc += fabs(t1 + t2 + t3 + t4 + t5 + t6 + t8 - t7) / em;   // 0/0 -> NaN as in the reference
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
        int per_colour = (max_np + 1) / 2;
        int nim = 0;
        for (int e = 0; e < nsys; ++e) nim = sys[e].nim > nim ? sys[e].nim : nim;
        // equations with fewer sweeps drop out of later launches
        for (int ns = 0; ns < nim; ++ns)
            for (int half = 0; half < 2; ++half) {
                k_adlbl3_rb<R><<<nsys * per_colour, threads, 0, st>>>(g, b, 0, per_colour, ns);
                k_adlbl3_rb<R><<<nsys * per_colour, threads, 0, st>>>(g, b, 1, per_colour, ns);
            }
    }
}

template void launch_residual<double>(const Ctx<double>&, const Sys<double>&, int, cudaStream_t);
template void launch_residual<float>(const Ctx<float>&, const Sys<float>&, int, cudaStream_t);
template void launch_adlbl3_scr<double>(const GeoT<double>&, const Sys<double>*, const AdiScratch<double>*, int, int, cudaStream_t);
template void launch_adlbl3_scr<float>(const GeoT<float>&, const Sys<float>*, const AdiScratch<float>*, int, int, cudaStream_t);

}  // namespace gfm
