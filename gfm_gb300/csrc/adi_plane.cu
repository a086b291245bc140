// adi_plane.cu -- the red-black line solver (GFM_ADI_REDBLACK) with one CTA
// per plane visit: ADLZ (Adlbl3.f90:103-141) of one x-plane, both passes
// L = 1, 2 with their averages, in shared memory.
//
// Per ADLBL3 call (Adlbl3.f90:10-97) the system is rewritten once into
// plane-major arrays:
//
//   XP  the unknown with a one-point border on every side, plane p of the
//       class (I = IB + 2p, p = -1 .. npl) holding (nJ+2) x (nK+2) points,
//       K fastest: element (p, jj, kk) at ((p+1)(nJ+2) + jj+1)(nK+2) + kk+1;
//   YC, YX, YP  the rows of the y-lines (I, *, K), K fastest within the plane
//       ((p nJ + jj) nK + kk): YC = (AS21, AS31, AS32, BS), YX = (AS11, AS12)
//       and YP = (1/ALP, PT) with the Thomas pivots of the line,
//       ALP = AP - PT(prev) AS21, PT = AS22/ALP (ADLZY, Adlbl3.f90:147-181);
//   ZC, ZP  the rows of the z-lines (I, J, *), J fastest ((p nK + kk) nJ + jj):
//       ZC = (AS31, AS21, AS22, -), ZP = (1/ALP, PT) with ALP = AP - PT(prev)
//       AS31, PT = AS32/ALP (ADLYZ, Adlbl3.f90:187-221).
//
// The matrices do not change during the call, so the pivots are the values
// every visit of the reference would form.  A row the reference copies
// unchanged (|ALP| <= 1e-20 or a blocked cell) stores 1/ALP = 0 and PT = -0.0,
// a value no other row stores.  The coefficients are rewritten by a tiled
// transpose (k_rbp_fill); the pivots by one thread per line walking its rows
// (k_rbp_pivots), with the loads of the next rows in flight while the chain
// runs over the current ones.
//
// A visit (k_rbp_visit) loads its plane of XP into shared memory, runs the
// y-lines of pass L=1 (which also form the x-neighbour part of the right-hand
// side, BX = BS + AS12 XT(I+2) + AS11 XT(I-2), fixed for the visit since the
// other colour does not move), the z-lines of pass L=1 averaging into the
// y-line results, then pass L=2 the same way from that average, and writes the
// plane back.  The lines of a pass are cut into segments: lanes of a warp take
// 32 neighbouring lines (so a warp's loads of one row are contiguous in the
// record layout of that direction), warps take segments of at most M rows, and
// the affine recurrences of the forward elimination and the back substitution
// are joined across segments by a scan of the segment maps in shared memory.
// Each visit thus reads the records of its plane once from DRAM (pass L=2
// finds them in L2) and the intermediate results never leave the SM.
#include <algorithm>

#include "state.cuh"

namespace gfm {

namespace {

template <typename R>
struct __align__(2 * sizeof(R)) Pair { R x, y; };

template <typename R>
struct RbpBatch {
    Sys<R> sys[8];
    R* xp[8];
    Quad<R>* yc[8];
    Pair<R>* yx[8];
    Pair<R>* yp[8];
    Quad<R>* zc[8];
    Pair<R>* zp[8];
    int nsys;
};

struct PlaneDims {
    int npl, nJ, nK;
};
template <typename R>
__host__ __device__ __forceinline__ PlaneDims dims_of(const Sys<R>& s) {
    return PlaneDims{(s.ie - s.ib) / 2 + 1, (s.je - s.jb) / 2 + 1, (s.ke - s.kb) / 2 + 1};
}
__host__ __device__ __forceinline__ int xp_index(const PlaneDims& d, int p, int jj, int kk) {
    return ((p + 1) * (d.nJ + 2) + jj + 1) * (d.nK + 2) + kk + 1;
}
// the copy-row marker PT = -0.0
__device__ __forceinline__ bool rbp_copy(float pt) { return __float_as_uint(pt) == 0x80000000u; }
__device__ __forceinline__ bool rbp_copy(double pt) {
    return (unsigned long long)__double_as_longlong(pt) == 0x8000000000000000ull;
}

// ---------------------------------------------------------------------------
// XT <-> XP, through a 32 x 32 tile in shared memory: plane index fastest on
// the class side, K fastest on the plane side.  Block (32, 8); grid x over
// (plane tiles) x (K tiles), y = J row of XP (border included), z = system.
// ---------------------------------------------------------------------------
template <typename R, bool IN>
__global__ void k_rbp_copy(GeoT<R> g, RbpBatch<R> b) {
    __shared__ R tile[32][33];
    pdl_wait();
    pdl_trigger();
    const Sys<R>& s = b.sys[blockIdx.z];
    const PlaneDims d = dims_of(s);
    // IN copies the border too (planes -1..npl, rows -1..nJ, -1..nK); OUT the interior
    const int o = IN ? 1 : 0;
    const int np = d.npl + 2 * o, nj = d.nJ + 2 * o, nk = d.nK + 2 * o;
    const int jr = blockIdx.y;
    if (jr >= nj) return;
    const int ntp = (np + 31) / 32;
    const int p0 = (blockIdx.x % ntp) * 32, k0 = (blockIdx.x / ntp) * 32;
    if (k0 >= nk) return;
    const int J = s.jb + 2 * (jr - o);
    R* __restrict__ xp = b.xp[blockIdx.z];
    const int tx = threadIdx.x, ty = threadIdx.y;
    if (IN) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int kr = k0 + ty + 8 * r, pr = p0 + tx;
            if (kr < nk && pr < np)
                tile[ty + 8 * r][tx] = s.xt[pidx(g, s.ib + 2 * (pr - o), J, s.kb + 2 * (kr - o))];
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int pr = p0 + ty + 8 * r, kr = k0 + tx;
            if (kr < nk && pr < np) xp[xp_index(d, pr - o, jr - o, kr - o)] = tile[tx][ty + 8 * r];
        }
    } else {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int pr = p0 + ty + 8 * r, kr = k0 + tx;
            if (kr < nk && pr < np) tile[tx][ty + 8 * r] = xp[xp_index(d, pr, jr, kr)];
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int kr = k0 + ty + 8 * r, pr = p0 + tx;
            if (kr < nk && pr < np) s.xt[pidx(g, s.ib + 2 * pr, J, s.kb + 2 * kr)] = tile[ty + 8 * r][tx];
        }
    }
}

// ---------------------------------------------------------------------------
// The coefficients of the records (YC, YX of the y-lines; ZC of the z-lines),
// once per call, through a 32-plane x 16-line tile in shared memory: read with
// the plane index fastest (contiguous in the class arrays), written with the
// line index fastest (contiguous in the records).  Block (32, 8); grid x over
// (plane tiles) x (line tiles), y = row (J of a y-line record, K of a z-line
// record), z = system.
// ---------------------------------------------------------------------------
template <typename R, bool ZL>
__device__ __forceinline__ void rbp_fill(const GeoT<R>& g, const RbpBatch<R>& b, int bx, R (*tile)[16][33]) {
    constexpr int NF = ZL ? 3 : 6;
    const int e = blockIdx.z;
    const Sys<R>& s = b.sys[e];
    const PlaneDims d = dims_of(s);
    const int nlines = ZL ? d.nJ : d.nK, nrows = ZL ? d.nK : d.nJ;
    const int row = blockIdx.y;
    if (row >= nrows) return;
    const int ntp = (d.npl + 31) / 32;
    const int p0 = (bx % ntp) * 32, l0 = (bx / ntp) * 16;
    if (l0 >= nlines) return;
    const int tx = threadIdx.x, ty = threadIdx.y;
    // y-line record: AS21, AS31, AS32, BS, AS11, AS12; z-line record: AS31, AS21, AS22
    const R* src[NF];
    if (ZL) {
        src[0] = s.as[4]; src[1] = s.as[2]; src[2] = s.as[3];
    } else {
        src[0] = s.as[2]; src[1] = s.as[4]; src[2] = s.as[5];
        src[3 % NF] = s.bs; src[4 % NF] = s.as[0]; src[5 % NF] = s.as[1];
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int ll = ty + 8 * r, p = p0 + tx, l = l0 + ll;
        if (p < d.npl && l < nlines) {
            const int I = s.ib + 2 * p;
            const int o = (int)(ZL ? pidx(g, I, s.jb + 2 * l, s.kb + 2 * row) : pidx(g, I, s.jb + 2 * row, s.kb + 2 * l));
#pragma unroll
            for (int f = 0; f < NF; ++f) tile[f][ll][tx] = src[f][o];
        }
    }
    __syncthreads();
    const int tid = ty * 32 + tx;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int idx = tid + 256 * r;
        const int ll = idx & 15, pl = idx >> 4;
        const int p = p0 + pl, l = l0 + ll;
        if (p < d.npl && l < nlines) {
            if (ZL) {
                b.zc[e][(p * d.nK + row) * d.nJ + l] = Quad<R>{tile[0][ll][pl], tile[1][ll][pl], tile[2][ll][pl], R(0)};
            } else {
                const int q = (p * d.nJ + row) * d.nK + l;
                b.yc[e][q] = Quad<R>{tile[0][ll][pl], tile[1][ll][pl], tile[2][ll][pl], tile[3 % NF][ll][pl]};
                b.yx[e][q] = Pair<R>{tile[4 % NF][ll][pl], tile[5 % NF][ll][pl]};
            }
        }
    }
}

// the y-line records in blocks [0, nyb) of grid x, the z-line records in
// the rest: both directions in one launch
template <typename R>
__global__ void __launch_bounds__(256) k_rbp_fill(GeoT<R> g, RbpBatch<R> b, int nyb) {
    __shared__ R tile[6][16][33];
    pdl_wait();
    pdl_trigger();
    if ((int)blockIdx.x < nyb) rbp_fill<R, false>(g, b, blockIdx.x, tile);
    else rbp_fill<R, true>(g, b, blockIdx.x - nyb, tile);
}

// ---------------------------------------------------------------------------
// Pivots of every line, once per call: a thread walks one line (plane p, a
// fixed cross index) row by row through the pivot chain of ADLZY/ADLYZ.
// Lanes take 32 neighbouring planes, so each row's loads are contiguous in
// the class arrays; the rows are taken kPivRows at a time, the loads of the
// next batch issued before the chain runs over the current one.  A batch's
// pivots leave through a tile in shared memory with the line index fastest,
// contiguous in the records.  Block (32, 8): 32 planes x 8 lines; grid x over
// (plane tiles) x (line tiles), y = system.  ZL: z-lines (rows along K, lines
// indexed by J), else y-lines (rows along J, lines indexed by K).
// ---------------------------------------------------------------------------
constexpr int kPivRows = 8;
template <typename R, bool ZL>
__device__ __forceinline__ void rbp_pivots(const GeoT<R>& g, const RbpBatch<R>& b, int bx,
                                           Pair<R> (*tile)[8][33]) {
    constexpr int C = kPivRows;
    const int e = blockIdx.y;
    const Sys<R>& s = b.sys[e];
    const PlaneDims d = dims_of(s);
    const int nlines = ZL ? d.nJ : d.nK, nrows = ZL ? d.nK : d.nJ;
    const int ntp = (d.npl + 31) / 32;
    const int p0 = (bx % ntp) * 32, l0 = (bx / ntp) * 8;
    if (l0 >= nlines) return;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int p = p0 + tx, l = l0 + ty;
    const bool act = p < d.npl && l < nlines;
    // y-line (I,*,K): sub AS21 = as[2], next AS22 = as[3]; z-line (I,J,*): sub AS31 = as[4], next AS32 = as[5]
    const R* __restrict__ a_sub = s.as[ZL ? 4 : 2];
    const R* __restrict__ a_next = s.as[ZL ? 5 : 3];
    const R* __restrict__ a_p = s.ap;
    const int8_t* __restrict__ ibc = g.ib;
    const int I = s.ib + 2 * p;
    const int ostep = ZL ? (int)(pidx(g, 0, 0, 2) - pidx(g, 0, 0, 0)) : (int)(pidx(g, 0, 2, 0) - pidx(g, 0, 0, 0));
    const int o0 = act ? (int)(ZL ? pidx(g, I, s.jb + 2 * l, s.kb) : pidx(g, I, s.jb, s.kb + 2 * l)) : 0;
    const int tid = ty * 32 + tx;
    R cap[C], csub[C], cnxt[C];
    bool cblk[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
        if (act && c < nrows) {
            const int o = o0 + c * ostep;
            cap[c] = a_p[o]; csub[c] = a_sub[o]; cnxt[c] = a_next[o]; cblk[c] = ibc[o] >= 1;
        }
    }
    R pt_prev = R(0);
    for (int r0 = 0; r0 < nrows; r0 += C) {
        R nap[C], nsub[C], nnxt[C];
        bool nblk[C];
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const int r = r0 + C + c;
            if (act && r < nrows) {
                const int o = o0 + r * ostep;
                nap[c] = a_p[o]; nsub[c] = a_sub[o]; nnxt[c] = a_next[o]; nblk[c] = ibc[o] >= 1;
            }
        }
#pragma unroll
        for (int c = 0; c < C; ++c) {
            if (act && r0 + c < nrows) {
                const R alp = cap[c] - pt_prev * csub[c];
                R ia, pt;
                if (fabs(alp) <= R(1.0e-20) || cblk[c]) {
                    ia = R(0);
                    pt = -R(0);
                    pt_prev = R(0);
                } else {
                    ia = R(1) / alp;
                    pt = cnxt[c] / alp + R(0);   // +0.0: no -0.0 here
                    pt_prev = pt;
                }
                tile[c][ty][tx] = Pair<R>{ia, pt};
            }
        }
        __syncthreads();
        // C rows x 8 lines x 32 planes, the line index fastest
#pragma unroll
        for (int i = 0; i < C; ++i) {
            const int idx = tid + 256 * i;
            const int ll = idx & 7, pl = (idx >> 3) & 31, c = idx >> 8;
            const int pw = p0 + pl, lw = l0 + ll, rw = r0 + c;
            if (pw < d.npl && lw < nlines && rw < nrows) {
                if (ZL) b.zp[e][(pw * d.nK + rw) * d.nJ + lw] = tile[c][ll][pl];
                else b.yp[e][(pw * d.nJ + rw) * d.nK + lw] = tile[c][ll][pl];
            }
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < C; ++c) {
            cap[c] = nap[c]; csub[c] = nsub[c]; cnxt[c] = nnxt[c]; cblk[c] = nblk[c];
        }
    }
}

// the y-line pivots in blocks [0, nyb) of grid x, the z-line pivots in the
// rest: both directions in one launch
template <typename R>
__global__ void __launch_bounds__(256) k_rbp_pivots(GeoT<R> g, RbpBatch<R> b, int nyb) {
    __shared__ Pair<R> tile[kPivRows][8][33];
    pdl_wait();
    pdl_trigger();
    if ((int)blockIdx.x < nyb) rbp_pivots<R, false>(g, b, blockIdx.x, tile);
    else rbp_pivots<R, true>(g, b, blockIdx.x - nyb, tile);
}

// ---------------------------------------------------------------------------
// One pass over the y-lines (ZL false) or the z-lines (ZL true) of the plane
// in shared memory.  src: the plane as before the pass (bordered, row pitch PS
// over K, J rows); dst: the y-line results (ZL false) or their average with the
// z-line results (ZL true), written into dst's interior.  FIRST: pass L=1 of a
// y-line forms BX from the record and the neighbouring planes and keeps it in
// bxs; otherwise BX is read from bxs.
// ---------------------------------------------------------------------------
template <typename R, int M, bool ZL, bool FIRST>
__device__ __forceinline__ void rbp_pass(const RbpBatch<R>& b, int e, const PlaneDims& d, int p, int PS,
                                         const R* __restrict__ src, R* __restrict__ dst, R* __restrict__ bxs,
                                         R* __restrict__ sA, R* __restrict__ sB) {
    const int nlines = ZL ? d.nJ : d.nK, n = ZL ? d.nK : d.nJ;
    const int G = (nlines + 31) >> 5;
    int S = ((int)(blockDim.x >> 5)) / G;
    S = S < 1 ? 1 : (S > n ? n : S);
    const int m = (n + S - 1) / S;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = warp % G, seg = warp / G;
    const int line = grp * 32 + lane;
    const bool active = seg < S && line < nlines;
    const int e0 = seg * m;
    int cnt = active ? n - e0 : 0;
    cnt = cnt < 0 ? 0 : (cnt > m ? m : cnt);
    // shared-memory offsets: (jj, kk) of the bordered plane at (jj+1)*PS + kk+1,
    // of bxs at jj*PS + kk; a row step and the two across-line neighbours
    const int rstep = ZL ? 1 : PS, across = ZL ? PS : 1;
    const int c0 = ZL ? (line + 1) * PS + 1 : PS + line + 1;   // row 0 of the line
    const int bx0 = ZL ? line * PS : line;
    const int bstep = ZL ? 1 : PS;
    R xlo = R(0), xhi = R(0);
    if (active) {
        xlo = src[c0 - rstep];
        xhi = src[c0 + n * rstep];
    }
    R rr[M], al[M], pv[M];
#pragma unroll
    for (int i = 0; i < M; ++i) {
        if (i < cnt) {
            const int row = e0 + i;
            const int c = c0 + row * rstep;
            // A = (AS_sub, AS_across-, AS_across+, -), W = (1/ALP, PT)
            R bx;
            Quad<R> A;
            Pair<R> W;
            if (ZL) {
                const int q = (p * d.nK + row) * d.nJ + line;
                A = b.zc[e][q];
                W = b.zp[e][q];
                bx = bxs[bx0 + row * bstep];
            } else {
                const int q = (p * d.nJ + row) * d.nK + line;
                A = b.yc[e][q];
                W = b.yp[e][q];
                if (FIRST) {
                    const Pair<R> X = b.yx[e][q];
                    const R* __restrict__ xp = b.xp[e];
                    const R xm = xp[xp_index(d, p - 1, row, line)];
                    const R xq = xp[xp_index(d, p + 1, row, line)];
                    bx = (A.w + X.y * xq) + X.x * xm;   // BS + AS12 XT(I+2) + AS11 XT(I-2)
                    bxs[bx0 + row * bstep] = bx;
                } else {
                    bx = bxs[bx0 + row * bstep];
                }
            }
            // y: + AS32 XT(K+2) + AS31 XT(K-2); z: + AS22 XT(J+2) + AS21 XT(J-2)
            const R v = W.x * ((bx + A.z * src[c + across]) + A.y * src[c - across]);
            const bool cp = rbp_copy(W.y);
            rr[i] = cp ? src[c] : v;
            al[i] = A.x * W.x;   // AS_sub/ALP; 0 on a copied row
            pv[i] = W.y;
        }
    }
    // forward elimination of the segment from a zero start: q = r + a q(prev)
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
    sA[threadIdx.x] = cnt > 0 ? Pc : R(1);
    sB[threadIdx.x] = cnt > 0 ? qc : R(0);
    __syncthreads();
    // carry into the segment: the maps of the segments before it, in order
    // (their loads taken four at a time ahead of the chain)
    R qin = xlo;
    for (int k0 = 0; k0 < seg; k0 += 4) {
        R a4[4], b4[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int k = k0 + u;
            if (k < seg) { a4[u] = sA[(k * G + grp) * 32 + lane]; b4[u] = sB[(k * G + grp) * 32 + lane]; }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (k0 + u < seg) qin = a4[u] * qin + b4[u];
    }
#pragma unroll
    for (int i = 0; i < M; ++i)
        if (i < cnt) q[i] = q[i] + P[i] * qin;
    __syncthreads();
    // back substitution of the segment from a zero end: x = q + PT x(next)
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
    sA[threadIdx.x] = cnt > 0 ? Rc : R(1);
    sB[threadIdx.x] = cnt > 0 ? xc : R(0);
    __syncthreads();
    R xin = xhi;
    for (int k0 = S - 1; k0 > seg; k0 -= 4) {
        R a4[4], b4[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int k = k0 - u;
            if (k > seg) { a4[u] = sA[(k * G + grp) * 32 + lane]; b4[u] = sB[(k * G + grp) * 32 + lane]; }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (k0 - u > seg) xin = a4[u] * xin + b4[u];
    }
#pragma unroll
    for (int i = 0; i < M; ++i) {
        if (i < cnt) {
            const int c = c0 + (e0 + i) * rstep;
            const R x = q[i] + P[i] * xin;
            dst[c] = ZL ? (dst[c] + x) / R(2) : x;   // (XT2 + XT3)/2
        }
    }
    __syncthreads();
}

template <typename R>
__host__ __device__ __forceinline__ int rbp_pitch(int nK) { return (nK + 2) | 1; }
template <typename R>
__host__ __device__ __forceinline__ size_t rbp_smem_bytes(const PlaneDims& d, int nt) {
    const int PS = rbp_pitch<R>(d.nK);
    return (size_t)(2 * (d.nJ + 2) * PS + d.nJ * PS + 2 * nt) * sizeof(R);
}

// Asynchronous prefetch of [ptr, ptr + bytes) into L2 (whole 16-byte units
// around the range; the arrays given here extend past every range asked for).
__device__ __forceinline__ void l2_prefetch(const void* ptr, size_t bytes) {
    unsigned long long a = (unsigned long long)ptr, end = a + bytes;
    a &= ~15ull;
    end = (end + 15) & ~15ull;
    while (a < end) {
        const unsigned n = (unsigned)((end - a) < (1ull << 20) ? (end - a) : (1ull << 20));
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"(n) : "memory");
        a += n;
    }
}

// One colour visit: every plane p = colour, colour + 2, .. of the call's
// planes (I = IB + 2p), one CTA each.
template <typename R, int NT, int M>
__global__ void __launch_bounds__(NT, 1) k_rbp_visit(RbpBatch<R> b, int colour, int sweep) {
    extern __shared__ __align__(16) unsigned char rbp_smem[];
    const int e = blockIdx.y;
    const Sys<R>& s = b.sys[e];
    if (sweep >= s.nim) return;
    const PlaneDims d = dims_of(s);
    const int npc = (d.npl - colour + 1) / 2;
    if ((int)blockIdx.x >= npc) return;
    const int p = colour + 2 * (int)blockIdx.x;
    const int XJ = d.nK + 2, np = (d.nJ + 2) * XJ;
    const int base = (p + 1) * np;
    R* __restrict__ xp = b.xp[e];
    if (threadIdx.x == 0) {
        // everything the visit reads from global memory, on its way to L2:
        // the records of the plane (fixed during the call, so this may run
        // while the kernel before is finishing) and, after the wait, the
        // plane and its two neighbours in XP
        const size_t pc = (size_t)d.nJ * d.nK;
        l2_prefetch(b.yc[e] + p * pc, pc * sizeof(Quad<R>));
        l2_prefetch(b.yp[e] + p * pc, pc * sizeof(Pair<R>));
        l2_prefetch(b.yx[e] + p * pc, pc * sizeof(Pair<R>));
        l2_prefetch(b.zc[e] + p * pc, pc * sizeof(Quad<R>));
        l2_prefetch(b.zp[e] + p * pc, pc * sizeof(Pair<R>));
    }
    pdl_wait();
    pdl_trigger();
    if (threadIdx.x == 0) {
        l2_prefetch(xp + base - np, (size_t)np * sizeof(R));
        l2_prefetch(xp + base + np, (size_t)np * sizeof(R));
    }
    const int PS = rbp_pitch<R>(d.nK);
    const int PB = (d.nJ + 2) * PS;
    R* xa = reinterpret_cast<R*>(rbp_smem);
    R* xb = xa + PB;
    R* bxs = xb + PB;
    R* sA = bxs + d.nJ * PS;
    R* sB = sA + NT;
    // the plane with its border, two J rows of 128 points a warp at a time
    // (their loads issued together); the border also into xb (the line ends)
    {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        constexpr int NW = NT / 32;
        for (int j0 = 2 * warp; j0 < d.nJ + 2; j0 += 2 * NW)
            for (int k0 = 0; k0 < XJ; k0 += 128) {
                R v[2][4];
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int jr = j0 + a, kr = k0 + lane + 32 * u;
                        if (jr < d.nJ + 2 && kr < XJ) v[a][u] = xp[base + jr * XJ + kr];
                    }
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int jr = j0 + a, kr = k0 + lane + 32 * u;
                        if (jr < d.nJ + 2 && kr < XJ) {
                            xa[jr * PS + kr] = v[a][u];
                            if (jr == 0 || jr == d.nJ + 1 || kr == 0 || kr == d.nK + 1) xb[jr * PS + kr] = v[a][u];
                        }
                    }
            }
    }
    __syncthreads();
    // pass L=1: y-lines into xb, then the z-lines averaged into it
    rbp_pass<R, M, false, true>(b, e, d, p, PS, xa, xb, bxs, sA, sB);
    // a plane with one z-row (KB >= KE) keeps the y-line pass alone (Adlbl3.f90:124-130)
    const bool one_row = s.kb >= s.ke;
    if (!one_row) {
        rbp_pass<R, M, true, false>(b, e, d, p, PS, xa, xb, bxs, sA, sB);
        // pass L=2 from the average: y-lines into xa, then the z-lines averaged into it
        rbp_pass<R, M, false, false>(b, e, d, p, PS, xb, xa, bxs, sA, sB);
        rbp_pass<R, M, true, false>(b, e, d, p, PS, xb, xa, bxs, sA, sB);
    }
    const R* out = one_row ? xb : xa;
    for (int jj = threadIdx.x >> 5; jj < d.nJ; jj += NT / 32)
        for (int kk = threadIdx.x & 31; kk < d.nK; kk += 32) xp[xp_index(d, p, jj, kk)] = out[(jj + 1) * PS + kk + 1];
}

constexpr int kRbpM = 8;            // rows of a segment held in registers
constexpr int kRbpThreads = 768;    // threads of a visit CTA (80 registers a thread, one CTA per SM)
constexpr int kRbpSmall = 256;      // threads of a visit CTA for planes whose passes fit 8 warps
constexpr size_t kRbpMaxSmem = 227 * 1024;

// segments a pass of n-row lines, nlines of them, gets from the CTA (the
// formula of rbp_pass); the pass fits when no segment exceeds M rows
inline bool rbp_pass_fits(int nlines, int n, int nt = kRbpThreads) {
    const int G = (nlines + 31) / 32;
    int S = (nt / 32) / G;
    S = S < 1 ? 1 : (S > n ? n : S);
    return (n + S - 1) / S <= kRbpM;
}

}  // namespace

template <typename R>
int launch_rbp(const GeoT<R>& g, const Sys<R>* sys, const AdiScratch<R>* scr, int nsys, cudaStream_t st, int rb_flags) {
    const bool pdl = (rb_flags & kRbPdl) != 0;
    RbpBatch<R> b;
    b.nsys = nsys;
    size_t smem = 0;
    int max_np = 0, max_nj = 0, max_nk = 0, nim = 0;
    // planes small enough for 8 warps run on CTAs of that size: a few
    // hundred points a plane leave most of a larger CTA idle at its barriers
    bool small = true;
    for (int e = 0; e < nsys; ++e) {
        const PlaneDims d = dims_of(sys[e]);
        if (!rbp_pass_fits(d.nK, d.nJ) || !rbp_pass_fits(d.nJ, d.nK)) return 0;
        small = small && rbp_pass_fits(d.nK, d.nJ, kRbpSmall) && rbp_pass_fits(d.nJ, d.nK, kRbpSmall);
        smem = std::max(smem, rbp_smem_bytes<R>(d, kRbpThreads));
        b.sys[e] = sys[e];
        // the records in the scratch of the segmented form (2*CBH elements each)
        const long long NH = 2LL * g.CBH;
        b.xp[e] = scr[e].xs;
        b.yc[e] = scr[e].ya;
        b.yx[e] = reinterpret_cast<Pair<R>*>(scr[e].yb);
        b.yp[e] = reinterpret_cast<Pair<R>*>(scr[e].yb) + NH;
        b.zc[e] = scr[e].za;
        b.zp[e] = reinterpret_cast<Pair<R>*>(scr[e].zb);
        max_np = std::max(max_np, d.npl);
        max_nj = std::max(max_nj, d.nJ);
        max_nk = std::max(max_nk, d.nK);
        nim = std::max(nim, sys[e].nim);
    }
    if (smem > kRbpMaxSmem) return 0;
    // in FP64 the small planes go to the segmented colour passes, which keep
    // more lines in flight per SM for the FP64 pipe (TC21: 2.6 against 3.5 ms
    // an iteration)
    if (rb_flags & kRbNoSmall) small = false;
    if (small && sizeof(R) == 8 && !(rb_flags & kRbSmallF64)) return 0;
    const unsigned tiles_in = (unsigned)(((max_np + 2 + 31) / 32) * ((max_nk + 2 + 31) / 32));
    const unsigned tiles_out = (unsigned)(((max_np + 31) / 32) * ((max_nk + 31) / 32));
    const unsigned ptiles = (unsigned)((max_np + 31) / 32);
    launch_k(pdl, k_rbp_copy<R, true>, dim3(tiles_in, max_nj + 2, nsys), dim3(32, 8), 0, st, g, b);
    const int fy = (int)(ptiles * ((max_nk + 15) / 16)), fz = (int)(ptiles * ((max_nj + 15) / 16));
    launch_k(pdl, k_rbp_fill<R>, dim3((unsigned)(fy + fz), std::max(max_nj, max_nk), nsys), dim3(32, 8), 0, st, g, b, fy);
    const int py = (int)(ptiles * ((max_nk + 7) / 8)), pz = (int)(ptiles * ((max_nj + 7) / 8));
    launch_k(pdl, k_rbp_pivots<R>, dim3((unsigned)(py + pz), nsys), dim3(32, 8), 0, st, g, b, py);
    const dim3 gv((unsigned)((max_np + 1) / 2), nsys);
    for (int ns = 0; ns < nim; ++ns)
        for (int half = 0; half < 2; ++half)
            for (int colour = 0; colour < 2; ++colour)
                if (small)
                    launch_k(pdl, k_rbp_visit<R, kRbpSmall, kRbpM>, gv, dim3(kRbpSmall), smem, st, b, colour, ns);
                else
                    launch_k(pdl, k_rbp_visit<R, kRbpThreads, kRbpM>, gv, dim3(kRbpThreads), smem, st, b, colour, ns);
    launch_k(pdl, k_rbp_copy<R, false>, dim3(tiles_out, max_nj, nsys), dim3(32, 8), 0, st, g, b);
    return 4 + 4 * nim;
}

int prepare_rbp() {
    const bool ok = cudaFuncSetAttribute(k_rbp_visit<float, kRbpThreads, kRbpM>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRbpMaxSmem) == cudaSuccess &&
                    cudaFuncSetAttribute(k_rbp_visit<double, kRbpThreads, kRbpM>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRbpMaxSmem) == cudaSuccess &&
                    cudaFuncSetAttribute(k_rbp_visit<float, kRbpSmall, kRbpM>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRbpMaxSmem) == cudaSuccess &&
                    cudaFuncSetAttribute(k_rbp_visit<double, kRbpSmall, kRbpM>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRbpMaxSmem) == cudaSuccess;
    return ok ? GFM_OK : GFM_E_CUDA;
}

template int launch_rbp<float>(const GeoT<float>&, const Sys<float>*, const AdiScratch<float>*, int, cudaStream_t, int);
template int launch_rbp<double>(const GeoT<double>&, const Sys<double>*, const AdiScratch<double>*, int, cudaStream_t,
                                int);

}  // namespace gfm
