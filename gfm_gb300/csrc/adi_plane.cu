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
//   YA, YB  the rows of the y-lines (I, *, K), K fastest within the plane
//       ((p nJ + jj) nK + kk): YA = (AS21, AS31, AS32, 1/ALP), YB = (BS, AS11,
//       AS12, PT) with the Thomas pivots of the line, ALP = AP - PT(prev) AS21,
//       PT = AS22/ALP (ADLZY, Adlbl3.f90:147-181);
//   ZA, ZP  the rows of the z-lines (I, J, *), J fastest ((p nK + kk) nJ + jj):
//       ZA = (AS31, AS21, AS22, 1/ALP), ZP = PT with ALP = AP - PT(prev) AS31,
//       PT = AS32/ALP (ADLYZ, Adlbl3.f90:187-221).
//
// The matrices do not change during the call, so the pivots are the values
// every visit of the reference would form.  A row the reference copies
// unchanged (|ALP| <= 1e-20 or a blocked cell) stores 1/ALP = 0 and PT = -0.0,
// a value no other row stores.
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
struct RbpBatch {
    Sys<R> sys[8];
    R* xp[8];
    Quad<R>* ya[8];
    Quad<R>* yb[8];
    Quad<R>* za[8];
    R* zp[8];
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
// Records and pivots of every line, once per call.  A thread walks one line
// (plane p, fixed cross index) row by row, the pivot chain of ADLZY/ADLYZ;
// lanes take 32 neighbouring planes, so the loads of the class arrays are
// contiguous.  The records of one row go through a shared-memory tile and
// leave with the cross index fastest, contiguous in the record layout.
// Block 32 x 8: 32 planes x 8 lines; grid x over (plane tiles) x (line
// tiles), y = system.  ZL: z-lines (rows along K, lines indexed by J), else
// y-lines (rows along J, lines indexed by K).
// ---------------------------------------------------------------------------
template <typename R, bool ZL>
__global__ void __launch_bounds__(256) k_rbp_factor(GeoT<R> g, RbpBatch<R> b) {
    __shared__ Quad<R> ta[2][32][9];
    __shared__ Quad<R> tb[2][32][9];
    pdl_wait();
    pdl_trigger();
    const int e = blockIdx.y;
    const Sys<R>& s = b.sys[e];
    const PlaneDims d = dims_of(s);
    const int nlines = ZL ? d.nJ : d.nK, nrows = ZL ? d.nK : d.nJ;
    const int ntp = (d.npl + 31) / 32;
    const int p0 = (blockIdx.x % ntp) * 32, l0 = (blockIdx.x / ntp) * 8;
    if (l0 >= nlines) return;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int p = p0 + tx, l = l0 + ty;
    const bool act = p < d.npl && l < nlines;
    // y-line (I,*,K): sub AS21 = as[2], next AS22 = as[3], across AS31/AS32 = as[4]/as[5]
    // z-line (I,J,*): sub AS31 = as[4], next AS32 = as[5], across AS21/AS22 = as[2]/as[3]
    const R* __restrict__ a_sub = s.as[ZL ? 4 : 2];
    const R* __restrict__ a_next = s.as[ZL ? 5 : 3];
    const R* __restrict__ a_c0 = s.as[ZL ? 2 : 4];
    const R* __restrict__ a_c1 = s.as[ZL ? 3 : 5];
    const int I = s.ib + 2 * p;
    const int ostep = ZL ? (int)(pidx(g, 0, 0, 2) - pidx(g, 0, 0, 0)) : (int)(pidx(g, 0, 2, 0) - pidx(g, 0, 0, 0));
    const int o0 = act ? (int)(ZL ? pidx(g, I, s.jb + 2 * l, s.kb) : pidx(g, I, s.jb, s.kb + 2 * l)) : 0;
    // writer side: thread (tx, ty) -> plane p0 + (tid / 8), line l0 + (tid % 8)
    const int tid = ty * 32 + tx;
    const int wp = p0 + (tid >> 3), wl = l0 + (tid & 7);
    const bool wact = wp < d.npl && wl < nlines;
    R pt_prev = R(0);
    for (int r = 0; r < nrows; ++r) {
        const int buf = r & 1;
        if (act) {
            const int o = o0 + r * ostep;
            const R ap = s.ap[o], sub = a_sub[o], nxt = a_next[o];
            const R c0 = a_c0[o], c1 = a_c1[o];
            const bool blk = g.ib[o] >= 1;
            const R alp = ap - pt_prev * sub;
            Quad<R> A, B;
            R ia, pt;
            if (fabs(alp) <= R(1.0e-20) || blk) {
                ia = R(0);
                pt = -R(0);
                pt_prev = R(0);
            } else {
                ia = R(1) / alp;
                pt = nxt / alp + R(0);   // +0.0: no -0.0 here
                pt_prev = pt;
            }
            if (ZL) {
                A = Quad<R>{sub, c0, c1, ia};                      // (AS31, AS21, AS22, 1/ALP)
                B = Quad<R>{pt, R(0), R(0), R(0)};
            } else {
                A = Quad<R>{sub, c0, c1, ia};                      // (AS21, AS31, AS32, 1/ALP)
                B = Quad<R>{s.bs[o], s.as[0][o], s.as[1][o], pt};  // (BS, AS11, AS12, PT)
            }
            ta[buf][tx][ty] = A;
            tb[buf][tx][ty] = B;
        }
        __syncthreads();
        if (wact) {
            const Quad<R> A = ta[buf][tid >> 3][tid & 7];
            const Quad<R> B = tb[buf][tid >> 3][tid & 7];
            if (ZL) {
                const int q = (wp * d.nK + r) * d.nJ + wl;
                b.za[e][q] = A;
                b.zp[e][q] = B.x;
            } else {
                const int q = (wp * d.nJ + r) * d.nK + wl;
                b.ya[e][q] = A;
                b.yb[e][q] = B;
            }
        }
        // the next row writes the other buffer; the barrier of that row
        // orders this row's reads before the buffer is written again
    }
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
            R bx, pt;
            Quad<R> A;
            if (ZL) {
                const int q = (p * d.nK + row) * d.nJ + line;
                A = b.za[e][q];
                pt = b.zp[e][q];
                bx = bxs[bx0 + row * bstep];
            } else {
                const int q = (p * d.nJ + row) * d.nK + line;
                A = b.ya[e][q];
                const Quad<R> B = b.yb[e][q];
                pt = B.w;
                if (FIRST) {
                    const R* __restrict__ xp = b.xp[e];
                    const R xm = xp[xp_index(d, p - 1, row, line)];
                    const R xq = xp[xp_index(d, p + 1, row, line)];
                    bx = (B.x + B.z * xq) + B.y * xm;   // BS + AS12 XT(I+2) + AS11 XT(I-2)
                    bxs[bx0 + row * bstep] = bx;
                } else {
                    bx = bxs[bx0 + row * bstep];
                }
            }
            // y: + AS32 XT(K+2) + AS31 XT(K-2); z: + AS22 XT(J+2) + AS21 XT(J-2)
            const R v = A.w * ((bx + A.z * src[c + across]) + A.y * src[c - across]);
            const bool cp = rbp_copy(pt);
            rr[i] = cp ? src[c] : v;
            al[i] = A.x * A.w;   // AS_sub/ALP; 0 on a copied row
            pv[i] = pt;
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
    R qin = xlo;
    for (int k = 0; k < seg && k < S; ++k) qin = sA[(k * G + grp) * 32 + lane] * qin + sB[(k * G + grp) * 32 + lane];
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
    for (int k = S - 1; k > seg; --k) xin = sA[(k * G + grp) * 32 + lane] * xin + sB[(k * G + grp) * 32 + lane];
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

// One colour visit: every plane p = colour, colour + 2, .. of the call's
// planes (I = IB + 2p), one CTA each.
template <typename R, int NT, int M>
__global__ void __launch_bounds__(NT, 1) k_rbp_visit(RbpBatch<R> b, int colour, int sweep) {
    extern __shared__ __align__(16) unsigned char rbp_smem[];
    pdl_wait();
    pdl_trigger();
    const int e = blockIdx.y;
    const Sys<R>& s = b.sys[e];
    if (sweep >= s.nim) return;
    const PlaneDims d = dims_of(s);
    const int npc = (d.npl - colour + 1) / 2;
    if ((int)blockIdx.x >= npc) return;
    const int p = colour + 2 * (int)blockIdx.x;
    const int PS = rbp_pitch<R>(d.nK);
    const int PB = (d.nJ + 2) * PS;
    R* xa = reinterpret_cast<R*>(rbp_smem);
    R* xb = xa + PB;
    R* bxs = xb + PB;
    R* sA = bxs + d.nJ * PS;
    R* sB = sA + NT;
    R* __restrict__ xp = b.xp[e];
    // the plane with its border; the border also into xb (the line ends)
    const int XJ = d.nK + 2, np = (d.nJ + 2) * XJ;
    const int base = (p + 1) * np;
    for (int t = threadIdx.x; t < np; t += NT) {
        const int jr = t / XJ, kr = t - jr * XJ;
        const R v = xp[base + t];
        xa[jr * PS + kr] = v;
        if (jr == 0 || jr == d.nJ + 1 || kr == 0 || kr == d.nK + 1) xb[jr * PS + kr] = v;
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
    for (int t = threadIdx.x; t < d.nJ * d.nK; t += NT) {
        const int jj = t / d.nK, kk = t - jj * d.nK;
        xp[xp_index(d, p, jj, kk)] = out[(jj + 1) * PS + kk + 1];
    }
}

constexpr int kRbpM = 8;            // rows of a segment held in registers
constexpr int kRbpThreads = 768;    // threads of a visit CTA (80 registers a thread, one CTA per SM)
constexpr size_t kRbpMaxSmem = 227 * 1024;

// segments a pass of n-row lines, nlines of them, gets from the CTA (the
// formula of rbp_pass); the pass fits when no segment exceeds M rows
inline bool rbp_pass_fits(int nlines, int n) {
    const int G = (nlines + 31) / 32;
    int S = (kRbpThreads / 32) / G;
    S = S < 1 ? 1 : (S > n ? n : S);
    return (n + S - 1) / S <= kRbpM;
}

}  // namespace

template <typename R>
int launch_rbp(const GeoT<R>& g, const Sys<R>* sys, const AdiScratch<R>* scr, int nsys, cudaStream_t st, bool pdl) {
    RbpBatch<R> b;
    b.nsys = nsys;
    size_t smem = 0;
    int max_np = 0, max_nj = 0, max_nk = 0, nim = 0;
    int ft_y = 0, ft_z = 0;
    for (int e = 0; e < nsys; ++e) {
        const PlaneDims d = dims_of(sys[e]);
        if (!rbp_pass_fits(d.nK, d.nJ) || !rbp_pass_fits(d.nJ, d.nK)) return 0;
        smem = std::max(smem, rbp_smem_bytes<R>(d, kRbpThreads));
        b.sys[e] = sys[e];
        b.xp[e] = scr[e].xs;
        b.ya[e] = scr[e].ya;
        b.yb[e] = scr[e].yb;
        b.za[e] = scr[e].za;
        b.zp[e] = scr[e].x2;
        max_np = std::max(max_np, d.npl);
        max_nj = std::max(max_nj, d.nJ);
        max_nk = std::max(max_nk, d.nK);
        nim = std::max(nim, sys[e].nim);
        ft_y = std::max(ft_y, ((d.npl + 31) / 32) * ((d.nK + 7) / 8));
        ft_z = std::max(ft_z, ((d.npl + 31) / 32) * ((d.nJ + 7) / 8));
    }
    if (smem > kRbpMaxSmem) return 0;
    const unsigned tiles_in = (unsigned)(((max_np + 2 + 31) / 32) * ((max_nk + 2 + 31) / 32));
    const unsigned tiles_out = (unsigned)(((max_np + 31) / 32) * ((max_nk + 31) / 32));
    launch_k(pdl, k_rbp_copy<R, true>, dim3(tiles_in, max_nj + 2, nsys), dim3(32, 8), 0, st, g, b);
    launch_k(pdl, k_rbp_factor<R, false>, dim3((unsigned)ft_y, nsys), dim3(32, 8), 0, st, g, b);
    launch_k(pdl, k_rbp_factor<R, true>, dim3((unsigned)ft_z, nsys), dim3(32, 8), 0, st, g, b);
    const dim3 gv((unsigned)((max_np + 1) / 2), nsys);
    for (int ns = 0; ns < nim; ++ns)
        for (int half = 0; half < 2; ++half)
            for (int colour = 0; colour < 2; ++colour)
                launch_k(pdl, k_rbp_visit<R, kRbpThreads, kRbpM>, gv, dim3(kRbpThreads), smem, st, b, colour, ns);
    launch_k(pdl, k_rbp_copy<R, false>, dim3(tiles_out, max_nj, nsys), dim3(32, 8), 0, st, g, b);
    return 4 + 4 * nim;
}

int prepare_rbp() {
    const bool ok = cudaFuncSetAttribute(k_rbp_visit<float, kRbpThreads, kRbpM>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRbpMaxSmem) == cudaSuccess &&
                    cudaFuncSetAttribute(k_rbp_visit<double, kRbpThreads, kRbpM>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRbpMaxSmem) == cudaSuccess;
    return ok ? GFM_OK : GFM_E_CUDA;
}

template int launch_rbp<float>(const GeoT<float>&, const Sys<float>*, const AdiScratch<float>*, int, cudaStream_t, bool);
template int launch_rbp<double>(const GeoT<double>&, const Sys<double>*, const AdiScratch<double>*, int, cudaStream_t,
                                bool);

}  // namespace gfm
