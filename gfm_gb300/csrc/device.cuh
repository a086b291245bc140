// device.cuh -- device-side layout, context and helpers of the GB300 solver.
//
// Layout.  The reference stores every field on its doubled staggered grid
// A(MP,NP,LP): cell centres at (even,even,even), x-faces at (odd,even,even),
// edges and corners at the other parity classes (Grid3.f90:8-300).  A kernel
// working on one class would touch every other element of a Fortran row.  On
// the device each field is split by parity class: class c = (I&1)|(J&1)<<1|
// (K&1)<<2 is a dense (PX,HY,HZ) block, element (I,J,K) at
//     c*CB + ((K>>1)*HY + (J>>1))*PX + (I>>1).
// The map is a bijection with the doubled grid, so every reference loop over
// one class becomes a unit-stride, coalesced sweep, and neighbour (I+-1) is the
// same (J,K) row of the neighbouring class.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gfm_gb300.h"
#include "physics.h"

namespace gfm {

// Grid geometry on the device (coordinate arrays 1-based: index 0 unused),
// coordinates stored in the arithmetic type R of the kernels using them.
template <typename R>
struct GeoT {
    int MP, NP, LP;
    int HX, HY, HZ, PX;        // half extents (MP/2+1 ...) and padded row pitch
    long long CB;              // elements per parity class
    int PXH, CBH;              // colour-split copy of one class: row pitch, elements per half
    int MPM1, MPM2, NPM1, NPM2, LPM1, LPM2;
    int NJY1, NJY2, LKZ1, LKZ2;
    int NJY1V[4], NJY2V[4], LKZ1V[4], LKZ2V[4];
    int NCELLS;
    const R *X, *DX, *Rr, *DR, *RS, *Z, *DZ;
    const int8_t* ib;          // IBCELL, parity split
    // half-blocked cells (IBCELL -1, -2): BV_F(IBC), BA_F(IX,IBC) at
    // BAF[3*(IBC-1) + IX-1]; HALF is 0 when the grid has none
    R BVF[2], BAF[6];
    int HALF;
};
using Geo = GeoT<double>;

// Offsets are formed in 32-bit arithmetic: a field holds fewer than 2^31
// elements (checked when a handle is created).
template <typename R>
__host__ __device__ __forceinline__ long long pidx(const GeoT<R>& g, int I, int J, int K) {
    int c = (I & 1) | ((J & 1) << 1) | ((K & 1) << 2);
    return (long long)(c * (int)g.CB + ((K >> 1) * g.HY + (J >> 1)) * g.PX + (I >> 1));
}

// grid-stride loop over [0, n) in 32-bit arithmetic (n < 2^31)
#define GFM_FOR(t, n) \
    for (int t = blockIdx.x * blockDim.x + threadIdx.x, t##_end = (int)(n); t < t##_end; t += gridDim.x * blockDim.x)
template <typename R>
__device__ __forceinline__ int IBC(const GeoT<R>& g, int I, int J, int K) { return g.ib[pidx(g, I, J, K)]; }

// VOL_C0 (Grid3.f90:395-405): the cell's volume, times BV_F on a
// half-blocked cell
template <typename R>
__device__ __forceinline__ R vol_c0(const GeoT<R>& g, int I, int J, int K) {
    const R v = g.DX[I] * g.DR[J] * g.RS[J] * g.DZ[K];
    if (g.HALF) {
        const int ib = IBC(g, I, J, K);
        if (ib <= -1) return v * g.BVF[-ib - 1];
    }
    return v;
}
// AREA_C (Grid3.f90:411-471): the face area normal to direction ix of the
// cell; 0 on a wall, times BA_F on a half-blocked cell, and on a cell with
// IBCELL >= 2 times BA_F of a half-blocked neighbour two positions away
// along ix (the + side first)
template <typename R>
__device__ __forceinline__ R area_c(const GeoT<R>& g, int I, int J, int K, int ix) {
    const int ib = IBC(g, I, J, K);
    if (ib == 1) return R(0);
    const R a = ix == 1 ? g.DR[J] * g.RS[J] * g.DZ[K] : ix == 2 ? g.DX[I] * g.DZ[K] : g.DX[I] * g.DR[J] * g.RS[J];
    if (!g.HALF || ib == 0) return a;
    if (ib <= -1) return a * g.BAF[3 * (-ib - 1) + ix - 1];
    int nb = 0;
    if (ix == 1) {
        if (I <= g.MPM2 && IBC(g, I + 2, J, K) <= -1) nb = IBC(g, I + 2, J, K);
        else if (I >= 4 && IBC(g, I - 2, J, K) <= -1) nb = IBC(g, I - 2, J, K);
    } else if (ix == 2) {
        if (J <= g.NPM2 && IBC(g, I, J + 2, K) <= -1) nb = IBC(g, I, J + 2, K);
        else if (J >= 4 && IBC(g, I, J - 2, K) <= -1) nb = IBC(g, I, J - 2, K);
    } else {
        if (K <= g.LPM2 && IBC(g, I, J, K + 2) <= -1) nb = IBC(g, I, J, K + 2);
        else if (K >= 4 && IBC(g, I, J, K - 2) <= -1) nb = IBC(g, I, J, K - 2);
    }
    return nb <= -1 ? a * g.BAF[3 * (-nb - 1) + ix - 1] : a;
}

// Programmatic dependent launch.  A kernel launched by launch_k with pdl set
// may begin (block scheduling, prologue) while the kernel before it in the
// stream is still finishing.  pdl_wait() returns once that kernel has
// completed and its writes are visible, so every kernel launched this way
// calls it before it touches global memory; completion is then transitive
// along the chain.  pdl_trigger() lets the next kernel begin launching.  Both
// are no-ops in a kernel launched without the attribute.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
template <typename... KArgs, typename... Args>
inline void launch_k(bool pdl, void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args) {
    if (!pdl) {
        k<<<grid, block, smem, st>>>(args...);
        return;
    }
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, args...);
}

// Scalar constants of the run (gfm_params plus derived complements).
struct Prm {
    double t0, h_0, dnst0, ug0, gmfr, pg0, r0;
    double reyg, reyg2, epsr, taur, eun, qr0, q0, tk0;
    double gra[3];
    double amu, trdg, wt0, stoich;
    double cmu, ct1, ct2;
    double p_mx, p_mn, t_mx, t_mn, u_mx, u_mn, f_mx, f_mn;
    double rf[21], rfc[21], rfl[21], rflc[21];
    double sigma[12];
    double rf_hsource, h_g;
    double sig, ri, hck;
    int react, wall_sink;
    // constants of the run that the reference recomputes in its cell loops,
    // evaluated once on the host:
    double rt20;   // REYG2*SQRT(EPSR)*CMU**0.25 (Gflow.f90:74, wall functions)
    double cbl0;   // 2.5*SQRT(EPSR)/TAUR*CMU**0.75 (Source.f90:579, epsilon wall penalty)
};

// Deterministic FP64 reductions: every block writes one partial per slot into
// `partials`, a single-block kernel sums them in a fixed order.
constexpr int kRedSlots = 64;      // independent sums per iteration
constexpr int kRedBlocks = 1024;   // max blocks contributing per pass

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        double w = __shfl_down_sync(0xffffffffu, v, o);
        v = (w > v) ? w : v;
    }
    return v;
}
// Block-wide sum of v; result valid in thread 0.  Requires blockDim.x % 32 == 0.
__device__ __forceinline__ double block_sum(double v, double* sh) {
    v = warp_sum(v);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    int nw = blockDim.x >> 5;
    v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (w == 0) v = warp_sum(v);
    __syncthreads();
    return v;
}
__device__ __forceinline__ double block_max(double v, double* sh) {
    v = warp_max(v);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    int nw = blockDim.x >> 5;
    v = (threadIdx.x < nw) ? sh[threadIdx.x] : -1.0e308;
    if (w == 0) v = warp_max(v);
    __syncthreads();
    return v;
}

}  // namespace gfm
