// lpsolve.cu -- solver side of the learned p' initial guess: network inputs
// from the p' system, the guess written into p' before the line solve with a
// fallback to the zero start, and training targets from a converged solve.
//
// The voxel grid is the solve range of the p' equation on the cell centres,
// I = 4..MP-2, J = 4..NP-2, K = 4..LP-2 (step 2): nx = MP/2-2 and so on, voxel
// v = (k*ny + j)*nx + i for I = 4+2i, J = 4+2j, K = 4+2k.  Input channels:
//   0: (BS/AP)/s on open cells, s = RMS of BS/AP over the open cells;
//   1: 1 on open cells, 0 on blocked ones;  2..15: 0.
// The network predicts the shape of p' (training targets are scaled to unit
// RMS); its magnitude comes from the system: the guess is alpha*g with alpha
// minimising |b - alpha*M g| (FP64), M g = AP g - sum AS g_nb, so its residual
// never exceeds that of the zero start.
#include <cuda_bf16.h>

#include "state.cuh"

namespace gfm {

constexpr int kSlotLpQ = 40, kSlotLpN = 41, kSlotLpGB = 42, kSlotLpGG = 43, kSlotLpBB = 44;

template <typename R>
__device__ __forceinline__ int lp_voxel(const GeoT<R>& g, int v, int nx, int ny) {
    const int i = v % nx, j = (v / nx) % ny, k = v / (nx * ny);
    return (int)pidx(g, 4 + 2 * i, 4 + 2 * j, 4 + 2 * k);
}

// partial sums of (BS/AP)^2 and of the open count
template <typename R>
__global__ void k_lp_scale_part(Ctx<R> c, int nx, int ny, int nz) {
    __shared__ double sh[32];
    const int n = nx * ny * nz;
    double a = 0.0, b = 0.0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int o = lp_voxel(c.g, v, nx, ny);
        const double ap = (double)c.APc[o];
        if (c.g.ib[o] < 1 && ap != 0.0) {
            const double q = (double)c.BSq[o] / ap;
            a += q * q;
            b += 1.0;
        }
    }
    const double sa = block_sum(a, sh), sb = block_sum(b, sh);
    if (threadIdx.x == 0) {
        c.partials[kSlotLpQ * kRedBlocks + blockIdx.x] = sa;
        c.partials[kSlotLpN * kRedBlocks + blockIdx.x] = sb;
    }
}
// sum of the first nb partials of a slot by one block, in a fixed order; valid in thread 0
__device__ double fixed_sum(const double* partials, int slot, int nb, double* sh) {
    double v = 0.0;
    for (int q = threadIdx.x; q < nb; q += blockDim.x) v += partials[slot * kRedBlocks + q];
    return block_sum(v, sh);
}
// s = sqrt(mean (BS/AP)^2)
__global__ void k_lp_scale_fin(const double* partials, double* scal, int nb) {
    __shared__ double sh[32];
    const double a = fixed_sum(partials, kSlotLpQ, nb, sh), b = fixed_sum(partials, kSlotLpN, nb, sh);
    if (threadIdx.x != 0) return;
    const double s = b > 0.0 ? sqrt(a / b) : 0.0;
    scal[S_LP_SCALE] = (s > 1.0e-30 && isfinite(s)) ? s : 1.0;
}
template <typename R>
__global__ void k_lp_feat(Ctx<R> c, __nv_bfloat16* __restrict__ feats, int nx, int ny, int nz) {
    const int n = nx * ny * nz;
    const double inv = 1.0 / c.scal[S_LP_SCALE];
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int o = lp_voxel(c.g, v, nx, ny);
        const double ap = (double)c.APc[o];
        const bool open = c.g.ib[o] < 1 && ap != 0.0;
        const float q = open ? (float)((double)c.BSq[o] / ap * inv) : 0.f;
        const uint32_t w0 = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(q)) |
                            ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(open ? 1.f : 0.f)) << 16);
        uint4* f = reinterpret_cast<uint4*>(feats + (size_t)v * 16);
        f[0] = make_uint4(w0, 0u, 0u, 0u);
        f[1] = make_uint4(0u, 0u, 0u, 0u);
    }
}
// x = g (network output, channel 0) on open voxels of the solve range
template <typename R>
__global__ void k_lp_guess(Ctx<R> c, const float* __restrict__ out16, R* x, int nx, int ny, int nz) {
    const int n = nx * ny * nz;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int o = lp_voxel(c.g, v, nx, ny);
        if (c.g.ib[o] < 1 && c.APc[o] != R(0)) x[o] = R(out16[(size_t)v * 16]);
    }
}
// FP64 sums of (M g).b, (M g).(M g) and b.b over the open voxels
template <typename R>
__global__ void k_lp_check_part(Ctx<R> c, const R* x, int nx, int ny, int nz) {
    __shared__ double sh[32];
    const int n = nx * ny * nz;
    const int sy = c.g.PX, sz = c.g.PX * c.g.HY;
    double gb = 0.0, gg = 0.0, bb = 0.0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int o = lp_voxel(c.g, v, nx, ny);
        if (c.g.ib[o] >= 1) continue;
        const double b = (double)c.BSq[o];
        const double mg = (double)c.APc[o] * (double)x[o] -
                          ((double)c.ASc[0][o] * (double)x[o - 1] + (double)c.ASc[1][o] * (double)x[o + 1] +
                           (double)c.ASc[2][o] * (double)x[o - sy] + (double)c.ASc[3][o] * (double)x[o + sy] +
                           (double)c.ASc[4][o] * (double)x[o - sz] + (double)c.ASc[5][o] * (double)x[o + sz]);
        gb += mg * b;
        gg += mg * mg;
        bb += b * b;
    }
    const double a = block_sum(gb, sh), b2 = block_sum(gg, sh), c2 = block_sum(bb, sh);
    if (threadIdx.x == 0) {
        c.partials[kSlotLpGB * kRedBlocks + blockIdx.x] = a;
        c.partials[kSlotLpGG * kRedBlocks + blockIdx.x] = b2;
        c.partials[kSlotLpBB * kRedBlocks + blockIdx.x] = c2;
    }
}
// alpha = (Mg.b)/(Mg.Mg); residual ratio |b - alpha Mg|/|b| = sqrt(1 - (Mg.b)^2/(|Mg|^2 |b|^2));
// the guess is kept when that ratio is below 1
__global__ void k_lp_decide(const double* partials, double* scal, int nb) {
    __shared__ double sh[32];
    const double gb = fixed_sum(partials, kSlotLpGB, nb, sh), gg = fixed_sum(partials, kSlotLpGG, nb, sh),
                 bb = fixed_sum(partials, kSlotLpBB, nb, sh);
    if (threadIdx.x != 0) return;
    const double alpha = gg > 0.0 ? gb / gg : 0.0;
    const double r2 = (gg > 0.0 && bb > 0.0) ? 1.0 - gb * gb / (gg * bb) : 1.0;
    const double ratio = sqrt(r2 > 0.0 ? r2 : 0.0);
    const bool use = isfinite(alpha) && isfinite(ratio) && ratio < 1.0;
    scal[S_LP_RATIO] = isfinite(ratio) ? ratio : 1.0;
    scal[S_LP_USED] = use ? 1.0 : 0.0;
    scal[S_LP_ALPHA] = use ? alpha : 0.0;
}
// x = alpha * g (alpha = 0 when the guess is not kept)
template <typename R>
__global__ void k_lp_apply(Ctx<R> c, R* x, int nx, int ny, int nz) {
    const int n = nx * ny * nz;
    const double alpha = c.scal[S_LP_ALPHA];
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int o = lp_voxel(c.g, v, nx, ny);
        if (c.g.ib[o] < 1) x[o] = R(alpha * (double)x[o]);
    }
}
// training target: x scaled to unit RMS over the open voxels
template <typename R>
__global__ void k_lp_tnorm_part(Ctx<R> c, const R* x, int nx, int ny, int nz) {
    __shared__ double sh[32];
    const int n = nx * ny * nz;
    double a = 0.0, b = 0.0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int o = lp_voxel(c.g, v, nx, ny);
        if (c.g.ib[o] < 1 && c.APc[o] != R(0)) {
            const double q = (double)x[o];
            a += q * q;
            b += 1.0;
        }
    }
    const double sa = block_sum(a, sh), sb = block_sum(b, sh);
    if (threadIdx.x == 0) {
        c.partials[kSlotLpQ * kRedBlocks + blockIdx.x] = sa;
        c.partials[kSlotLpN * kRedBlocks + blockIdx.x] = sb;
    }
}
__global__ void k_lp_tnorm_fin(const double* partials, double* scal, int nb) {
    __shared__ double sh[32];
    const double a = fixed_sum(partials, kSlotLpQ, nb, sh), b = fixed_sum(partials, kSlotLpN, nb, sh);
    if (threadIdx.x != 0) return;
    const double s = b > 0.0 ? sqrt(a / b) : 0.0;
    scal[S_LP_TSCALE] = (s > 1.0e-300 && isfinite(s)) ? s : 1.0;
}
template <typename R>
__global__ void k_lp_target(Ctx<R> c, const R* __restrict__ x, float* __restrict__ tgt, int nx, int ny, int nz) {
    const int n = nx * ny * nz;
    const double inv = 1.0 / c.scal[S_LP_TSCALE];
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int o = lp_voxel(c.g, v, nx, ny);
        tgt[v] = (c.g.ib[o] < 1 && c.APc[o] != R(0)) ? (float)((double)x[o] * inv) : 0.f;
    }
}

inline int lp_blocks(long long n) {
    long long b = (n + 255) / 256;
    return (int)(b < 1 ? 1 : (b > kRedBlocks ? kRedBlocks : b));
}

template <typename R>
void launch_lp_features(const Ctx<R>& c, void* feats, int nx, int ny, int nz, cudaStream_t s) {
    const long long n = (long long)nx * ny * nz;
    const int nb = lp_blocks(n);
    k_lp_scale_part<R><<<nb, 256, 0, s>>>(c, nx, ny, nz);
    k_lp_scale_fin<<<1, 256, 0, s>>>(c.partials, c.scal, nb);
    k_lp_feat<R><<<lp_blocks(n), 256, 0, s>>>(c, static_cast<__nv_bfloat16*>(feats), nx, ny, nz);
}
template <typename R>
void launch_lp_guess(const Ctx<R>& c, const float* out16, R* x, int nx, int ny, int nz, cudaStream_t s) {
    const long long n = (long long)nx * ny * nz;
    const int nb = lp_blocks(n);
    k_lp_guess<R><<<nb, 256, 0, s>>>(c, out16, x, nx, ny, nz);
    k_lp_check_part<R><<<nb, 256, 0, s>>>(c, x, nx, ny, nz);
    k_lp_decide<<<1, 256, 0, s>>>(c.partials, c.scal, nb);
    k_lp_apply<R><<<nb, 256, 0, s>>>(c, x, nx, ny, nz);
}
template <typename R>
void launch_lp_target(const Ctx<R>& c, const R* x, float* tgt, int nx, int ny, int nz, cudaStream_t s) {
    const long long n = (long long)nx * ny * nz;
    const int nb = lp_blocks(n);
    k_lp_tnorm_part<R><<<nb, 256, 0, s>>>(c, x, nx, ny, nz);
    k_lp_tnorm_fin<<<1, 256, 0, s>>>(c.partials, c.scal, nb);
    k_lp_target<R><<<nb, 256, 0, s>>>(c, x, tgt, nx, ny, nz);
}

#define INST(R)                                                                                       \
    template void launch_lp_features<R>(const Ctx<R>&, void*, int, int, int, cudaStream_t);           \
    template void launch_lp_guess<R>(const Ctx<R>&, const float*, R*, int, int, int, cudaStream_t);   \
    template void launch_lp_target<R>(const Ctx<R>&, const R*, float*, int, int, int, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace gfm
