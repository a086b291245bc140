// lp.cu -- learned initial guess for the pressure-correction (p') equation.
//
// A small 3-D convolutional encoder-decoder maps the Jacobi-scaled right-hand
// side of the p' system to an approximation of its solution; the line solver
// then starts from that guess instead of zero.  Everything here is BF16 on
// the tensor cores with FP32 accumulation (mma.sync m16n8k16), trained on the
// GPU by the kernels below (forward, input gradient, weight gradient, Adam).
//
// Tensors are voxel-major with channels innermost: element (v, c) of a tensor
// with channel stride CS and channel offset CO sits at v*CS + CO + c, voxel
// v = (z*ny + y)*nx + x.  Network (all convolutions 3x3x3, stride 1, zero
// padding 1; 16 input channels of which 2 are used):
//
//   c1: X(16)  -> A1(16) relu          full resolution
//   c2: A1(16) -> CAT[0:16] relu       (E0, the skip)
//   pool: E0   -> P0(16)               2x2x2 average, half resolution
//   c3: P0(16) -> A2(32) relu
//   c4: A2(32) -> E1(32) relu
//   up: E1     -> CAT[16:48]           nearest, full resolution
//   c5: CAT(48)-> A3(16) relu
//   c6: A3(16) -> OUT(16), FP32, linear; channel 0 is the output
//
// Loss: mean over open voxels of (OUT[v][0] - T[v])^2.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gfm_gb300.h"
#include "lp.cuh"

namespace gfm {
namespace lp {

typedef __nv_bfloat16 bf16;

// ---- parameter layout -------------------------------------------------------
const LayerSpec kLayers[kNumLayers] = {
    {16, 16}, {16, 16}, {16, 32}, {32, 32}, {48, 16}, {16, 16}};

int weight_offset(int l) {
    int off = 0;
    for (int i = 0; i < l; ++i) off += 27 * kLayers[i].cin * kLayers[i].cout + kLayers[i].cout;
    return off;
}
int num_params() { return weight_offset(kNumLayers); }

// ---- mma helpers ---------------------------------------------------------------
__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
__device__ __forceinline__ uint32_t ld_pair(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }
__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}


// ---- convolution (forward and input gradient) ---------------------------------
// out[v][co] = bias[co] + sum_t sum_ci in[v + d_t][ci] * W[t][co][ci]
// A block computes a 16 x 4 x 2 voxel tile: the input tile with a one-voxel
// halo (18 x 6 x 4 voxels) and the layer's 27*COUT*CIN weights are staged in
// shared memory once, then warp w computes the 16 voxels of row (w%4, w/4)
// for every tap from there.  The staged channel stride is CIN+8, which keeps
// the eight voxel rows of an A fragment on distinct banks.  Rows of the A
// fragment are voxels, columns input channels; B columns are output channels.
constexpr int kTX = 16, kTY = 4, kTZ = 2;
// one block per tile: with a block staging its halo while others compute,
// this measured faster than resident blocks walking the tiles
constexpr long long kConvBlocks = 1LL << 30;
constexpr int kHX = kTX + 2, kHY = kTY + 2, kHZ = kTZ + 2, kHalo = kHX * kHY * kHZ;
template <int CIN, int COUT>
constexpr size_t conv_smem() { return (size_t)(27 * COUT * CIN + kHalo * (CIN + 8)) * sizeof(bf16); }

template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_conv(Grid3 gd, const bf16* __restrict__ in, int in_cs, int in_co,
                                             const bf16* __restrict__ w, const float* __restrict__ bias,
                                             bf16* __restrict__ out, float* __restrict__ out_f, int out_cs, int out_co,
                                             int relu) {
    constexpr int CP = CIN + 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    bf16* sw = reinterpret_cast<bf16*>(smem_raw);
    bf16* sx = sw + 27 * COUT * CIN;
    {   // the layer's weights, once per block
        const uint32_t* w32 = reinterpret_cast<const uint32_t*>(w);
        uint32_t* sw32 = reinterpret_cast<uint32_t*>(sw);
        for (int i = threadIdx.x; i < 27 * COUT * CIN / 2; i += blockDim.x) sw32[i] = w32[i];
    }
    const int tx_n = (gd.nx + kTX - 1) / kTX, ty_n = (gd.ny + kTY - 1) / kTY, tz_n = (gd.nz + kTZ - 1) / kTZ;
    const int ntiles = tx_n * ty_n * tz_n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, tq = lane & 3;
    const int ty = warp & 3, tz = warp >> 2;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int x0 = (tile % tx_n) * kTX, y0 = ((tile / tx_n) % ty_n) * kTY, z0 = (tile / (tx_n * ty_n)) * kTZ;
        __syncthreads();   // the previous tile's reads of sx are done
        // halo tile, 32-bit words of channel pairs, zero outside the grid
        for (int i = threadIdx.x; i < kHalo * (CIN / 2); i += blockDim.x) {
            const int h = i / (CIN / 2), k = i % (CIN / 2);
            const int hx = h % kHX, hy = (h / kHX) % kHY, hz = h / (kHX * kHY);
            const int x = x0 - 1 + hx, y = y0 - 1 + hy, z = z0 - 1 + hz;
            uint32_t v = 0u;
            if (x >= 0 && x < gd.nx && y >= 0 && y < gd.ny && z >= 0 && z < gd.nz)
                v = ld_pair(in + (size_t)((z * gd.ny + y) * gd.nx + x) * in_cs + in_co + 2 * k);
            *reinterpret_cast<uint32_t*>(sx + (size_t)h * CP + 2 * k) = v;
        }
        __syncthreads();
        float acc[COUT / 8][4];
#pragma unroll
        for (int n = 0; n < COUT / 8; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
        for (int t = 0; t < 27; ++t) {
            const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
            const int hrow = ((tz + dz + 1) * kHY + (ty + dy + 1)) * kHX + dx + 1;
            const bf16* r0 = sx + (size_t)(hrow + g) * CP;
            const bf16* r1 = sx + (size_t)(hrow + g + 8) * CP;
#pragma unroll
            for (int kc = 0; kc < CIN / 16; ++kc) {
                const int c0 = kc * 16 + 2 * tq;
                uint32_t a[4] = {ld_pair(r0 + c0), ld_pair(r1 + c0), ld_pair(r0 + c0 + 8), ld_pair(r1 + c0 + 8)};
#pragma unroll
                for (int n = 0; n < COUT / 8; ++n) {
                    const bf16* wr = sw + ((size_t)t * COUT + n * 8 + g) * CIN + c0;
                    uint32_t b[2] = {ld_pair(wr), ld_pair(wr + 8)};
                    mma16816(acc[n], a, b);
                }
            }
        }
        // epilogue: bias, relu, store (rows g and g+8, columns 2tq, 2tq+1 of each n-tile)
        const int y = y0 + ty, z = z0 + tz;
        if (y >= gd.ny || z >= gd.nz) continue;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int x = x0 + g + 8 * h;
            if (x >= gd.nx) continue;
            const int v = (z * gd.ny + y) * gd.nx + x;
#pragma unroll
            for (int n = 0; n < COUT / 8; ++n) {
                const int co = n * 8 + 2 * tq;
                float q0 = acc[n][2 * h], q1 = acc[n][2 * h + 1];
                if (bias) { q0 += bias[co]; q1 += bias[co + 1]; }
                if (relu) { q0 = fmaxf(q0, 0.f); q1 = fmaxf(q1, 0.f); }
                const size_t o = (size_t)v * out_cs + out_co + co;
                if (out_f) { out_f[o] = q0; out_f[o + 1] = q1; }
                else *reinterpret_cast<uint32_t*>(out + o) = pack2(__float2bfloat16_rn(q0), __float2bfloat16_rn(q1));
            }
        }
    }
}

// ---- weight gradient ------------------------------------------------------------
// dW[t][co][ci] += sum_v dy[v][co] * x[v + d_t][ci]: a GEMM with M = co, N = ci,
// K = voxels.  Block (chunk of voxels, tap): each warp takes 16-voxel slices
// of the chunk; the warps' sums are added in warp order and the block writes
// its partial to part[chunk][t][co][ci]; k_wgrad_sum adds the chunks in
// order, so the gradient does not depend on scheduling.
constexpr int kWgChunk = 2048;   // voxels per block
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_wgrad(Grid3 gd, const bf16* __restrict__ dy, int dy_cs, int dy_co,
                                              const bf16* __restrict__ x, int x_cs, int x_co, float* __restrict__ part) {
    __shared__ float red[8][COUT * CIN];
    const int t = blockIdx.y;
    const int dx = t % 3 - 1, dyy = (t / 3) % 3 - 1, dz = t / 9 - 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int g = lane >> 2, tq = lane & 3;
    const int nv = gd.nvox();
    float acc[COUT / 16][CIN / 8][4];
#pragma unroll
    for (int m = 0; m < COUT / 16; ++m)
#pragma unroll
        for (int n = 0; n < CIN / 8; ++n) acc[m][n][0] = acc[m][n][1] = acc[m][n][2] = acc[m][n][3] = 0.f;
    const int vbeg = blockIdx.x * kWgChunk;
    for (int s = vbeg + warp * 16; s < vbeg + kWgChunk && s < nv; s += nwarp * 16) {
        // K index k <-> voxel s + k; this thread needs k = 2tq, 2tq+1, 2tq+8, 2tq+9
        int kv[4] = {s + 2 * tq, s + 2 * tq + 1, s + 2 * tq + 8, s + 2 * tq + 9};
        const bf16* xs[4];
        bool din[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int v = kv[q];
            din[q] = v < nv;
            const int vv = din[q] ? v : 0;
            const int x0 = vv % gd.nx, y0 = (vv / gd.nx) % gd.ny, z0 = vv / (gd.nx * gd.ny);
            const int xx = x0 + dx, yy = y0 + dyy, zz = z0 + dz;
            const bool ok = din[q] && xx >= 0 && xx < gd.nx && yy >= 0 && yy < gd.ny && zz >= 0 && zz < gd.nz;
            xs[q] = ok ? x + (size_t)((zz * gd.ny + yy) * gd.nx + xx) * x_cs + x_co : nullptr;
        }
        const bf16 zero = __float2bfloat16_rn(0.f);
#pragma unroll
        for (int m = 0; m < COUT / 16; ++m) {
            // A (M=co x K=voxel, row-major): a0 = (co g, k 2tq..+1), a1 = (co g+8, ...), a2/a3 with k+8
            uint32_t a[4];
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int co = m * 16 + g + 8 * hh;
                const bf16 e0 = din[0] ? dy[(size_t)kv[0] * dy_cs + dy_co + co] : zero;
                const bf16 e1 = din[1] ? dy[(size_t)kv[1] * dy_cs + dy_co + co] : zero;
                const bf16 e2 = din[2] ? dy[(size_t)kv[2] * dy_cs + dy_co + co] : zero;
                const bf16 e3 = din[3] ? dy[(size_t)kv[3] * dy_cs + dy_co + co] : zero;
                a[hh] = pack2(e0, e1);
                a[2 + hh] = pack2(e2, e3);
            }
#pragma unroll
            for (int n = 0; n < CIN / 8; ++n) {
                // B (K=voxel x N=ci): b0 = (k 2tq..+1, ci g), b1 = (k 2tq+8..+9, ci g)
                const int ci = n * 8 + g;
                const bf16 f0 = xs[0] ? xs[0][ci] : zero;
                const bf16 f1 = xs[1] ? xs[1][ci] : zero;
                const bf16 f2 = xs[2] ? xs[2][ci] : zero;
                const bf16 f3 = xs[3] ? xs[3][ci] : zero;
                uint32_t b[2] = {pack2(f0, f1), pack2(f2, f3)};
                mma16816(acc[m][n], a, b);
            }
        }
    }
    // D (M=co x N=ci): d0,d1 = (co g, ci 2tq..+1), d2,d3 = (co g+8, ...); each
    // element of the warp's tile is held by exactly one lane
    float* mine = red[warp];
#pragma unroll
    for (int m = 0; m < COUT / 16; ++m)
#pragma unroll
        for (int n = 0; n < CIN / 8; ++n) {
            const int co = m * 16 + g, ci = n * 8 + 2 * tq;
            mine[co * CIN + ci] = acc[m][n][0];
            mine[co * CIN + ci + 1] = acc[m][n][1];
            mine[(co + 8) * CIN + ci] = acc[m][n][2];
            mine[(co + 8) * CIN + ci + 1] = acc[m][n][3];
        }
    __syncthreads();
    for (int i = threadIdx.x; i < COUT * CIN; i += blockDim.x) {
        float s = 0.f;
        for (int w = 0; w < nwarp; ++w) s += red[w][i];
        part[((size_t)blockIdx.x * 27 + t) * COUT * CIN + i] = s;
    }
}
// dw[i] += sum over chunks of part[chunk][i], in chunk order
__global__ void k_wgrad_sum(int nchunk, int n, const float* __restrict__ part, float* __restrict__ dw) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int c = 0; c < nchunk; ++c) s += part[(size_t)c * n + i];
        dw[i] += s;
    }
}

// bias gradient: db[co] += sum_v dy[v][co]; one block per channel, fixed order
__global__ void k_bgrad(int nv, int cout, const bf16* __restrict__ dy, int dy_cs, int dy_co, float* __restrict__ db) {
    __shared__ float sh[256];
    const int co = blockIdx.x;
    float s = 0.f;
    for (int v = threadIdx.x; v < nv; v += blockDim.x) s += __bfloat162float(dy[(size_t)v * dy_cs + dy_co + co]);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[co] += sh[0];
}

// ---- pooling, upsampling, activation gradient -----------------------------------
// fine grid (nx,ny,nz) even in every direction; coarse = half
__global__ void k_pool(Grid3 fine, const bf16* __restrict__ in, int in_cs, int in_co, bf16* __restrict__ out, int c) {
    const int cx = fine.nx / 2, cy = fine.ny / 2, cz = fine.nz / 2;
    const int n = cx * cy * cz * c;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ch = i % c, vc = i / c;
        const int x = vc % cx, y = (vc / cx) % cy, z = vc / (cx * cy);
        float s = 0.f;
        for (int q = 0; q < 8; ++q) {
            const int fx = 2 * x + (q & 1), fy = 2 * y + ((q >> 1) & 1), fz = 2 * z + (q >> 2);
            s += __bfloat162float(in[(size_t)((fz * fine.ny + fy) * fine.nx + fx) * in_cs + in_co + ch]);
        }
        out[(size_t)vc * c + ch] = __float2bfloat16_rn(s * 0.125f);
    }
}
// d_in[fine] = d_skip[fine] + d_out[coarse]/8  (the skip tensor's own gradient plus the pool's)
__global__ void k_pool_bwd(Grid3 fine, const bf16* __restrict__ dskip, int ds_cs, int ds_co,
                           const bf16* __restrict__ dout, bf16* __restrict__ din, int c) {
    const int n = fine.nvox() * c;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ch = i % c, v = i / c;
        const int x = v % fine.nx, y = (v / fine.nx) % fine.ny, z = v / (fine.nx * fine.ny);
        const int vc = ((z / 2) * (fine.ny / 2) + y / 2) * (fine.nx / 2) + x / 2;
        const float s = __bfloat162float(dskip[(size_t)v * ds_cs + ds_co + ch]) + 0.125f * __bfloat162float(dout[(size_t)vc * c + ch]);
        din[(size_t)v * c + ch] = __float2bfloat16_rn(s);
    }
}
// one thread per fine voxel, channels copied 8 at a time (16-byte vectors:
// c, out_cs and out_co are multiples of 8)
__global__ void k_up(Grid3 fine, const bf16* __restrict__ in, bf16* __restrict__ out, int out_cs, int out_co, int c) {
    const int n = fine.nvox();
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int x = v % fine.nx, y = (v / fine.nx) % fine.ny, z = v / (fine.nx * fine.ny);
        const int vc = ((z / 2) * (fine.ny / 2) + y / 2) * (fine.nx / 2) + x / 2;
        const uint4* src = reinterpret_cast<const uint4*>(in + (size_t)vc * c);
        uint4* dst = reinterpret_cast<uint4*>(out + (size_t)v * out_cs + out_co);
        for (int q = 0; q < c / 8; ++q) dst[q] = src[q];
    }
}
__global__ void k_up_bwd(Grid3 fine, const bf16* __restrict__ dout, int do_cs, int do_co, bf16* __restrict__ din, int c) {
    const int cx = fine.nx / 2, cy = fine.ny / 2, cz = fine.nz / 2;
    const int n = cx * cy * cz * c;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ch = i % c, vc = i / c;
        const int x = vc % cx, y = (vc / cx) % cy, z = vc / (cx * cy);
        float s = 0.f;
        for (int q = 0; q < 8; ++q) {
            const int fx = 2 * x + (q & 1), fy = 2 * y + ((q >> 1) & 1), fz = 2 * z + (q >> 2);
            s += __bfloat162float(dout[(size_t)((fz * fine.ny + fy) * fine.nx + fx) * do_cs + do_co + ch]);
        }
        din[(size_t)vc * c + ch] = __float2bfloat16_rn(s);
    }
}
// dy *= (y > 0), y read with its own stride
__global__ void k_relu_bwd(int nv, int c, bf16* __restrict__ dy, int dy_cs, int dy_co, const bf16* __restrict__ y,
                           int y_cs, int y_co) {
    const int n = nv * c;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ch = i % c, v = i / c;
        if (!(__bfloat162float(y[(size_t)v * y_cs + y_co + ch]) > 0.f)) dy[(size_t)v * dy_cs + dy_co + ch] = __float2bfloat16_rn(0.f);
    }
}

// ---- loss, optimiser, weight staging ----------------------------------------------
// dout[v][0] = 2 (out[v][0] - t[v]) / nopen on open voxels (feature channel 1 = 1), 0 elsewhere;
// sums of the squared error and of the open count into acc[0], acc[1]
__global__ void k_loss(int nv, const float* __restrict__ out, const bf16* __restrict__ feat, const float* __restrict__ tgt,
                       const float* __restrict__ nopen, bf16* __restrict__ dout, double* acc) {
    __shared__ double sh[2][32];
    double se = 0.0, no = 0.0;
    const float inv = 1.f / fmaxf(nopen[0], 1.f);
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        const bool open = __bfloat162float(feat[(size_t)v * 16 + 1]) > 0.5f;
        const float e = open ? out[(size_t)v * 16] - tgt[v] : 0.f;
        for (int c = 0; c < 16; ++c) dout[(size_t)v * 16 + c] = __float2bfloat16_rn(c == 0 ? 2.f * e * inv : 0.f);
        se += (double)e * e;
        no += open ? 1.0 : 0.0;
    }
    for (int o = 16; o > 0; o >>= 1) {
        se += __shfl_down_sync(0xffffffffu, se, o);
        no += __shfl_down_sync(0xffffffffu, no, o);
    }
    if ((threadIdx.x & 31) == 0) { sh[0][threadIdx.x >> 5] = se; sh[1][threadIdx.x >> 5] = no; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { a += sh[0][w]; b += sh[1][w]; }
        atomicAdd(&acc[0], a);
        atomicAdd(&acc[1], b);
    }
}
// number of open voxels (feature channel 1) -> nopen[0]
__global__ void k_count_open(int nv, const bf16* __restrict__ feat, float* nopen) {
    float s = 0.f;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x)
        s += __bfloat162float(feat[(size_t)v * 16 + 1]) > 0.5f ? 1.f : 0.f;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(nopen, s);
}
__global__ void k_adam(int n, float* __restrict__ p, float* __restrict__ gr, float* __restrict__ m, float* __restrict__ v,
                       float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = gr[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        gr[i] = 0.f;
    }
}
// BF16 copies of a layer's weights: forward W[t][co][ci] and, for the input
// gradient, the mirrored transpose WT[26-t][ci][co]
__global__ void k_stage(int cin, int cout, const float* __restrict__ wf, bf16* __restrict__ w, bf16* __restrict__ wt) {
    const int n = 27 * cin * cout;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ci = i % cin, co = (i / cin) % cout, t = i / (cin * cout);
        const bf16 b = __float2bfloat16_rn(wf[i]);
        w[i] = b;
        wt[((size_t)(26 - t) * cin + ci) * cout + co] = b;
    }
}

// ---- the network ------------------------------------------------------------------
inline int nblk(long long n, int t = 256) {
    long long b = (n + t - 1) / t;
    return (int)(b < 1 ? 1 : (b > 8192 ? 8192 : b));
}

template <int CIN, int COUT>
int conv_attr() {
    return cudaFuncSetAttribute(k_conv<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)conv_smem<CIN, COUT>()) == cudaSuccess;
}
template <int CIN, int COUT>
void conv(const Grid3& gd, const bf16* in, int in_cs, int in_co, const bf16* w, const float* bias, bf16* out, float* out_f,
          int out_cs, int out_co, bool relu, cudaStream_t st) {
    const long long ntiles = (long long)((gd.nx + kTX - 1) / kTX) * ((gd.ny + kTY - 1) / kTY) * ((gd.nz + kTZ - 1) / kTZ);
    const int blocks = (int)(ntiles < kConvBlocks ? ntiles : kConvBlocks);
    k_conv<CIN, COUT><<<blocks, 256, conv_smem<CIN, COUT>(), st>>>(gd, in, in_cs, in_co, w, bias, out, out_f, out_cs,
                                                                    out_co, relu ? 1 : 0);
}
template <int CIN, int COUT>
void wgrad(const Grid3& gd, const bf16* dy, int dy_cs, int dy_co, const bf16* x, int x_cs, int x_co, float* dw, float* part,
           cudaStream_t st) {
    const long long nv = (long long)gd.nx * gd.ny * gd.nz;
    const int nchunk = (int)((nv + kWgChunk - 1) / kWgChunk);
    k_wgrad<CIN, COUT><<<dim3(nchunk, 27), 256, 0, st>>>(gd, dy, dy_cs, dy_co, x, x_cs, x_co, part);
    const int n = 27 * CIN * COUT;
    k_wgrad_sum<<<nblk(n), 256, 0, st>>>(nchunk, n, part, dw);
}

int Net::create(int nx, int ny, int nz, uint64_t seed) {
    if (nx < 2 || ny < 2 || nz < 2 || (nx & 1) || (ny & 1) || (nz & 1)) { err = "grid dimensions must be even"; return GFM_E_ARG; }
    if ((long long)nx * ny * nz * 48 >= (1LL << 31)) { err = "grid too large"; return GFM_E_ARG; }
    mx = nx; my = ny; mz = nz;
    if (!(conv_attr<16, 16>() && conv_attr<16, 32>() && conv_attr<32, 32>() && conv_attr<48, 16>() &&
          conv_attr<16, 48>() && conv_attr<32, 16>())) {
        err = "cannot raise the shared-memory limit of the convolution kernels";
        return GFM_E_CUDA;
    }
    const long long v0 = (long long)nx * ny * nz, v1 = v0 / 8;
    np = num_params();
    auto fal = [&](float** p, long long n) { return cudaMalloc((void**)p, sizeof(float) * (n > 0 ? n : 1)) == cudaSuccess; };
    auto bal = [&](bf16** p, long long n) { return cudaMalloc((void**)p, sizeof(bf16) * (n > 0 ? n : 1)) == cudaSuccess; };
    bool ok = fal(&p32, np) && fal(&g32, np) && fal(&m32, np) && fal(&v32, np) && fal(&nopen, 1) &&
              cudaMalloc((void**)&lacc, 2 * sizeof(double)) == cudaSuccess;
    for (int l = 0; l < kNumLayers; ++l) {
        const long long nw = 27LL * kLayers[l].cin * kLayers[l].cout;
        ok = ok && bal(&w16[l], nw) && bal(&wt16[l], nw) && bal(&wtc[l], nw);
    }
    ok = ok && cudaMalloc((void**)&tc_err, sizeof(int)) == cudaSuccess;
    ok = ok && fal(&wg_part, ((v0 + kWgChunk - 1) / kWgChunk) * 27LL * 1024);   // chunks x taps x the largest cout*cin
    ok = ok && bal(&A1, v0 * 16) && bal(&CAT, v0 * 48) && bal(&P0, v1 * 16) && bal(&A2, v1 * 32) && bal(&E1, v1 * 32) &&
         bal(&A3, v0 * 16) && fal(&OUT, v0 * 16) && bal(&dOUT, v0 * 16) && bal(&dA3, v0 * 16) && bal(&dCAT, v0 * 48) &&
         bal(&dE1, v1 * 32) && bal(&dA2, v1 * 32) && bal(&dP0, v1 * 16) && bal(&dE0, v0 * 16) && bal(&dA1, v0 * 16);
    if (!ok) { err = "device allocation failed"; return GFM_E_NOMEM; }
    // He-uniform initial weights from splitmix64, zero biases
    std::vector<float> h((size_t)np, 0.f);
    uint64_t s = seed ? seed : 0x9e3779b97f4a7c15ull;
    auto next = [&]() {
        s += 0x9e3779b97f4a7c15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return (double)((z ^ (z >> 31)) >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < kNumLayers; ++l) {
        const int off = weight_offset(l), fan_in = 27 * kLayers[l].cin;
        const double a = std::sqrt(6.0 / fan_in) * (l == kNumLayers - 1 ? 0.1 : 1.0);
        for (int i = 0; i < 27 * kLayers[l].cin * kLayers[l].cout; ++i) {
            const int ci = i % kLayers[l].cin, co = (i / kLayers[l].cin) % kLayers[l].cout;
            float wv = (float)((2.0 * next() - 1.0) * a);
            if (l == 0 && ci >= kFeatChannels) wv = 0.f;   // unused input channels
            if (l == kNumLayers - 1 && co > 0) wv = 0.f;   // only output channel 0 is read
            h[off + i] = wv;
        }
    }
    if (cudaMemcpy(p32, h.data(), sizeof(float) * np, cudaMemcpyHostToDevice) != cudaSuccess) return GFM_E_CUDA;
    cudaMemset(tc_err, 0, sizeof(int));
    {
        const char* w = std::getenv("GFM_LP_WAIT1");
        tc_wait1 = w ? std::atoi(w) : -1;
    }
    if (prepare_tc() != GFM_OK) { err = "cannot raise the shared-memory limit of the tcgen05 convolutions"; return GFM_E_CUDA; }
    cudaMemset(g32, 0, sizeof(float) * np);
    cudaMemset(m32, 0, sizeof(float) * np);
    cudaMemset(v32, 0, sizeof(float) * np);
    stage(0);
    return cudaDeviceSynchronize() == cudaSuccess ? GFM_OK : GFM_E_CUDA;
}

void Net::release() {
    void* ps[] = {p32, g32, m32, v32, nopen, lacc, A1, CAT, P0, A2, E1, A3, OUT, dOUT, dA3, dCAT, dE1, dA2, dP0, dE0, dA1, tc_err,
                  wg_part};
    for (void* p : ps) if (p) cudaFree(p);
    for (int l = 0; l < kNumLayers; ++l) {
        if (w16[l]) cudaFree(w16[l]);
        if (wt16[l]) cudaFree(wt16[l]);
        if (wtc[l]) cudaFree(wtc[l]);
    }
}

void Net::stage(cudaStream_t st) {
    for (int l = 0; l < kNumLayers; ++l) {
        const int n = 27 * kLayers[l].cin * kLayers[l].cout;
        k_stage<<<nblk(n), 256, 0, st>>>(kLayers[l].cin, kLayers[l].cout, p32 + weight_offset(l), w16[l], wt16[l]);
        stage_tc(kLayers[l].cin, kLayers[l].cout, p32 + weight_offset(l), wtc[l], st);
    }
}

int Net::check_dims(int nx, int ny, int nz) const {
    if (nx < 2 || ny < 2 || nz < 2 || (nx & 1) || (ny & 1) || (nz & 1)) return GFM_E_ARG;
    if ((long long)nx * ny * nz > (long long)mx * my * mz) return GFM_E_LIMIT;
    return GFM_OK;
}

void Net::forward(const bf16* X, int nx, int ny, int nz, cudaStream_t st) {
    const Grid3 f{nx, ny, nz}, c{nx / 2, ny / 2, nz / 2};
    const float* b = p32;
    auto bias = [&](int l) { return b + weight_offset(l) + 27 * kLayers[l].cin * kLayers[l].cout; };
    if (use_tc) {
        conv_tc<16, 16>(f, X, 16, 0, wtc[0], bias(0), A1, nullptr, 16, 0, true, tc_err, tc_wait1, st);
        conv_tc<16, 16>(f, A1, 16, 0, wtc[1], bias(1), CAT, nullptr, 48, 0, true, tc_err, tc_wait1, st);
    } else {
        conv<16, 16>(f, X, 16, 0, w16[0], bias(0), A1, nullptr, 16, 0, true, st);
        conv<16, 16>(f, A1, 16, 0, w16[1], bias(1), CAT, nullptr, 48, 0, true, st);
    }
    k_pool<<<nblk((long long)c.nx * c.ny * c.nz * 16), 256, 0, st>>>(f, CAT, 48, 0, P0, 16);
    if (use_tc) {
        conv_tc<16, 32>(c, P0, 16, 0, wtc[2], bias(2), A2, nullptr, 32, 0, true, tc_err, tc_wait1, st);
        conv_tc<32, 32>(c, A2, 32, 0, wtc[3], bias(3), E1, nullptr, 32, 0, true, tc_err, tc_wait1, st);
    } else {
        conv<16, 32>(c, P0, 16, 0, w16[2], bias(2), A2, nullptr, 32, 0, true, st);
        conv<32, 32>(c, A2, 32, 0, w16[3], bias(3), E1, nullptr, 32, 0, true, st);
    }
    k_up<<<nblk((long long)nx * ny * nz), 256, 0, st>>>(f, E1, CAT, 48, 16, 32);
    if (use_tc) {
        conv_tc<48, 16>(f, CAT, 48, 0, wtc[4], bias(4), A3, nullptr, 16, 0, true, tc_err, tc_wait1, st);
        conv_tc<16, 16>(f, A3, 16, 0, wtc[5], bias(5), nullptr, OUT, 16, 0, false, tc_err, tc_wait1, st);
    } else {
        conv<48, 16>(f, CAT, 48, 0, w16[4], bias(4), A3, nullptr, 16, 0, true, st);
        conv<16, 16>(f, A3, 16, 0, w16[5], bias(5), nullptr, OUT, 16, 0, false, st);
    }
}

// gradients of the loss for one sample, accumulated into g32
void Net::backward(const bf16* X, const float* T, int nx, int ny, int nz, cudaStream_t st) {
    const Grid3 f{nx, ny, nz}, c{nx / 2, ny / 2, nz / 2};
    const int v0 = nx * ny * nz, v1 = v0 / 8;
    auto dw = [&](int l) { return g32 + weight_offset(l); };
    auto db = [&](int l) { return g32 + weight_offset(l) + 27 * kLayers[l].cin * kLayers[l].cout; };
    cudaMemsetAsync(nopen, 0, sizeof(float), st);
    k_count_open<<<nblk(v0), 256, 0, st>>>(v0, X, nopen);
    k_loss<<<nblk(v0), 256, 0, st>>>(v0, OUT, X, T, nopen, dOUT, lacc);
    // c6: A3 -> OUT (linear)
    wgrad<16, 16>(f, dOUT, 16, 0, A3, 16, 0, dw(5), wg_part, st);
    k_bgrad<<<16, 256, 0, st>>>(v0, 16, dOUT, 16, 0, db(5));
    conv<16, 16>(f, dOUT, 16, 0, wt16[5], nullptr, dA3, nullptr, 16, 0, false, st);
    k_relu_bwd<<<nblk((long long)v0 * 16), 256, 0, st>>>(v0, 16, dA3, 16, 0, A3, 16, 0);
    // c5: CAT -> A3
    wgrad<48, 16>(f, dA3, 16, 0, CAT, 48, 0, dw(4), wg_part, st);
    k_bgrad<<<16, 256, 0, st>>>(v0, 16, dA3, 16, 0, db(4));
    conv<16, 48>(f, dA3, 16, 0, wt16[4], nullptr, dCAT, nullptr, 48, 0, false, st);
    // up: E1 -> CAT[16:48]
    k_up_bwd<<<nblk((long long)v1 * 32), 256, 0, st>>>(f, dCAT, 48, 16, dE1, 32);
    k_relu_bwd<<<nblk((long long)v1 * 32), 256, 0, st>>>(v1, 32, dE1, 32, 0, E1, 32, 0);
    // c4: A2 -> E1
    wgrad<32, 32>(c, dE1, 32, 0, A2, 32, 0, dw(3), wg_part, st);
    k_bgrad<<<32, 256, 0, st>>>(v1, 32, dE1, 32, 0, db(3));
    conv<32, 32>(c, dE1, 32, 0, wt16[3], nullptr, dA2, nullptr, 32, 0, false, st);
    k_relu_bwd<<<nblk((long long)v1 * 32), 256, 0, st>>>(v1, 32, dA2, 32, 0, A2, 32, 0);
    // c3: P0 -> A2
    wgrad<16, 32>(c, dA2, 32, 0, P0, 16, 0, dw(2), wg_part, st);
    k_bgrad<<<32, 256, 0, st>>>(v1, 32, dA2, 32, 0, db(2));
    conv<32, 16>(c, dA2, 32, 0, wt16[2], nullptr, dP0, nullptr, 16, 0, false, st);
    // pool: E0 = CAT[0:16] -> P0; E0 also feeds c5 directly
    k_pool_bwd<<<nblk((long long)v0 * 16), 256, 0, st>>>(f, dCAT, 48, 0, dP0, dE0, 16);
    k_relu_bwd<<<nblk((long long)v0 * 16), 256, 0, st>>>(v0, 16, dE0, 16, 0, CAT, 48, 0);
    // c2: A1 -> E0
    wgrad<16, 16>(f, dE0, 16, 0, A1, 16, 0, dw(1), wg_part, st);
    k_bgrad<<<16, 256, 0, st>>>(v0, 16, dE0, 16, 0, db(1));
    conv<16, 16>(f, dE0, 16, 0, wt16[1], nullptr, dA1, nullptr, 16, 0, false, st);
    k_relu_bwd<<<nblk((long long)v0 * 16), 256, 0, st>>>(v0, 16, dA1, 16, 0, A1, 16, 0);
    // c1: X -> A1
    wgrad<16, 16>(f, dA1, 16, 0, X, 16, 0, dw(0), wg_part, st);
    k_bgrad<<<16, 256, 0, st>>>(v0, 16, dA1, 16, 0, db(0));
}

void Net::adam(float lr, int step, cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
    k_adam<<<nblk(np), 256, 0, st>>>(np, p32, g32, m32, v32, lr, b1, b2, 1e-8f, c1, c2);
    stage(st);
}

}  // namespace lp
}  // namespace gfm

// ---- C ABI ---------------------------------------------------------------------------
using gfm::lp::Net;
using gfm::lp::bf16;

namespace {
thread_local std::string g_lp_err;
}

extern "C" int gfm_lp_create(int nx, int ny, int nz, uint64_t seed, gfm_lp** out) {
    if (!out) return GFM_E_ARG;
    *out = nullptr;
    Net* n = new (std::nothrow) Net();
    if (!n) return GFM_E_NOMEM;
    int rc = n->create(nx, ny, nz, seed);
    if (rc != GFM_OK) {
        g_lp_err = n->err;
        n->release();
        delete n;
        return rc;
    }
    *out = reinterpret_cast<gfm_lp*>(n);
    return GFM_OK;
}
extern "C" void gfm_lp_destroy(gfm_lp* lp) {
    if (!lp) return;
    Net* n = reinterpret_cast<Net*>(lp);
    cudaDeviceSynchronize();
    n->release();
    delete n;
}
extern "C" int gfm_lp_num_params(void) { return gfm::lp::num_params(); }
extern "C" int gfm_lp_get_params(gfm_lp* lp, float* params, float* grads) {
    if (!lp) return GFM_E_ARG;
    Net* n = reinterpret_cast<Net*>(lp);
    if (cudaDeviceSynchronize() != cudaSuccess) return GFM_E_CUDA;
    if (params && cudaMemcpy(params, n->p32, sizeof(float) * n->np, cudaMemcpyDeviceToHost) != cudaSuccess) return GFM_E_CUDA;
    if (grads && cudaMemcpy(grads, n->g32, sizeof(float) * n->np, cudaMemcpyDeviceToHost) != cudaSuccess) return GFM_E_CUDA;
    return GFM_OK;
}
extern "C" int gfm_lp_set_params(gfm_lp* lp, const float* params) {
    if (!lp || !params) return GFM_E_ARG;
    Net* n = reinterpret_cast<Net*>(lp);
    for (int i = 0; i < n->np; ++i) if (!std::isfinite(params[i])) return GFM_E_NAN;
    if (cudaMemcpy(n->p32, params, sizeof(float) * n->np, cudaMemcpyHostToDevice) != cudaSuccess) return GFM_E_CUDA;
    cudaMemset(n->g32, 0, sizeof(float) * n->np);
    cudaMemset(n->m32, 0, sizeof(float) * n->np);
    cudaMemset(n->v32, 0, sizeof(float) * n->np);
    n->stage(0);
    return cudaDeviceSynchronize() == cudaSuccess ? GFM_OK : GFM_E_CUDA;
}
extern "C" int gfm_lp_forward(gfm_lp* lp, const void* feats, float* out, int nx, int ny, int nz, void* stream) {
    if (!lp || !feats) return GFM_E_ARG;
    Net* n = reinterpret_cast<Net*>(lp);
    int rc = n->check_dims(nx, ny, nz);
    if (rc != GFM_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    n->forward(static_cast<const bf16*>(feats), nx, ny, nz, st);
    if (out) {
        const long long v0 = (long long)nx * ny * nz;
        // channel 0 of OUT -> out (strided copy)
        if (cudaMemcpy2DAsync(out, sizeof(float), n->OUT, 16 * sizeof(float), sizeof(float), (size_t)v0,
                              cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            return GFM_E_CUDA;
    }
    return cudaGetLastError() == cudaSuccess ? GFM_OK : GFM_E_CUDA;
}
extern "C" int gfm_lp_train_step(gfm_lp* lp, const void* feats, const float* target, int nx, int ny, int nz, float lr,
                                 int update, double* loss, void* stream) {
    if (!lp || !feats || !target) return GFM_E_ARG;
    Net* n = reinterpret_cast<Net*>(lp);
    int rc = n->check_dims(nx, ny, nz);
    if (rc != GFM_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaMemsetAsync(n->lacc, 0, 2 * sizeof(double), st);
    n->forward(static_cast<const bf16*>(feats), nx, ny, nz, st);
    n->backward(static_cast<const bf16*>(feats), target, nx, ny, nz, st);
    if (update) n->adam(lr, ++n->steps, st);
    if (loss) {
        double h[2];
        if (cudaMemcpyAsync(h, n->lacc, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess) return GFM_E_CUDA;
        if (cudaStreamSynchronize(st) != cudaSuccess) return GFM_E_CUDA;
        *loss = h[1] > 0 ? h[0] / h[1] : 0.0;
    }
    return cudaGetLastError() == cudaSuccess ? GFM_OK : GFM_E_CUDA;
}
extern "C" int gfm_lp_set_tensor_path(gfm_lp* lp, int tcgen05) {
    if (!lp) return GFM_E_ARG;
    reinterpret_cast<Net*>(lp)->use_tc = tcgen05 != 0;
    return GFM_OK;
}
// 0: every tcgen05 tile's first bounded wait for its MMAs succeeded; 1: a
// first wait ran out (the second one saw the MMAs end, output written); 2: a
// tile gave up (output not written, the pass's result invalid)
extern "C" int gfm_lp_tensor_status(gfm_lp* lp) {
    if (!lp) return GFM_E_ARG;
    Net* n = reinterpret_cast<Net*>(lp);
    int v = 0;
    if (cudaDeviceSynchronize() != cudaSuccess) return GFM_E_CUDA;
    if (cudaMemcpy(&v, n->tc_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return GFM_E_CUDA;
    return v;
}
extern "C" const char* gfm_lp_last_error(void) { return g_lp_err.c_str(); }
