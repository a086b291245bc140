// lp_tc.cu -- forward convolution of the learned p' guess on the fifth-
// generation tensor cores (tcgen05.mma, accumulator in tensor memory).
//
// Same operation as k_conv in lp.cu: out[v][co] = bias[co] +
// sum_t sum_ci in[v + d_t][ci] * W[t][co][ci], 3x3x3 taps, zero padding.
//
// A CTA computes a tile of 8 (x) by 16 (y) voxels of one z-slice: M = 128
// rows of the implicit GEMM, N = COUT, K = 27 taps x CIN in steps of 16.
// Operands sit in shared memory in the no-swizzle K-major layout of
// 8-row x 16-byte core matrices:
//   A, the input tile with a one-voxel halo, [hz][hy][c8][hx][8 channels]:
//     for tap (dx,dy,dz) the 128 x 16 operand starts at (dz+1, dy+1, c8, dx+1);
//     its 8 rows of a core matrix are 8 consecutive x (16 B apart), the next
//     core matrix along M is the next y row (C8*HX*16 B), along K the next
//     channel group (HX*16 B);
//   B, the weights, [t][c8][co][8 channels]: next core matrix along N is
//     +128 B, along K +COUT*16 B.
// One thread issues the 27*CIN/16 MMAs; their completion arrives on an
// mbarrier (bounded wait, error flag on expiry); the four warps then read
// their 32 TMEM lanes (= voxel rows) with tcgen05.ld and store the result.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/gfm_gb300.h"
#include "lp.cuh"

namespace gfm {
namespace lp {

typedef __nv_bfloat16 bf16;

constexpr int kTcX = 8, kTcY = 16;   // tile: 128 voxels = M
constexpr int kTcHX = kTcX + 2, kTcHY = kTcY + 2, kTcHZ = 3;
constexpr int kTcThreads = 128;
constexpr int kTcWaitLimit = 1 << 22;   // mbarrier polls before the tile gives up

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: no swizzle, K-major core matrices
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo_k, uint32_t sbo_mn) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo_k >> 4) & 0x3FFFu) << 16;    // leading byte offset: next core matrix along K
    d |= (uint64_t)((sbo_mn >> 4) & 0x3FFFu) << 32;   // stride byte offset: next core matrix along M/N
    d |= (uint64_t)1 << 46;                           // descriptor version of tcgen05
    return d;                                         // base offset 0, layout: no swizzle
}
// instruction descriptor, kind::f16: D f32, A and B bf16, both K-major
__host__ __device__ constexpr uint32_t umma_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity, int limit) {
    for (int i = 0; i < limit; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(addr), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

template <int CIN, int COUT>
struct TcShape {
    static constexpr int C8 = CIN / 8;
    static constexpr int A_BYTES = kTcHZ * kTcHY * C8 * kTcHX * 16;
    static constexpr int B_BYTES = 27 * C8 * COUT * 16;
    static constexpr int B_PAD = 4096;   // keeps every descriptor reach inside the allocation
    static constexpr int TCOLS = COUT <= 32 ? 32 : 64;
    static constexpr size_t SMEM = (size_t)A_BYTES + B_BYTES + B_PAD + 64;
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(kTcThreads) k_conv_tc(Grid3 gd, const bf16* __restrict__ in, int in_cs, int in_co,
                                                       const bf16* __restrict__ wtc, const float* __restrict__ bias,
                                                       bf16* __restrict__ out, float* __restrict__ out_f, int out_cs,
                                                       int out_co, int relu, int* err, int wait1) {
    using S = TcShape<CIN, COUT>;
    constexpr int C8 = S::C8;
    extern __shared__ __align__(128) unsigned char sm[];
    unsigned char* sA = sm;
    unsigned char* sB = sm + S::A_BYTES;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sB + S::B_BYTES + S::B_PAD);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tx_n = (gd.nx + kTcX - 1) / kTcX;
    const int x0 = (blockIdx.x % tx_n) * kTcX, y0 = (blockIdx.x / tx_n) * kTcY, z0 = blockIdx.y;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(S::TCOLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    // weights (already in the core-matrix order) and the halo tile, 16 bytes at a time
    {
        const uint4* wsrc = reinterpret_cast<const uint4*>(wtc);
        uint4* wdst = reinterpret_cast<uint4*>(sB);
        for (int i = tid; i < S::B_BYTES / 16; i += kTcThreads) wdst[i] = wsrc[i];
        uint4* adst = reinterpret_cast<uint4*>(sA);
        for (int i = tid; i < S::A_BYTES / 16; i += kTcThreads) {
            const int hx = i % kTcHX, c8 = (i / kTcHX) % C8, hy = (i / (kTcHX * C8)) % kTcHY, hz = i / (kTcHX * C8 * kTcHY);
            const int x = x0 - 1 + hx, y = y0 - 1 + hy, z = z0 - 1 + hz;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (x >= 0 && x < gd.nx && y >= 0 && y < gd.ny && z >= 0 && z < gd.nz)
                v = *reinterpret_cast<const uint4*>(in + (size_t)((z * gd.ny + y) * gd.nx + x) * in_cs + in_co + c8 * 8);
            adst[i] = v;
        }
    }
    // generic-proxy shared-memory writes -> visible to the tensor core
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t mb = smem_u32(mbar);

    if (tid == 0) {
        constexpr uint32_t idesc = umma_idesc(128, COUT);
        const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
        constexpr uint32_t a_lbo = kTcHX * 16, a_sbo = C8 * kTcHX * 16;   // K: next c8; M: next y row
        constexpr uint32_t b_lbo = COUT * 16, b_sbo = 128;                // K: next c8; N: next 8 outputs
        int first = 1;
        for (int t = 0; t < 27; ++t) {
            const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
#pragma unroll
            for (int kc = 0; kc < CIN / 16; ++kc) {
                const uint32_t aoff = ((((dz + 1) * kTcHY + (dy + 1)) * C8 + 2 * kc) * kTcHX + (dx + 1)) * 16;
                const uint32_t boff = ((t * C8 + 2 * kc) * COUT) * 16;
                const uint64_t da = umma_desc(a0 + aoff, a_lbo, a_sbo);
                const uint64_t db = umma_desc(b0 + boff, b_lbo, b_sbo);
                const uint32_t acc = first ? 0u : 1u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(idesc), "r"(acc));
                first = 0;
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb) : "memory");
    }
    // the wait is bounded (wait1 polls); the outcome is made uniform over the
    // block so the warp-collective TMEM reads below run in all warps or in
    // none.  On expiry the flag is raised (1) and the MMAs are waited for
    // again; the tile's output is written only when they ended.
    bool done = __syncthreads_and(mbar_wait(mb, 0, wait1));
    if (!done) {
        if (tid == 0) atomicMax(err, 1);
        done = __syncthreads_and(mbar_wait(mb, 0, kTcWaitLimit));
        // a second expiry (2): the tile is abandoned and its tensor memory
        // released below all the same, so that no later CTA on this SM waits
        // for it; the launch's output is invalid either way
        if (!done && tid == 0) atomicMax(err, 2);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (done) {
        // warp w owns TMEM lanes 32w..32w+31 = voxel rows; row i = 8*y + x of the tile
        const int i = 32 * warp + lane;
        const int x = x0 + (i % kTcX), y = y0 + i / kTcX, z = z0;
        const bool ok = x < gd.nx && y < gd.ny;
        const size_t o = ok ? (size_t)((z * gd.ny + y) * gd.nx + x) * out_cs + out_co : 0;
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
            uint32_t r[16];
            const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (ok) {
                float f[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    f[q] = __uint_as_float(r[q]) + (bias ? bias[c0 + q] : 0.f);
                    if (relu) f[q] = fmaxf(f[q], 0.f);
                }
                if (out_f) {
                    float4* d = reinterpret_cast<float4*>(out_f + o + c0);
#pragma unroll
                    for (int q = 0; q < 4; ++q) d[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
                } else {
                    uint32_t h[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        h[q] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(f[2 * q])) |
                               ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(f[2 * q + 1])) << 16);
                    uint4* d = reinterpret_cast<uint4*>(out + o + c0);
                    d[0] = make_uint4(h[0], h[1], h[2], h[3]);
                    d[1] = make_uint4(h[4], h[5], h[6], h[7]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(S::TCOLS));
}

// weights of one layer in the B operand order [t][c8][co][8], from the FP32 master W[t][co][ci]
__global__ void k_stage_tc(int cin, int cout, const float* __restrict__ wf, bf16* __restrict__ wtc) {
    const int n = 27 * cin * cout;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ci = i % cin, co = (i / cin) % cout, t = i / (cin * cout);
        wtc[(((size_t)t * (cin / 8) + ci / 8) * cout + co) * 8 + (ci % 8)] = __float2bfloat16_rn(wf[i]);
    }
}

template <int CIN, int COUT>
int conv_tc_attr() {
    return cudaFuncSetAttribute(k_conv_tc<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)TcShape<CIN, COUT>::SMEM) == cudaSuccess;
}
int prepare_tc() {
    return conv_tc_attr<16, 16>() && conv_tc_attr<16, 32>() && conv_tc_attr<32, 32>() && conv_tc_attr<48, 16>() ? GFM_OK
                                                                                                               : GFM_E_CUDA;
}
void stage_tc(int cin, int cout, const float* wf, bf16* wtc, cudaStream_t st) {
    const int n = 27 * cin * cout;
    k_stage_tc<<<(n + 255) / 256, 256, 0, st>>>(cin, cout, wf, wtc);
}
template <int CIN, int COUT>
void conv_tc(const Grid3& gd, const bf16* in, int in_cs, int in_co, const bf16* wtc, const float* bias, bf16* out,
             float* out_f, int out_cs, int out_co, bool relu, int* err, int wait1, cudaStream_t st) {
    const dim3 grid((unsigned)(((gd.nx + kTcX - 1) / kTcX) * ((gd.ny + kTcY - 1) / kTcY)), (unsigned)gd.nz);
    k_conv_tc<CIN, COUT><<<grid, kTcThreads, TcShape<CIN, COUT>::SMEM, st>>>(
        gd, in, in_cs, in_co, wtc, bias, out, out_f, out_cs, out_co, relu ? 1 : 0, err, wait1 >= 0 ? wait1 : kTcWaitLimit);
}
template void conv_tc<16, 16>(const Grid3&, const bf16*, int, int, const bf16*, const float*, bf16*, float*, int, int, bool,
                              int*, int, cudaStream_t);
template void conv_tc<16, 32>(const Grid3&, const bf16*, int, int, const bf16*, const float*, bf16*, float*, int, int, bool,
                              int*, int, cudaStream_t);
template void conv_tc<32, 32>(const Grid3&, const bf16*, int, int, const bf16*, const float*, bf16*, float*, int, int, bool,
                              int*, int, cudaStream_t);
template void conv_tc<48, 16>(const Grid3&, const bf16*, int, int, const bf16*, const float*, bf16*, float*, int, int, bool,
                              int*, int, cudaStream_t);

}  // namespace lp
}  // namespace gfm
