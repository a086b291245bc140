// lp.cuh -- the learned p' initial guess: network object shared by the
// training entry points (lp.cu) and the solver, which runs its forward pass
// inside the captured iteration.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

namespace gfm {
namespace lp {

struct LayerSpec {
    int cin, cout;
};
// voxel grid, x fastest: voxel (z*ny + y)*nx + x
struct Grid3 {
    int nx, ny, nz;
    __host__ __device__ __forceinline__ int nvox() const { return nx * ny * nz; }
};
constexpr int kNumLayers = 6;
constexpr int kFeatChannels = 2;   // Jacobi-scaled right-hand side, open-cell mask
extern const LayerSpec kLayers[kNumLayers];
int weight_offset(int layer);      // into the flat FP32 parameter vector: W[27][cout][cin] then b[cout]
int num_params();

// Network with buffers for grids of up to mx*my*mz voxels (even extents).
struct Net {
    int mx = 0, my = 0, mz = 0, np = 0, steps = 0;
    float *p32 = nullptr, *g32 = nullptr, *m32 = nullptr, *v32 = nullptr;   // parameters, gradients, Adam moments
    __nv_bfloat16* w16[kNumLayers] = {};    // BF16 weights W[t][cout][cin]
    __nv_bfloat16* wt16[kNumLayers] = {};   // mirrored transposes for the input gradient
    __nv_bfloat16 *A1 = nullptr, *CAT = nullptr, *P0 = nullptr, *A2 = nullptr, *E1 = nullptr, *A3 = nullptr;
    float* OUT = nullptr;                    // 16 channels, FP32; channel 0 is the prediction
    __nv_bfloat16 *dOUT = nullptr, *dA3 = nullptr, *dCAT = nullptr, *dE1 = nullptr, *dA2 = nullptr, *dP0 = nullptr,
                  *dE0 = nullptr, *dA1 = nullptr;
    float* nopen = nullptr;
    double* lacc = nullptr;                  // squared error, open-voxel count of the last step
    // forward convolutions on tcgen05 (lp_tc.cu): weights in the operand order, expiry flag
    __nv_bfloat16* wtc[kNumLayers] = {};
    int* tc_err = nullptr;
    int tc_wait1 = -1;                       // polls of the first bounded MMA wait (<0: the default limit);
                                             // GFM_LP_WAIT1 at create, for tests of the expiry path
    float* wg_part = nullptr;                // per-chunk weight-gradient partials (fixed-order sums)
    bool use_tc = true;
    std::string err;

    int create(int nx, int ny, int nz, uint64_t seed);
    void release();
    void stage(cudaStream_t st);             // BF16 copies of the FP32 parameters
    int check_dims(int nx, int ny, int nz) const;
    void forward(const __nv_bfloat16* feats, int nx, int ny, int nz, cudaStream_t st);
    void backward(const __nv_bfloat16* feats, const float* target, int nx, int ny, int nz, cudaStream_t st);
    void adam(float lr, int step, cudaStream_t st);
};

// tcgen05 forward convolution (lp_tc.cu)
int prepare_tc();
void stage_tc(int cin, int cout, const float* wf, __nv_bfloat16* wtc, cudaStream_t st);
template <int CIN, int COUT>
void conv_tc(const Grid3& gd, const __nv_bfloat16* in, int in_cs, int in_co, const __nv_bfloat16* wtc, const float* bias,
             __nv_bfloat16* out, float* out_f, int out_cs, int out_co, bool relu, int* err, int wait1,
             cudaStream_t st);

}  // namespace lp
}  // namespace gfm
