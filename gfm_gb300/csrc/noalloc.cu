// noalloc.cu -- gfm_adlbl3_noalloc: one ADLBL3 line solve (the reference's
// Gauss-Seidel plane march, Adlbl3.f90:10-221) on arrays the caller already
// holds on the device, with no device allocation of any kind.
//
// Who needs it: code that runs inside a host program which owns all device
// memory -- a plugin under another framework's caching allocator, a memory
// pool sized once at start-up, a process with a hard device-memory quota --
// cannot call cudaMalloc (or any allocating library routine) behind its
// host's back, and so cannot create a gfm_gpu handle, whose buffers are
// allocated at create time.  This entry point takes every input and output as
// a device pointer from the caller and keeps its own working storage in a
// fixed, statically sized device array that is part of the loaded library.
//
// Scratch: PT and XT2 of the y-lines and PT and XT3 of the z-lines of ONE
// x-plane at a time, kNaMaxPlanePoints points each (4 x 65536 doubles = 2 MiB
// per GPU, held until the process exits).  The CUDA runtime may load this
// file's module, and with it the array, only when the entry point is first
// called on a device (lazy module loading): a host that reserves the device's
// memory for its own pool at start-up should make one call first (nim = 0
// does no device work) so the array is in place before the pool takes the
// rest.  Planes with more points than the limit are rejected with
// GFM_E_LIMIT.  Every scratch element a call reads
// was written earlier in the same call, so nothing has to be cleared between
// calls.  All calls share the one array: calls whose kernels overlap on the GPU
// (concurrent streams, or several host threads) race on it and give wrong
// results; serialise them.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/gfm_gb300.h"

constexpr int kNaMaxPlanePoints = 65536;   // (J,K) points of one plane of the solved class
constexpr int kNaMaxDevices = 64;

// The working storage.  Host code must not pass `gfm_noalloc_scratch` itself to
// a kernel: on the host the name is only a stand-in for the device symbol.  Its
// device address is looked up with cudaGetSymbolAddress (na_scratch below).
static __device__ __align__(256) double gfm_noalloc_scratch[4 * kNaMaxPlanePoints];

namespace {

struct NaSys {
    double* xt;
    const double* ap;
    const double* as[6];
    const double* bs;
    const int16_t* ibc;
    int mp, np;
    int ib, ie, jb, je, kb, ke, nim;
};

// offset of (I,J,K), 1-based, in the reference's column-major A(MP,NP,LP)
__device__ __forceinline__ long long fidx(const NaSys& s, int I, int J, int K) {
    return (long long)(I - 1) + (long long)s.mp * ((long long)(J - 1) + (long long)s.np * (K - 1));
}

// One plane visit (ADLZ, Adlbl3.f90:103-141) by the whole CTA.  The y-line
// and z-line recurrences follow ADLZY/ADLYZ (Adlbl3.f90:147-221) term by term,
// with exact division, as the march mode of the handle-based solver does.
__device__ void na_plane(const NaSys& s, double* __restrict__ scr, int I) {
    const int nJ = (s.je - s.jb) / 2 + 1, nK = (s.ke - s.kb) / 2 + 1, npt = nJ * nK;
    double* pty = scr;
    double* xt2 = scr + npt;
    double* ptz = scr + 2 * npt;
    double* xt3 = scr + 3 * npt;
    double* xt = s.xt;
    for (int L = 1; L <= 2; ++L) {
        for (int t = threadIdx.x; t < nK + nJ; t += blockDim.x) {
            if (t < nK) {
                const int K = s.kb + 2 * t;
                double pt_prev = 0.0, qt_prev = xt[fidx(s, I, s.jb - 2, K)];
                for (int J = s.jb, jj = 0; J <= s.je; J += 2, ++jj) {
                    const long long o = fidx(s, I, J, K);
                    const int q = t * nJ + jj;
                    double alp = s.ap[o] - pt_prev * s.as[2][o];
                    double bsy = s.bs[o];
                    double pt, qt;
                    if (fabs(alp) <= 1.0e-20 || s.ibc[o] >= 1) {
                        pt = 0.0;
                        qt = xt[o];
                    } else {
                        bsy = bsy + s.as[1][o] * xt[fidx(s, I + 2, J, K)] + s.as[0][o] * xt[fidx(s, I - 2, J, K)];
                        bsy = bsy + s.as[5][o] * xt[fidx(s, I, J, K + 2)] + s.as[4][o] * xt[fidx(s, I, J, K - 2)];
                        pt = s.as[3][o] / alp;
                        qt = (bsy + s.as[2][o] * qt_prev) / alp;
                    }
                    pty[q] = pt;
                    xt2[q] = qt;
                    pt_prev = pt;
                    qt_prev = qt;
                }
                double nxt = xt[fidx(s, I, s.je + 2, K)];
                for (int jj = nJ - 1; jj >= 0; --jj) {
                    const int q = t * nJ + jj;
                    const double v = nxt * pty[q] + xt2[q];
                    xt2[q] = v;
                    nxt = v;
                }
            } else {
                const int jj = t - nK, J = s.jb + 2 * jj;
                double pt_prev = 0.0, qt_prev = xt[fidx(s, I, J, s.kb - 2)];
                for (int K = s.kb, kk = 0; K <= s.ke; K += 2, ++kk) {
                    const long long o = fidx(s, I, J, K);
                    const int q = kk * nJ + jj;
                    double alp = s.ap[o] - pt_prev * s.as[4][o];
                    double bsy = s.bs[o];
                    double pt, qt;
                    if (fabs(alp) <= 1.0e-20 || s.ibc[o] >= 1) {
                        pt = 0.0;
                        qt = xt[o];
                    } else {
                        bsy = bsy + s.as[1][o] * xt[fidx(s, I + 2, J, K)] + s.as[0][o] * xt[fidx(s, I - 2, J, K)];
                        bsy = bsy + s.as[3][o] * xt[fidx(s, I, J + 2, K)] + s.as[2][o] * xt[fidx(s, I, J - 2, K)];
                        pt = s.as[5][o] / alp;
                        qt = (bsy + s.as[4][o] * qt_prev) / alp;
                    }
                    ptz[q] = pt;
                    xt3[q] = qt;
                    pt_prev = pt;
                    qt_prev = qt;
                }
                double nxt = xt[fidx(s, I, J, s.ke + 2)];
                for (int kk = nK - 1; kk >= 0; --kk) {
                    const int q = kk * nJ + jj;
                    const double v = nxt * ptz[q] + xt3[q];
                    xt3[q] = v;
                    nxt = v;
                }
            }
        }
        __syncthreads();
        // a plane with a single z-row (KB >= KE) takes its first y-line pass
        // and nothing more (Adlbl3.f90:124-130); the z-lines solved above
        // are not used
        const bool one_row = s.kb >= s.ke;
        for (int t = threadIdx.x; t < npt; t += blockDim.x) {
            const int kk = t / nJ, jj = t % nJ;
            xt[fidx(s, I, s.jb + 2 * jj, s.kb + 2 * kk)] = one_row ? xt2[t] : (xt2[t] + xt3[t]) / 2.0;
        }
        __syncthreads();
        if (one_row) return;
    }
}

// The planes are visited in the reference's order, IB..IE then IE..IB, NIM
// times, so a single CTA walks them.
__global__ void k_adlbl3_noalloc(NaSys s, double* scr) {
    for (int ns = 0; ns < s.nim; ++ns) {
        for (int I = s.ib; I <= s.ie; I += 2) na_plane(s, scr, I);
        for (int I = s.ie; I >= s.ib; I -= 2) na_plane(s, scr, I);
    }
}

std::mutex g_na_mu;
double* g_na_ptr[kNaMaxDevices] = {};

// Device address of the scratch array in the current context.  It is looked
// up on every call: an address kept from an earlier call belongs to the
// context that was current then, and a reset of the device or another
// context made current on the same device would leave it pointing at memory
// that is no longer mapped.  While `stream` is capturing, no lookup is made
// (it may load the module); the address found by this device's last call
// outside a capture is used, and without one the call returns
// GFM_E_UNSUPPORTED.
int na_scratch(cudaStream_t stream, double** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return GFM_E_CUDA;
    if (dev < 0 || dev >= kNaMaxDevices) return GFM_E_UNSUPPORTED;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess) return GFM_E_CUDA;
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (cs != cudaStreamCaptureStatusNone) {
        if (!g_na_ptr[dev]) return GFM_E_UNSUPPORTED;
        *out = g_na_ptr[dev];
        return GFM_OK;
    }
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, gfm_noalloc_scratch) != cudaSuccess || !p) return GFM_E_CUDA;
    g_na_ptr[dev] = static_cast<double*>(p);
    *out = g_na_ptr[dev];
    return GFM_OK;
}

// device-resident (or managed) memory of the current device
bool on_device(const void* p, int dev) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace

extern "C" int gfm_adlbl3_noalloc(int mp, int np, int lp, const int16_t* ibcell, double* xt, const double* ap,
                                  const double* const as[6], const double* bs, int ib, int ie, int jb, int je, int kb,
                                  int ke, int nim, void* stream) {
    if (!ibcell || !xt || !ap || !as || !bs || nim < 0) return GFM_E_ARG;
    for (int q = 0; q < 6; ++q) if (!as[q]) return GFM_E_ARG;
    if (mp < 8 || np < 8 || lp < 8) return GFM_E_ARG;
    if (((ib ^ ie) & 1) || ((jb ^ je) & 1) || ((kb ^ ke) & 1) || ib < 3 || jb < 3 || kb < 3 || ie > mp - 2 ||
        je > np - 2 || ke > lp - 2 || ie < ib || je < jb || ke < kb)
        return GFM_E_ARG;
    const long long plane = (long long)((je - jb) / 2 + 1) * ((ke - kb) / 2 + 1);
    if (plane > kNaMaxPlanePoints) return GFM_E_LIMIT;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return GFM_E_CUDA;
    const void* ptrs[] = {ibcell, xt, ap, as[0], as[1], as[2], as[3], as[4], as[5], bs};
    for (const void* p : ptrs) if (!on_device(p, dev)) return GFM_E_ARG;
    double* scr = nullptr;
    int rc = na_scratch(static_cast<cudaStream_t>(stream), &scr);
    if (rc != GFM_OK) return rc;
    if (nim == 0) return GFM_OK;
    NaSys s;
    s.xt = xt; s.ap = ap; s.bs = bs; s.ibc = ibcell;
    for (int q = 0; q < 6; ++q) s.as[q] = as[q];
    s.mp = mp; s.np = np;
    s.ib = ib; s.ie = ie; s.jb = jb; s.je = je; s.kb = kb; s.ke = ke; s.nim = nim;
    k_adlbl3_noalloc<<<1, 256, 0, static_cast<cudaStream_t>(stream)>>>(s, scr);
    return cudaGetLastError() == cudaSuccess ? GFM_OK : GFM_E_CUDA;
}
