// wall.cu -- the wall radiosity exchange on the device: the part of QRNF
// after the volume transfer (wall_q_amb and wallq, Qwall.f90:990-1245,
// 1585-1655; get_radiation_from_boundaries, Qwall.f90:1489-1577).
//
// The boundary patches exchange radiation through normalised view factors
// VF(n,m) (prepare_for_wall_radiation_calculation step 7, Qwall.f90:562-666),
// a dense nb x nb matrix formed once per handle and kept in HBM (FP64 on the
// FP64 path, FP32 on the mixed one: 22 GB for the 73,728 patches of the
// 192x96x64 furnace).  A radiosity sweep is then one pass over that matrix:
// one warp per row forms the radiation incident on its patch,
// rad(i) = sum_j VF(i,j) J(j), and the patch's new radiosity.  The reference
// sweeps Gauss-Seidel in patch order, which is a chain of nb dependent row
// updates; here every row of a sweep reads the previous sweep's radiosities
// (Jacobi).  Both iterate the same map to the same fixed point, with the
// reference's stopping rules (mean relative change below 1e-10, then three
// more sweeps; the outer loop on the melt flux).  Sums over patches are
// formed per block in a fixed order and added on the host in block order.
#include "state.cuh"

namespace gfm {

namespace {

// per-patch kernels: a fixed grid, partial sums per block
__device__ __forceinline__ void wall_partial(double v, double* sh, double* part, int slot) {
    const double s = block_sum(v, sh);
    if (threadIdx.x == 0) part[slot * kWallBlocks + blockIdx.x] = s;
}

// ---- view factors (Qwall.f90:562-666): one CTA per near patch n ----------------
template <typename V>
__global__ void __launch_bounds__(256) k_wall_vf(WallArgs a, V* vf) {
    __shared__ double sh[32];
    __shared__ double s_sum;
    const double pi = 3.141592653589793;
    const int nb = a.nb;
    for (int n = blockIdx.x; n < nb; n += gridDim.x) {
        const int on = a.ori[n], cn = on == 1 ? a.bi[n] : on == 2 ? a.bj[n] : a.bk[n];
        const bool plus = a.dir[n] == 0;
        const double xn = a.px[n], yn = a.py[n], zn = a.pz[n];
        // the unnormalised factor of far patch m, 0 where the reference skips it
        auto vfac = [&](int m) -> double {
            if (m == n) return 0.0;
            const int cm = on == 1 ? a.bi[m] : on == 2 ? a.bj[m] : a.bk[m];
            if (plus ? cm <= cn : cm >= cn) return 0.0;
            const double dx = xn - a.px[m], dy = yn - a.py[m], dz = zn - a.pz[m];
            const double dd = dx * dx + dy * dy + dz * dz;
            const double denominator = pi * (dd * dd);
            const int om = a.ori[m];
            const double dn = on == 1 ? a.px[m] - xn : on == 2 ? a.py[m] - yn : a.pz[m] - zn;
            if (om == on) return dn * dn * a.area[m] / denominator;
            const double dm = om == 1 ? a.px[m] - xn : om == 2 ? a.py[m] - yn : a.pz[m] - zn;
            return fabs(dn * dm) * a.area[m] / denominator;
        };
        double part = 0.0;
        for (int m = threadIdx.x; m < nb; m += blockDim.x) part += vfac(m);
        const double sum = block_sum(part, sh);
        if (threadIdx.x == 0) {
            s_sum = sum;
            a.vfsum[n] = sum;
        }
        __syncthreads();
        const double vs = s_sum;
        V* row = vf + (size_t)n * nb;
        for (int m = threadIdx.x; m < nb; m += blockDim.x) {
            const double v = vfac(m);
            row[m] = V(vs == 0.0 ? v : v / vs);
        }
        __syncthreads();
    }
}

// ---- RAD_EMIS's patch temperatures (Rad_emis.f90:186-273), T in K = T*T0 -------
template <typename R>
__global__ void k_wall_start(WallArgs a, const R* __restrict__ T, int first) {
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < a.nb; n += gridDim.x * blockDim.x) {
        const int t = a.typ[n];
        double bt;
        if (t == 4) bt = (double)T[a.o_b[n]] * a.t0;
        else if (!first) continue;
        else if (t == 3) bt = a.bT_exit[n];
        else bt = (double)T[a.o_bc[n]] * a.t0;
        a.bT[n] = bt;
        const double b2 = bt * bt;
        a.J[n] = a.sig * (b2 * b2);
    }
}

// ---- wallq's set-up (Qwall.f90:997-1025): qc, qeb, the melt cells' QE -----------
template <typename R>
__global__ void __launch_bounds__(256) k_wall_init(WallArgs a, const R* __restrict__ QA, R* __restrict__ QE) {
    __shared__ double sh[32];
    double inc[5] = {0, 0, 0, 0, 0};
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < a.nb; n += gridDim.x * blockDim.x) {
        const double qcn = (double)QA[a.o_bc[n]] / a.face_area[n];
        a.qc[n] = qcn;
        const double qa = qcn * a.area[n];
        inc[0] += qa;
        const int t = a.typ[n];
        const double b2 = a.bT[n] * a.bT[n], sb4 = a.sig * (b2 * b2);
        if (t == 1) inc[1] += qa;
        else if (t == 2) { inc[2] += qa; a.qeb[n] = sb4; }
        else if (t == 3) { inc[3] += qa; a.qeb[n] = sb4; }
        else if (t == 4) {
            inc[4] += qa;
            const double q = a.emis[n] * a.sig * (b2 * b2);
            a.qeb[n] = q;
            QE[a.o_bc[n]] = R(q);   // the reference keeps it for its print-out (Qwall.f90:1021)
        }
    }
    for (int s = 0; s < 5; ++s) wall_partial(inc[s], sh, a.part, W_INC_TOTAL + s);
}

// ---- wall sink <-> exchange: patch temperatures out, convective fluxes in -------
__global__ void k_wall_to_sink(WallArgs a, Patch* __restrict__ sink_patches) {
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < a.nb; n += gridDim.x * blockDim.x)
        if (a.sink[n] >= 0) sink_patches[a.sink[n]].bT = a.bT[n];
}
template <typename R>
__global__ void __launch_bounds__(256) k_wall_from_sink(WallArgs a, const R* __restrict__ qconv_sink) {
    __shared__ double sh[32];
    double tot = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < a.nb; n += gridDim.x * blockDim.x) {
        const double q = a.sink[n] >= 0 ? (double)qconv_sink[a.sink[n]] : 0.0;   // inlets, exits: 0
        a.qconv[n] = q;
        tot += q * a.area[n];
    }
    wall_partial(tot, sh, a.part, W_QCONV);
}

// the radiation a patch receives from the others: one warp per row of VF
__device__ __forceinline__ double vf_row_dot(const float* __restrict__ row, const double* __restrict__ J, int nb,
                                             int lane) {
    // FP32 factors: products of one group of four in FP32, groups added in FP64
    double acc = 0.0;
    int m = 4 * lane;
    const bool al = ((reinterpret_cast<size_t>(row) & 15) == 0);
    if (al) {
        for (; m + 3 < nb; m += 128) {
            const float4 v = __ldg(reinterpret_cast<const float4*>(row + m));
            acc += (double)v.x * J[m] + (double)v.y * J[m + 1] + (double)v.z * J[m + 2] + (double)v.w * J[m + 3];
        }
        for (int q = m; q < nb && q < m + 4; ++q) acc += (double)row[q] * J[q];
    } else {
        for (m = lane; m < nb; m += 32) acc += (double)row[m] * J[m];
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}
__device__ __forceinline__ double vf_row_dot(const double* __restrict__ row, const double* __restrict__ J, int nb,
                                             int lane) {
    double acc = 0.0;
    for (int m = lane; m < nb; m += 32) acc += __ldg(row + m) * J[m];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

// ---- one radiosity sweep (Qwall.f90:1056-1083), every row from the previous J ---
template <typename V>
__global__ void __launch_bounds__(256) k_wall_sweep(WallArgs a, const V* __restrict__ vf) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = warp; i < a.nb; i += nw) {
        const int t = a.typ[i];
        const double e = a.emis[i];
        double rad = 0.0;
        if (t == 1 || e < 1.0) rad = vf_row_dot(vf + (size_t)i * a.nb, a.J, a.nb, lane);
        if (lane == 0) {
            const double old = a.J[i];
            double jn;
            if (t == 1) {
                jn = a.qc[i] + a.qconv[i] - a.qamb[i] + rad;
                const double lo = e * a.radi_min;
                jn = jn > lo ? jn : lo;   // MAX(x, emis*radi_min)
            } else {
                jn = a.qeb[i] + (1.0 - e) * (rad + a.qc[i]);
            }
            a.Jn[i] = jn;
            a.rel[i] = old < 1.0e-10 ? 0.0 : fabs((old - jn) / old);
        }
    }
}

// sum of the relative changes, in block order
__global__ void __launch_bounds__(256) k_wall_rel_sum(WallArgs a) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < a.nb; n += gridDim.x * blockDim.x) s += a.rel[n];
    wall_partial(s, sh, a.part, W_REL);
}

// rad for the rows of the types in `mask` (bit t), from the current J
template <typename V>
__global__ void __launch_bounds__(256) k_wall_rad(WallArgs a, const V* __restrict__ vf, int mask) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = warp; i < a.nb; i += nw) {
        if (!((mask >> a.typ[i]) & 1)) continue;
        const double rad = vf_row_dot(vf + (size_t)i * a.nb, a.J, a.nb, lane);
        if (lane == 0) a.rad[i] = rad;
    }
}

// ---- wall temperatures and the melt flux (Qwall.f90:1134-1184) -----------------
__global__ void __launch_bounds__(256) k_wall_temps(WallArgs a) {
    __shared__ double sh[32];
    double qm = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nb; i += gridDim.x * blockDim.x) {
        const int t = a.typ[i];
        if (t == 1) {
            const double e = a.emis[i];
            double v = (a.J[i] - (a.qamb[i] - a.qconv[i]) * (1.0 - e) / e) / a.sig;
            v = 0.0 > v ? 0.0 : v;   // MAX(zero, ...)
            double bt = pow(v, 0.25);
            bt = a.t_mnk > bt ? a.t_mnk : bt;
            a.bT[i] = bt;
        } else if (t == 4) {
            qm += (a.qc[i] + a.qconv[i] + a.rad[i] - a.J[i]) * a.area[i];
        }
    }
    wall_partial(qm, sh, a.part, W_Q_MELT);
}

// ---- wall_q_amb (Qwall.f90:1585-1655), one wall material --------------------------
__global__ void __launch_bounds__(256) k_wall_qamb(WallArgs a) {
    __shared__ double sh[32];
    double loss = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < a.nb; n += gridDim.x * blockDim.x) {
        if (a.typ[n] != 1) { a.qamb[n] = 0.0; continue; }
        const double q = a.u_a0 * (a.bT[n] - a.t_a);
        a.qamb[n] = q;
        loss += q * a.area[n];
    }
    wall_partial(loss, sh, a.part, W_Q_LOSS);
}

// ---- after the loops (Qwall.f90:1192-1231): wall T into the field, the
// inlet, outlet and melt totals.  T is normalised here: the reference writes
// b_T into T (in K) and divides the whole array by T0 at the end of RAD_EMIS.
template <typename R>
__global__ void __launch_bounds__(256) k_wall_post(WallArgs a, R* __restrict__ T) {
    __shared__ double sh[32];
    double s[5] = {0, 0, 0, 0, 0};   // T area, q_rad_inlet, q_rad_outlet, qm_flame, qm_bnds
    double qmc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nb; i += gridDim.x * blockDim.x) {
        const int t = a.typ[i];
        if (t == 1) {
            T[a.o_b[i]] = R(a.bT[i] / a.t0);
            s[0] += a.bT[i] * a.area[i];
        } else if (t == 2) {
            s[1] += (a.qc[i] + a.rad[i] - a.qeb[i]) * a.area[i];
        } else if (t == 3) {
            s[2] += (a.qc[i] + a.rad[i] - a.qeb[i]) * a.area[i];
        } else if (t == 4) {
            const double e = a.emis[i];
            const double f_melt = 1.0 - a.qeb[i] / (e * (a.qc[i] + a.rad[i]) + a.qconv[i]);
            s[3] += f_melt * e * a.qc[i] * a.area[i];
            s[4] += f_melt * e * a.rad[i] * a.area[i];
            qmc += f_melt * a.qconv[i] * a.area[i];
        }
    }
    wall_partial(s[0], sh, a.part, W_T_AREA);
    wall_partial(s[1], sh, a.part, W_Q_RAD_IN);
    wall_partial(s[2], sh, a.part, W_Q_RAD_OUT);
    wall_partial(s[3], sh, a.part, W_QM_FLAME);
    wall_partial(s[4], sh, a.part, W_QM_BNDS);
    wall_partial(qmc, sh, a.part, W_QM_CONV);
}

// exits at a fraction of the mean wall temperature (Qwall.f90:1235-1244)
__global__ void k_wall_exits(WallArgs a, const int* __restrict__ frac_exit, const double* __restrict__ frac,
                             double avg_wall_T) {
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < a.nb; n += gridDim.x * blockDim.x)
        if (a.typ[n] == 3 && frac_exit[n]) a.bT[n] = frac[n] * avg_wall_T;
}

int rows_grid(int nb) {
    int b = (nb + 7) / 8;   // 8 warps a block, one row each
    return b < 1 ? 1 : (b > 4096 ? 4096 : b);
}

}  // namespace

int launch_wall_vf(const WallArgs& a, cudaStream_t st) {
    const int grid = a.nb < 65535 ? a.nb : 65535;
    if (a.vf64) k_wall_vf<double><<<grid, 256, 0, st>>>(a, a.vf64);
    else k_wall_vf<float><<<grid, 256, 0, st>>>(a, a.vf32);
    return cudaGetLastError() == cudaSuccess ? GFM_OK : GFM_E_CUDA;
}
template <typename R>
void launch_wall_start(const WallArgs& a, const R* T, int first, cudaStream_t st) {
    k_wall_start<R><<<kWallBlocks, 256, 0, st>>>(a, T, first);
}
template <typename R>
void launch_wall_init(const WallArgs& a, const R* QA, R* QE, cudaStream_t st) {
    k_wall_init<R><<<kWallBlocks, 256, 0, st>>>(a, QA, QE);
}
void launch_wall_to_sink(const WallArgs& a, Patch* sink_patches, cudaStream_t st) {
    k_wall_to_sink<<<kWallBlocks, 256, 0, st>>>(a, sink_patches);
}
template <typename R>
void launch_wall_from_sink(const WallArgs& a, const R* qconv_sink, cudaStream_t st) {
    k_wall_from_sink<R><<<kWallBlocks, 256, 0, st>>>(a, qconv_sink);
}
void launch_wall_sweep(const WallArgs& a, cudaStream_t st) {
    if (a.vf64) k_wall_sweep<double><<<rows_grid(a.nb), 256, 0, st>>>(a, a.vf64);
    else k_wall_sweep<float><<<rows_grid(a.nb), 256, 0, st>>>(a, a.vf32);
    k_wall_rel_sum<<<kWallBlocks, 256, 0, st>>>(a);
}
void launch_wall_rad(const WallArgs& a, int mask, cudaStream_t st) {
    if (a.vf64) k_wall_rad<double><<<rows_grid(a.nb), 256, 0, st>>>(a, a.vf64, mask);
    else k_wall_rad<float><<<rows_grid(a.nb), 256, 0, st>>>(a, a.vf32, mask);
}
void launch_wall_temps(const WallArgs& a, cudaStream_t st) { k_wall_temps<<<kWallBlocks, 256, 0, st>>>(a); }
void launch_wall_qamb(const WallArgs& a, cudaStream_t st) { k_wall_qamb<<<kWallBlocks, 256, 0, st>>>(a); }
template <typename R>
void launch_wall_post(const WallArgs& a, R* T, cudaStream_t st) {
    k_wall_post<R><<<kWallBlocks, 256, 0, st>>>(a, T);
}
void launch_wall_exits(const WallArgs& a, const int* frac_exit, const double* frac, double avg_wall_T, cudaStream_t st) {
    k_wall_exits<<<kWallBlocks, 256, 0, st>>>(a, frac_exit, frac, avg_wall_T);
}

#define INST(R)                                                                                    \
    template void launch_wall_start<R>(const WallArgs&, const R*, int, cudaStream_t);             \
    template void launch_wall_init<R>(const WallArgs&, const R*, R*, cudaStream_t);               \
    template void launch_wall_from_sink<R>(const WallArgs&, const R*, cudaStream_t);              \
    template void launch_wall_post<R>(const WallArgs&, R*, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace gfm
