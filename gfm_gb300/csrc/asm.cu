// asm.cu -- coefficient assembly, sources and per-cell property kernels.
//
// Every kernel restates one loop of the reference on one parity class; the
// per-position arithmetic keeps the Fortran expression order.  Citations name
// the reference routine each kernel follows.
#include "state.cuh"

namespace gfm {

#define A(arr, I, J, K) (arr)[pidx(g, (I), (J), (K))]

constexpr int kBlock = 256;

__host__ __device__ inline int cdiv(long long a, int b) { return (int)((a + b - 1) / b); }

// iteration space of one class: I in [i0,i1], J in [j0,j1], K in [k0,k1], step 2
struct Range {
    int i0, i1, j0, j1, k0, k1;
    __host__ __device__ long long count() const {
        long long ni = (i1 - i0) / 2 + 1, nj = (j1 - j0) / 2 + 1, nk = (k1 - k0) / 2 + 1;
        return (i1 < i0 || j1 < j0 || k1 < k0) ? 0 : ni * nj * nk;
    }
    __device__ void at(int t, int& I, int& J, int& K) const {
        const int ni = (i1 - i0) / 2 + 1, nj = (j1 - j0) / 2 + 1;
        I = i0 + 2 * (t % ni);
        const int r = t / ni;
        J = j0 + 2 * (r % nj);
        K = k0 + 2 * (r / nj);
    }
};

template <typename R> __device__ __forceinline__ R rmax(R a, R b) { return a > b ? a : b; }   // Fortran MAX(a,b)
template <typename R> __device__ __forceinline__ R rmin(R a, R b) { return a < b ? a : b; }

// ---------------------------------------------------------------------------
// Metric functions (Grid3.f90:310-392; VOL_C0 and AREA_C in device.cuh)
// ---------------------------------------------------------------------------

template <typename R>
__device__ R vol_c(const GeoT<R>& g, int I, int J, int K) {
    if (I & 1) {
        R vm = vol_c0(g, I - 1, J, K); if (IBC(g, I - 2, J, K) <= 0) vm = vm * R(0.5);
        R vp = vol_c0(g, I + 1, J, K); if (IBC(g, I + 2, J, K) <= 0) vp = vp * R(0.5);
        return vp + vm;
    } else if (J & 1) {
        R vm = vol_c0(g, I, J - 1, K); if (IBC(g, I, J - 2, K) <= 0) vm = vm * R(0.5);
        R vp = vol_c0(g, I, J + 1, K); if (IBC(g, I, J + 2, K) <= 0) vp = vp * R(0.5);
        return vp + vm;
    } else if (K & 1) {
        R vm = vol_c0(g, I, J, K - 1); if (IBC(g, I, J, K - 2) <= 0) vm = vm * R(0.5);
        R vp = vol_c0(g, I, J, K + 1); if (IBC(g, I, J, K + 2) <= 0) vp = vp * R(0.5);
        return vp + vm;
    }
    return vol_c0(g, I, J, K);
}
template <typename R>
__device__ R dxav(const GeoT<R>& g, int I, int J, int K) {
    if (IBC(g, I - 2, J, K) >= 1) return g.X[I + 1] - g.X[I - 2];
    if (IBC(g, I + 2, J, K) >= 1) return g.X[I + 2] - g.X[I - 1];
    return g.DX[I];
}
template <typename R>
__device__ R drav(const GeoT<R>& g, int I, int J, int K) {
    if (IBC(g, I, J - 2, K) >= 1) { R d = g.Rr[J + 1] - g.Rr[J - 2]; return (g.RS[J + 1] + g.RS[J - 2]) * R(0.5) / g.RS[J] * d; }
    if (IBC(g, I, J + 2, K) >= 1) { R d = g.Rr[J + 2] - g.Rr[J - 1]; return (g.RS[J + 2] + g.RS[J - 1]) * R(0.5) / g.RS[J] * d; }
    return g.DR[J];
}
template <typename R>
__device__ R dzav(const GeoT<R>& g, int I, int J, int K) {
    if (IBC(g, I, J, K - 2) >= 1) return g.Z[K + 1] - g.Z[K - 2];
    if (IBC(g, I, J, K + 2) >= 1) return g.Z[K + 2] - g.Z[K - 1];
    return g.DZ[K];
}
// FDDL (Gslv3x.f90:208-260)
template <typename R>
__device__ R fddl(const GeoT<R>& g, int I, int J, int K, int iu) {
    int b = IBC(g, I, J, K);
    const R big = R(1.0e20);
    if (iu == 1) {
        if (b <= 0) return g.DX[I];
        if (IBC(g, I + 1, J, K) == 0) return g.X[I + 1] - g.X[I];
        if (IBC(g, I - 1, J, K) == 0) return g.X[I] - g.X[I - 1];
        return big;
    } else if (iu == 2) {
        if (b <= 0) return g.DR[J] * g.RS[J];
        if (IBC(g, I, J + 1, K) == 0) return (g.Rr[J + 1] - g.Rr[J]) * g.RS[J];
        if (IBC(g, I, J - 1, K) == 0) return (g.Rr[J] - g.Rr[J - 1]) * g.RS[J];
        return big;
    }
    if (b <= 0) return g.DZ[K];
    if (IBC(g, I, J, K + 1) == 0) return g.Z[K + 1] - g.Z[K];
    if (IBC(g, I, J, K - 1) == 0) return g.Z[K] - g.Z[K - 1];
    return big;
}

// FLW / FLWD (Gslv3x.f90:292-329)
template <typename R>
__device__ R flw(const Ctx<R>& c, int I, int J, int K, int ix, int m) {
    const GeoT<R>& g = c.g;
    R area = area_c(g, I, J, K, ix);
    R f = A(c.THETA, I, J, K) * A(c.DNST, I, J, K) * A(c.UG[ix - 1], I, J, K) * area;
    return m == 1 ? rmax(R(0), f) : rmax(R(0), -f);
}
template <typename R>
__device__ R flwd(const Ctx<R>& c, int I, int J, int K, int ix, int m, R sgm) {
    const GeoT<R>& g = c.g;
    R area = area_c(g, I, J, K, ix);
    R ddl = ix == 1 ? g.DX[I] : (ix == 2 ? g.DR[J] : g.DZ[K]);
    R f = A(c.THETA, I, J, K) * A(c.DNST, I, J, K) * A(c.UG[ix - 1], I, J, K) * area;
    R diff = A(c.THETA, I, J, K) * A(c.GAMA, I, J, K) / sgm * area / ddl;
    return m == 1 ? da<R>(diff, f) + rmax(R(0), f) : da<R>(diff, f) + rmax(R(0), -f);
}

// ---------------------------------------------------------------------------
// Wall functions and THETA extrapolation (Gflow.f90:16-130).
// The reference scatters from every non-wall position into its wall
// neighbours; here each wall position gathers from its non-wall neighbours:
// GAMA takes the maximum of the contributions (order free), THETA the value of
// the last writer in the Fortran loop order (I outer, J, K inner; per position
// -x,+x,-y,+y,-z,+z), i.e. the first non-wall neighbour among +x,+y,+z,-z,-y,-x.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_wallfn(Ctx<R> c, const int* __restrict__ wl, int n) {
    const GeoT<R>& g = c.g;
    const R rt20 = R(c.p.rt20);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int I = wl[3 * t], J = wl[3 * t + 1], K = wl[3 * t + 2];
        // neighbour n = w + s*e_d writes w with distance d(n,w); order of last writer
        const int dirs[6][4] = {{1, 0, 0, +1}, {0, 1, 0, +1}, {0, 0, 1, +1}, {0, 0, 1, -1}, {0, 1, 0, -1}, {1, 0, 0, -1}};
        bool theta_done = false;
        R gmax = R(0);
        bool any = false;
        for (int q = 0; q < 6; ++q) {
            int s = dirs[q][3];
            int In = I + s * dirs[q][0], Jn = J + s * dirs[q][1], Kn = K + s * dirs[q][2];
            if (In < 2 || In > g.MP || Jn < 2 || Jn > g.NP || Kn < 2 || Kn > g.LP) continue;
            if (IBC(g, In, Jn, Kn) >= 1) continue;
            any = true;
            // the far point n+2s*e on the side away from the wall
            int Ifar = In + 2 * s * dirs[q][0], Jfar = Jn + 2 * s * dirs[q][1], Kfar = Kn + 2 * s * dirs[q][2];
            R dist, g1, g2;
            if (dirs[q][0]) {
                g1 = (g.X[In] - g.X[I]) * (g.X[In] - g.X[I]);
                g2 = (g.X[Ifar] - g.X[I]) * (g.X[Ifar] - g.X[I]);
                dist = s > 0 ? g.X[In] - g.X[I] : g.X[I] - g.X[In];
            } else if (dirs[q][1]) {
                g1 = (g.Rr[Jn] - g.Rr[J]) * (g.Rr[Jn] - g.Rr[J]);
                g2 = (g.Rr[Jfar] - g.Rr[J]) * (g.Rr[Jfar] - g.Rr[J]);
                dist = s > 0 ? g.Rr[Jn] - g.Rr[J] : g.Rr[J] - g.Rr[Jn];
            } else {
                g1 = (g.Z[Kn] - g.Z[K]) * (g.Z[Kn] - g.Z[K]);
                g2 = (g.Z[Kfar] - g.Z[K]) * (g.Z[Kfar] - g.Z[K]);
                dist = s > 0 ? g.Z[Kn] - g.Z[K] : g.Z[K] - g.Z[Kn];
            }
            if (!theta_done) {
                R x01 = g2 / (g2 - g1), x02 = g1 / (g1 - g2);
                A(c.THETA, I, J, K) = A(c.THETA, In, Jn, Kn) * x01 + A(c.THETA, Ifar, Jfar, Kfar) * x02;
                theta_done = true;
            }
            R cc = r_pow(A(c.T, In, Jn, Kn) / R(c.p.trdg), R(c.p.amu));
            R blvm = rt20 * A(c.DNST, In, Jn, Kn) * r_sqrt(A(c.GF[kK], In, Jn, Kn)) / cc;
            R vgam = cc / R(c.p.reyg2);
            R blv = blvm * dist;
            R gama0 = vgam * tgamf<R>(blv);
            gmax = rmax(gama0, gmax);
        }
        A(c.GAMA, I, J, K) = gmax;
        if (any) A(c.TMU, I, J, K) = R(c.p.reyg2) * gmax;
    }
}

// FZ <- UG on the three face classes (Gslv3v.f90:26-34)
template <typename R>
__global__ void k_copy_faces(Ctx<R> c) {
    const GeoT<R>& g = c.g;
    const int n = (int)g.CB;
    GFM_FOR(t, 3 * n) {
        const int iu = t / n;
        const int off = (1 << iu) * n + (t - iu * n);   // class 1 (x), 2 (y), 4 (z)
        c.FZ[off] = c.UG[iu][off];
    }
}

// ---------------------------------------------------------------------------
// Momentum: SRC1 (Source.f90:664-809) + GSLVX1/GSLV3X1/ECELL/VOL1
// (Gslv3x.f90:9-200) on the face class of direction IU1.
// ---------------------------------------------------------------------------
// 4 blocks of 256 per SM: the 64-register cap the compiler applies without
// launch bounds (it assumes 1024-thread blocks; free, it takes 101).  5 and 6
// (48 and 40 registers, small spills) measured within 0.2 % of it.
#ifndef GFM_MOM_MINB
#define GFM_MOM_MINB 4
#endif
template <typename R, int IU1>
__global__ void __launch_bounds__(kBlock, GFM_MOM_MINB) k_mom_assemble(Ctx<R> c, Range rg) {
    const GeoT<R>& g = c.g;
    const R zero = R(0);
    long long n = rg.count();
    GFM_FOR(t, n) {
        int I, J, K;
        rg.at(t, I, J, K);
        const long long o = pidx(g, I, J, K);
        if (g.ib[o] >= 1) {
            // reset values of GSLV3V (AP=1, AS=0) and SRC1 (BS=SFP=0)
            c.APm[o] = R(1);
            for (int q = 0; q < 6; ++q) c.ASm[q][o] = zero;
            c.BSm[o] = zero;
            c.SFPm[o] = zero;
            continue;
        }
        int NX[4] = {0, 0, 0, 0};
        NX[IU1] = 1;
        // ---- SRC1 -----------------------------------------------------------
        R bs, sfp;
        {
            R VIS[4][3], DXN[4], DX1[4], DX0[4];
            DXN[1] = g.DX[I]; DXN[2] = g.DR[J] * g.RS[J]; DXN[3] = g.DZ[K];
            for (int M = -1; M <= 1; M += 2) {
                int I1 = I + NX[1] * M, J1 = J + NX[2] * M, K1 = K + NX[3] * M;
                int I2 = I1 + NX[1] * M, J2 = J1 + NX[2] * M, K2 = K1 + NX[3] * M;
                if (IU1 == 1) { DX0[1] = g.DX[I]; DX1[1] = g.DX[I1]; }
                else if (IU1 == 2) { DX0[2] = g.DR[J] * g.RS[J]; DX1[2] = g.DR[J1] * g.RS[J1]; }
                else { DX0[3] = g.DZ[K]; DX1[3] = g.DZ[K1]; }
                R thgm;
                if (IBC(g, I2, J2, K2) == 2) {
                    thgm = A(c.THETA, I2, J2, K2) * A(c.GAMA, I2, J2, K2);
                    if (IU1 == 1) DXN[1] = DXN[1] + fabs(g.X[I2] - g.X[I1]);
                    if (IU1 == 2) DXN[2] = DXN[2] + fabs(g.Rr[J2] - g.Rr[J1]) * g.RS[J];
                    if (IU1 == 3) DXN[3] = DXN[3] + fabs(g.Z[K2] - g.Z[K1]);
                } else {
                    thgm = A(c.THETA, I1, J1, K1) * A(c.GAMA, I1, J1, K1);
                }
                if (M == -1) VIS[IU1][1] = thgm * (A(c.FZ, I, J, K) - A(c.FZ, I2, J2, K2)) / DX1[IU1];
                else VIS[IU1][2] = thgm * (A(c.FZ, I2, J2, K2) - A(c.FZ, I, J, K)) / DX1[IU1];
            }
            R vms = (VIS[IU1][2] - VIS[IU1][1]) / DXN[IU1];
            for (int IU = 1; IU <= 3; ++IU) {
                if (IU == IU1) continue;
                int I1 = I, J1 = J, K1 = K;
                for (int M = -1; M <= 1; M += 2) {
                    if (IU == 1) I1 = I + M; else if (IU == 2) J1 = J + M; else K1 = K + M;
                    R du0;
                    if (IU1 == 1) du0 = A(c.FZ, I + 1, J1, K1) - A(c.FZ, I - 1, J1, K1);
                    else if (IU1 == 2) du0 = A(c.FZ, I1, J + 1, K1) - A(c.FZ, I1, J - 1, K1);
                    else du0 = A(c.FZ, I1, J1, K + 1) - A(c.FZ, I1, J1, K - 1);
                    int M1 = (M + 3) / 2;
                    VIS[IU][M1] = A(c.THETA, I1, J1, K1) * A(c.GAMA, I1, J1, K1) * du0 / DX0[IU1];
                    if (IU == 2) VIS[IU][M1] = VIS[IU][M1] * g.RS[J1];
                }
                vms = vms + (VIS[IU][2] - VIS[IU][1]) / DXN[IU];
            }
            bs = vms + zero + zero;
            bs = bs + A(c.THETA, I, J, K) * A(c.DNST, I, J, K) * R(c.p.gra[IU1 - 1]);
            sfp = -zero;
        }
        // ---- GSLV3X1: own-direction coefficients --------------------------------
        const R sgm = R(1);
        R ap = zero, g0 = zero, as[6];
        for (int M = -1; M <= 1; M += 2) {
            int M1 = (M + 3) / 2;
            int I1 = I + NX[1] * M, J1 = J + NX[2] * M, K1 = K + NX[3] * M;
            int I2 = I1 + NX[1] * M, J2 = J1 + NX[2] * M, K2 = K1 + NX[3] * M;
            int ibc1 = IBC(g, I2, J2, K2);
            R a;
            if (ibc1 == 3) a = zero;
            else if (ibc1 == 2) a = flw(c, I2, J2, K2, IU1, M1);
            else a = flwd(c, I1, J1, K1, IU1, M1, sgm);
            as[(IU1 - 1) * 2 + (M1 - 1)] = a;
            ap = ap + a;
            g0 = g0 + a * A(c.FZ, I2, J2, K2);
        }
        // ---- ECELL ----------------------------------------------------------------
        R FFL[4][3];
        if (IU1 == 1) {
            int I1 = I - 1, I2 = I - 2;
            for (int M = 1; M <= 2; ++M) {
                FFL[1][M] = IBC(g, I2, J, K) >= 1 ? g.DX[I1] : fabs(g.X[I] - g.X[I1]);
                FFL[2][M] = FFL[1][M] * g.DZ[K];
                FFL[3][M] = FFL[1][M] * g.RS[J] * g.DR[J];
                I1 = I + 1; I2 = I + 2;
            }
        } else if (IU1 == 2) {
            int J1 = J - 1, J2 = J - 2;
            for (int M = 1; M <= 2; ++M) {
                FFL[2][M] = IBC(g, I, J2, K) >= 1 ? g.RS[J1] * g.DR[J1] : g.RS[J1] * fabs(g.Rr[J] - g.Rr[J1]);
                FFL[1][M] = FFL[2][M] * g.DZ[K];
                FFL[3][M] = FFL[2][M] * g.DX[I];
                J1 = J + 1; J2 = J + 2;
            }
        } else {
            int K1 = K - 1, K2 = K - 2;
            for (int M = 1; M <= 2; ++M) {
                FFL[3][M] = IBC(g, I, J, K2) >= 1 ? g.DZ[K1] : fabs(g.Z[K] - g.Z[K1]);
                FFL[1][M] = FFL[3][M] * g.RS[J] * g.DR[J];
                FFL[2][M] = FFL[3][M] * g.DX[I];
                K1 = K + 1; K2 = K + 2;
            }
        }
        // ---- cross-direction coefficients (Gslv3x.f90:35-77) -------------------
        for (int IU = 1; IU <= 3; ++IU) {
            if (IU == IU1) continue;
            int NY[4] = {0, 0, 0, 0};
            for (int M = -1; M <= 1; M += 2) {
                int M1 = (M + 3) / 2;
                NY[IU] = M;
                int I1 = I + NY[1], J1 = J + NY[2], K1 = K + NY[3];
                int I2 = I1 + NY[1], J2 = J1 + NY[2], K2 = K1 + NY[3];
                if (IBC(g, I1, J1, K1) == 3) { as[(IU - 1) * 2 + (M1 - 1)] = zero; continue; }
                R f = zero, diff = zero;
                int II1 = 0, JJ1 = 0, KK1 = 0;
                for (int Nn = -1; Nn <= 1; Nn += 2) {
                    int N1 = (Nn + 3) / 2;
                    II1 = I1 + NX[1] * Nn; JJ1 = J1 + NX[2] * Nn; KK1 = K1 + NX[3] * Nn;
                    int ibc1 = IBC(g, II1, JJ1, KK1);
                    if (ibc1 == 3) continue;
                    R area = FFL[IU][N1];
                    f = f + A(c.THETA, II1, JJ1, KK1) * A(c.DNST, II1, JJ1, KK1) * A(c.FZ, II1, JJ1, KK1) * area;
                    if (ibc1 == 2) continue;
                    R ddl = fddl(g, II1, JJ1, KK1, IU);
                    diff = diff + A(c.THETA, II1, JJ1, KK1) * A(c.GAMA, II1, JJ1, KK1) / sgm * area / ddl;
                }
                R fld = M1 == 1 ? da<R>(diff, f) + rmax(zero, f) : da<R>(diff, f) + rmax(zero, -f);
                if (IBC(g, II1, JJ1, KK1) == 2 && IBC(g, I2, J2, K2) == 1) {
                    R bs0 = fld * (A(c.UG[IU1 - 1], II1, J2, K2) - A(c.UG[IU1 - 1], I, J, K));
                    bs = bs + bs0;
                    as[(IU - 1) * 2 + (M1 - 1)] = zero;
                    continue;
                }
                as[(IU - 1) * 2 + (M1 - 1)] = fld;
                ap = ap + fld;
                g0 = g0 + fld * A(c.FZ, I2, J2, K2);
            }
        }
        // ---- VOL1 and the SIMPLER pseudo-velocity (Gslv3x.f90:100-110) ----------
        R area = area_c(g, I, J, K, IU1);
        R vol = (FFL[IU1][1] + FFL[IU1][2]) * area;
        if (IU1 == 1) {
            if (IBC(g, I - 1, J, K) <= -1) vol = vol - g.DX[I - 1] * area / R(2);
            if (IBC(g, I + 1, J, K) <= -1) vol = vol - g.DX[I + 1] * area / R(2);
        } else if (IU1 == 2) {
            if (IBC(g, I, J - 1, K) <= -1) vol = vol - g.RS[J - 1] * g.DR[J - 1] * area / R(2);
            if (IBC(g, I, J + 1, K) <= -1) vol = vol - g.RS[J + 1] * g.DR[J + 1] * area / R(2);
        } else {
            if (IBC(g, I, J, K - 1) <= -1) vol = vol - g.DZ[K - 1] * area / R(2);
            if (IBC(g, I, J, K + 1) <= -1) vol = vol - g.DZ[K + 1] * area / R(2);
        }
        bs = bs * vol;
        ap = ap + (zero - zero - sfp) * vol;
        if (fabs(ap) > R(1.0e-20)) c.UG[IU1 - 1][o] = (g0 + bs) / ap;
        c.APm[o] = ap;
        for (int q = 0; q < 6; ++q) c.ASm[q][o] = as[q];
        c.BSm[o] = bs;
        c.SFPm[o] = sfp;
    }
}

// ---------------------------------------------------------------------------
// Pressure equation: SOURCE NELG=4 (Source.f90:35-74) + coefficients
// (Gslv3v.f90:43-89) on the centre class.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_p_assemble(Ctx<R> c, Range rg) {
    const GeoT<R>& g = c.g;
    const R zero = R(0);
    long long n = rg.count();
    GFM_FOR(t, n) {
        int I, J, K;
        rg.at(t, I, J, K);
        const long long o = pidx(g, I, J, K);
        if (g.ib[o] >= 1) {
            c.APc[o] = R(1);
            for (int q = 0; q < 6; ++q) c.ASc[q][o] = zero;
            c.BSp[o] = c.P[o];
            continue;
        }
        R ax = area_c(g, I, J, K, 1), ay = area_c(g, I, J, K, 2), az = area_c(g, I, J, K, 3);
        R frx1 = (A(c.THETA, I - 1, J, K) * A(c.DNST, I - 1, J, K) * A(c.UG[0], I - 1, J, K)) * ax;
        R frx2 = (A(c.THETA, I + 1, J, K) * A(c.DNST, I + 1, J, K) * A(c.UG[0], I + 1, J, K)) * ax;
        R fry1 = (A(c.THETA, I, J - 1, K) * A(c.DNST, I, J - 1, K) * A(c.UG[1], I, J - 1, K)) * ay;
        R fry2 = (A(c.THETA, I, J + 1, K) * A(c.DNST, I, J + 1, K) * A(c.UG[1], I, J + 1, K)) * ay;
        R frz1 = (A(c.THETA, I, J, K - 1) * A(c.DNST, I, J, K - 1) * A(c.UG[2], I, J, K - 1)) * az;
        R frz2 = (A(c.THETA, I, J, K + 1) * A(c.DNST, I, J, K + 1) * A(c.UG[2], I, J, K + 1)) * az;
        R bs = ((frx1 - frx2) + (fry1 - fry2) + (frz1 - frz2) + zero) / R(c.p.eun);
        R sfp = zero;
        R ap = -sfp;
        R as[6];
        for (int d = 0; d < 3; ++d)
            for (int M = 1; M <= 2; ++M) {
                int I1 = I, J1 = J, K1 = K;
                if (d == 0) I1 = M == 1 ? I - 1 : I + 1;
                else if (d == 1) J1 = M == 1 ? J - 1 : J + 1;
                else K1 = M == 1 ? K - 1 : K + 1;
                R a = zero;
                R apf = A(c.APm, I1, J1, K1);
                if (IBC(g, I1, J1, K1) <= 0 && fabs(apf) > R(1.0e-20)) {
                    R area = d == 0 ? ax : (d == 1 ? ay : az);
                    R th = A(c.THETA, I1, J1, K1);
                    R lav_num = d == 0 ? dxav(g, I1, J1, K1) : (d == 1 ? drav(g, I1, J1, K1) : dzav(g, I1, J1, K1));
                    R lav_den = d == 0 ? g.DX[I1] : (d == 1 ? g.DR[J1] : g.DZ[K1]);
                    a = th * th * A(c.DNST, I1, J1, K1) * (area * area) / apf * lav_num / lav_den;
                }
                as[d * 2 + (M - 1)] = a;
                ap = ap + a;
            }
        c.APc[o] = ap;
        for (int q = 0; q < 6; ++q) c.ASc[q][o] = as[q];
        c.BSp[o] = bs;
    }
}

// BOUND(P,0,1) on open cells after the pressure solve (Gslv3v.f90:96-101)
template <typename R>
__global__ void k_bound_p(Ctx<R> c, Range rg) {
    const GeoT<R>& g = c.g;
    long long n = rg.count();
    GFM_FOR(t, n) {
        int I, J, K;
        rg.at(t, I, J, K);
        long long o = pidx(g, I, J, K);
        if (g.ib[o] >= 1) continue;
        R f = c.P[o];
        f = rmin(f, R(c.p.p_mx));
        f = rmax(f, R(c.p.p_mn));
        c.P[o] = f;
    }
}

// Momentum right-hand side with the new pressure (Gslv3v.f90:106-130)
template <typename R, int IU1>
__global__ void k_mom_prep(Ctx<R> c, Range rg) {
    const GeoT<R>& g = c.g;
    long long n = rg.count();
    GFM_FOR(t, n) {
        int I, J, K;
        rg.at(t, I, J, K);
        long long o = pidx(g, I, J, K);
        if (g.ib[o] >= 1) continue;
        R ap = c.APm[o] / R(c.p.rf[IU1 - 1]);
        c.APm[o] = ap;
        R vol = vol_c(g, I, J, K), dpdx;
        if (IU1 == 1) dpdx = (A(c.P, I - 1, J, K) - A(c.P, I + 1, J, K)) / g.DX[I];
        else if (IU1 == 2) dpdx = (A(c.P, I, J - 1, K) - A(c.P, I, J + 1, K)) / g.DR[J] / g.RS[J];
        else dpdx = (A(c.P, I, J, K - 1) - A(c.P, I, J, K + 1)) / g.DZ[K];
        c.BSm[o] = c.BSm[o] + R(c.p.eun) * c.THETA[o] * vol * dpdx + R(c.p.rfc[IU1 - 1]) * ap * c.FZ[o];
    }
}

template <typename R>
__device__ __forceinline__ R bound_vel(R f, const Prm& p) {
    f = rmin(f, R(p.u_mx));
    f = rmax(f, R(p.u_mn));
    if (fabs(f) < R(1.0e-12)) f = R(0);
    return f;
}

// BOUND and UG <- FZ after the momentum solve (Gslv3v.f90:137-143)
template <typename R>
__global__ void k_mom_finish(Ctx<R> c, Range rg, int iu) {
    const GeoT<R>& g = c.g;
    long long n = rg.count();
    GFM_FOR(t, n) {
        int I, J, K;
        rg.at(t, I, J, K);
        long long o = pidx(g, I, J, K);
        if (g.ib[o] >= 1) continue;
        R f = bound_vel(c.FZ[o], c.p);
        c.FZ[o] = f;
        c.UG[iu][o] = f;
    }
}

// SOURCE NELG=5: mass imbalance of the corrected velocities and res_mass
// (Source.f90:35-101); FZ(centres)=0 (Gslv3v.f90:157-161).  Per-block
// partial sums of r_mass and its maximum go to `partials` slots 0/1.
template <typename R>
__global__ void k_pcorr_source(Ctx<R> c, Range rg) {
    __shared__ double sh[32];
    const GeoT<R>& g = c.g;
    long long n = rg.count();
    double rsum = 0.0, rmx = 0.0;
    GFM_FOR(t, n) {
        int I, J, K;
        rg.at(t, I, J, K);
        long long o = pidx(g, I, J, K);
        if (g.ib[o] >= 1) continue;
        R ax = area_c(g, I, J, K, 1), ay = area_c(g, I, J, K, 2), az = area_c(g, I, J, K, 3);
        R frx1 = (A(c.THETA, I - 1, J, K) * A(c.DNST, I - 1, J, K) * A(c.UG[0], I - 1, J, K)) * ax;
        R frx2 = (A(c.THETA, I + 1, J, K) * A(c.DNST, I + 1, J, K) * A(c.UG[0], I + 1, J, K)) * ax;
        R fry1 = (A(c.THETA, I, J - 1, K) * A(c.DNST, I, J - 1, K) * A(c.UG[1], I, J - 1, K)) * ay;
        R fry2 = (A(c.THETA, I, J + 1, K) * A(c.DNST, I, J + 1, K) * A(c.UG[1], I, J + 1, K)) * ay;
        R frz1 = (A(c.THETA, I, J, K - 1) * A(c.DNST, I, J, K - 1) * A(c.UG[2], I, J, K - 1)) * az;
        R frz2 = (A(c.THETA, I, J, K + 1) * A(c.DNST, I, J, K + 1) * A(c.UG[2], I, J, K + 1)) * az;
        R bs = ((frx1 - frx2) + (fry1 - fry2) + (frz1 - frz2) + R(0)) / R(c.p.eun);
        c.BSq[o] = bs;
        if (IBC(g, I - 1, J, K) == 3 || IBC(g, I + 1, J, K) == 3 || IBC(g, I, J - 1, K) == 3 ||
            IBC(g, I, J + 1, K) == 3 || IBC(g, I, J, K - 1) == 3 || IBC(g, I, J, K + 1) == 3)
            continue;
        double fmx = fmax(fmax(fmax(fmax(fmax(fabs((double)frx1), fabs((double)frx2)), fabs((double)fry1)),
                                   fabs((double)fry2)), fabs((double)frz1)), fabs((double)frz2));
        double r_mass = fmx == 0.0 ? 0.0 : fabs((double)bs) * c.p.eun / fmx;
        rsum += r_mass;
        rmx = r_mass > rmx ? r_mass : rmx;
    }
    double s = block_sum(rsum, sh);
    double m = block_max(rmx, sh);
    if (threadIdx.x == 0) {
        c.partials[0 * kRedBlocks + blockIdx.x] = s;
        c.partials[1 * kRedBlocks + blockIdx.x] = m;
    }
}

template <typename R>
__global__ void k_zero_centres(Ctx<R> c) {
    GFM_FOR(t, c.g.CB)
        c.FZ[t] = R(0);   // class 0 = cell centres
}

// Velocity correction (Gslv3v.f90:179-204)
template <typename R, int IU1>
__global__ void k_velcorr(Ctx<R> c, Range rg) {
    const GeoT<R>& g = c.g;
    long long n = rg.count();
    GFM_FOR(t, n) {
        int I, J, K;
        rg.at(t, I, J, K);
        long long o = pidx(g, I, J, K);
        if (g.ib[o] >= 1 || fabs(c.APm[o]) < R(1.0e-20)) continue;
        R vol = vol_c(g, I, J, K), dpdx;
        if (IU1 == 1) dpdx = (A(c.FZ, I - 1, J, K) - A(c.FZ, I + 1, J, K)) / g.DX[I];
        else if (IU1 == 2) dpdx = (A(c.FZ, I, J - 1, K) - A(c.FZ, I, J + 1, K)) / g.DR[J] / g.RS[J];
        else dpdx = (A(c.FZ, I, J, K - 1) - A(c.FZ, I, J, K + 1)) / g.DZ[K];
        R g0 = R(c.p.eun) * c.THETA[o] * dpdx * vol / (c.APm[o] * R(c.p.rf[IU1 - 1]));
        c.UG[IU1 - 1][o] = bound_vel(c.UG[IU1 - 1][o] + g0, c.p);
    }
}

// ---------------------------------------------------------------------------
// Scalar transport (Gslv3g.f90:6-152 with SOURCE cases 6-12)
// ---------------------------------------------------------------------------
// fuel source: integral reaction submodel (Source.f90:104-242); writes CRATE,
// HRATE and the fuel equation's BS/SFP
template <typename R>
__global__ void k_fuel_source(Ctx<R> c, Range rg) {
    const GeoT<R>& g = c.g;
    long long n = rg.count();
    const R zero = R(0);
    GFM_FOR(t, n) {
        int I, J, K;
        rg.at(t, I, J, K);
        long long o = pidx(g, I, J, K);
        R* bs = c.BSs[0];
        R* sfp = c.SFPs[0];
        if (g.ib[o] >= 1) {
            bs[o] = c.GF[kYF][o]; sfp[o] = zero; c.CRATE[o] = zero; c.HRATE[o] = zero;
            continue;
        }
        R d11 = fabs(A(c.UG[0], I + 1, J, K) / g.DX[I]);
        R d12 = fabs(A(c.UG[0], I - 1, J, K) / g.DX[I]);
        R d21 = zero, d22 = zero, d31 = zero, d32 = zero;
        if (rg.j1 > 6) { d21 = fabs(A(c.UG[1], I, J + 1, K) / g.DR[J]); d22 = fabs(A(c.UG[1], I, J - 1, K) / g.DR[J]); }
        if (rg.k1 > 6) { d31 = fabs(A(c.UG[2], I, J, K + 1) / g.DZ[K]); d32 = fabs(A(c.UG[2], I, J, K - 1) / g.DZ[K]); }
        double dtime = rmax(rmax(rmax(rmax(rmax(rmax((double)d11, (double)d12), (double)d21), (double)d22), (double)d31), (double)d32), 1.0e-14);
        dtime = 1.0 / dtime;
        double drtime = dtime * c.p.r0 / c.p.ug0;
        double yf = c.GF[kYF][o], yo2 = c.GF[kYO2][o];
        double ayf = rmin(yf, yo2 / c.p.stoich);
        if (ayf < 1.0e-5) { c.CRATE[o] = zero; c.HRATE[o] = zero; sfp[o] = zero; bs[o] = zero; continue; }
        double zp1 = (double)c.GF[kYCO2][o] / kWco2, delr1;
        if (zp1 <= kSmall20) delr1 = 0.0;
        else { double zf = yf / kWf; delr1 = zp1 / (zf + zp1); }
        double time1 = zy1(c.delr, c.timed, delr1, c.nr0);
        double time2 = time1 + drtime;
        double delr2 = zy1(c.rtim, c.delrt, time2, c.nr0);
        double ayf0 = ayf / (1.0 - delr1) * (double)c.DNST[o] * (double)c.THETA[o];
        double sr = ayf0 * (delr2 - delr1) / dtime;
        if (sr <= 0.0) { c.CRATE[o] = zero; c.HRATE[o] = zero; sfp[o] = zero; bs[o] = zero; continue; }
        c.CRATE[o] = R(sr);
        sfp[o] = -c.CRATE[o] / (c.GF[kYF][o] + R(kSmall20));
        bs[o] = zero;
        c.HRATE[o] = c.CRATE[o] * R(c.p.q0);
    }
}

// q_conv per wall patch (Qwall.f90:1370-1475), T in K = T*T0
template <typename R>
__global__ void k_qconv(Ctx<R> c) {
    __shared__ double sh[32];
    const GeoT<R>& g = c.g;
    const double pi = 3.141592653589793;
    const double kappa_cmu = 0.4 * pow(9.0e-2, 0.25), E_cmu = 9.0 * pow(9.0e-2, 0.25);
    const double c_htw = 0.4 * ((pi / 4) / sin(pi / 4)) * sqrt(26.0) * (0.7 - 1.0) / pow(0.7, 0.25);
    const double cp1[5] = {2.156e+3 / 1.0057e+3, 2.0e+3 / 1.0057e+3, 2.0e+3 / 1.0057e+3, 0.9136e+3 / 1.0057e+3, 0.526e+3 / 1.0057e+3};
    double tot = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < c.n_patch; n += gridDim.x * blockDim.x) {
        const Patch& q = c.patch[n];
        long long o = pidx(g, q.inc, q.jnc, q.knc);
        double yf = c.GF[kYF][o], yco2 = c.GF[kYCO2][o], yh2o = c.GF[kYH2O][o], yo2 = c.GF[kYO2][o], yn2 = c.GF[kYN2][o];
        double cpmix = kCp0 * (cp1[0] * yf + cp1[1] * yco2 + cp1[2] * yh2o + cp1[3] * yo2 + cp1[4] * yn2);
        double Tgas = (double)c.T[o] * c.p.t0;
        double gmu = ((kGmu3 * Tgas + kGmu2) * Tgas + kGmu1) * Tgas + kGmu0;
        double k = c.GF[kK][o], rho = c.DNST[o], h_t;
        if (c.p.tk0 * k < 0.1) h_t = 0.0;
        else {
            double sq = sqrt(c.p.tk0 * k);
            double dtmp = (log(E_cmu * q.ds_q * c.p.dnst0 * rho * sq / gmu) + (c_htw / sq));
            if (dtmp < 0.01) h_t = 0.0;
            else { h_t = cpmix * kappa_cmu * c.p.dnst0 * rho * sq / dtmp; h_t = h_t < 50.0 ? h_t : 50.0; }
        }
        double qc = (c.p.h_g > h_t ? c.p.h_g : h_t) * (Tgas - q.bT);
        c.qconv[n] = R(qc);
        tot += qc * q.area;
    }
    double s = block_sum(tot, sh);
    if (threadIdx.x == 0) c.partials[4 * kRedBlocks + blockIdx.x] = s;
}

// Generic scalar assembly for equation L (1..7): the SOURCE case of its NELG,
// GSLV3G0 coefficients (new set or reuse of an equal-sigma set) and the
// relaxation (Gslv3g.f90:51-87).  The enthalpy case also computes GTE, the
// radiation term, the wall sink gathered per cell in patch order and the
// source relaxation with bs_hprev (Source.f90:269-522).
template <typename R, int L>
__global__ void k_scalar_assemble(Ctx<R> c, Range rg) {
    __shared__ double sh[32];
    const GeoT<R>& g = c.g;
    const R zero = R(0);
    constexpr int NELG = L == 1 ? 6 : L == 6 ? 7 : L == 3 ? 8 : L == 4 ? 9 : L == 5 ? 10 : L == 7 ? 11 : 12;
    R* ap_out = c.APs[L - 1];
    R* bs_out = c.BSs[L - 1];
    R* as_set[6];
    for (int q = 0; q < 6; ++q) as_set[q] = c.ASs[c.as_set[L - 1]][q];
    const R* fz = c.GF[L - 1];
    long long n = rg.count();
    double qreact = 0.0;
    const int itr_gas = (int)c.scal[S_ITR_GAS];
    const bool rad_active = c.scal[S_RAD_ACTIVE] > 0.0;
    GFM_FOR(t, n) {
        int I, J, K;
        rg.at(t, I, J, K);
        const long long o = pidx(g, I, J, K);
        const bool blocked = g.ib[o] >= 1;
        R bs = zero, sfp = zero;
        // ---- SOURCE -------------------------------------------------------------
        if (NELG == 6) {
            bs = c.BSs[0][o]; sfp = c.SFPs[0][o];
        } else if (blocked) {
            bs = fz[o]; sfp = zero;
        } else if (NELG == 7) {
            bs = c.p.react ? c.CRATE[o] * R(kWco2 / kWf) : zero;
        } else if (NELG == 12) {
            bs = c.p.react ? -c.CRATE[o] * R(c.p.stoich) : zero;
        } else if (NELG == 11) {
            bs = zero;
        } else if (NELG == 8) {
            // GTE (Source.f90:278-316)
            R dudx, dvdx, dwdx, dudr, dvdr, dwdr, dudz, dvdz, dwdz;
            if (IBC(g, I + 1, J, K) == 3 || IBC(g, I - 1, J, K) == 3) { dudx = dvdx = dwdx = zero; }
            else {
                dudx = (A(c.UG[0], I + 1, J, K) - A(c.UG[0], I - 1, J, K)) / g.DX[I];
                dvdx = (A(c.UG[1], I + 1, J, K) - A(c.UG[1], I - 1, J, K)) / g.DX[I];
                dwdx = (A(c.UG[2], I + 1, J, K) - A(c.UG[2], I - 1, J, K)) / g.DX[I];
            }
            if (rg.j1 < 6 || IBC(g, I, J + 1, K) == 3 || IBC(g, I, J - 1, K) == 3) { dudr = dvdr = dwdr = zero; }
            else {
                dudr = (A(c.UG[0], I, J + 1, K) - A(c.UG[0], I, J - 1, K)) / g.DR[J];
                dvdr = (A(c.UG[1], I, J + 1, K) - A(c.UG[1], I, J - 1, K)) / g.DR[J];
                dwdr = (A(c.UG[2], I, J + 1, K) - A(c.UG[2], I, J - 1, K)) / g.DR[J];
            }
            if (rg.k1 < 6 || IBC(g, I, J, K + 1) == 3 || IBC(g, I, J, K - 1) == 3) { dudz = dvdz = dwdz = zero; }
            else {
                dudz = (A(c.UG[0], I, J, K + 1) - A(c.UG[0], I, J, K - 1)) / g.DZ[K];
                dvdz = (A(c.UG[1], I, J, K + 1) - A(c.UG[1], I, J, K - 1)) / g.DZ[K];
                dwdz = (A(c.UG[2], I, J, K + 1) - A(c.UG[2], I, J, K - 1)) / g.DZ[K];
            }
            R s1 = dudr + dvdx, s2 = dwdr + dvdz, s3 = dudz + dwdx, s4 = dudx + dvdr + dwdz;
            R gte = R(2) * (dudx * dudx + dvdr * dvdr + zero * zero + dwdz * dwdz) + s1 * s1 + s2 * s2 + s3 * s3 - s4 * s4 / R(1.5);
            c.GTE[o] = gte;
            bs = zero + c.HRATE[o];
            sfp = -zero;
            R vol = vol_c(g, I, J, K);
            qreact += (double)c.HRATE[o] * c.p.qr0 * (double)vol;
        } else if (NELG == 9) {
            bs = R(2) / R(c.p.reyg * c.p.epsr) * c.THETA[o] * c.TMU[o] * c.GTE[o] - zero;
            sfp = -(R(c.p.taur) * c.THETA[o] * c.DNST[o] * c.GF[kEps][o] / (c.GF[kK][o] + R(kSmall20)));
        } else if (NELG == 10) {
            const R cbl0 = R(c.p.cbl0);
            R cbl = cbl0 * r_pow(c.GF[kK][o], R(1.5));
            const R BIGV = R(1.0e20);
            bool pen = false;
            if (g.MP > 8 && IBC(g, I + 1, J, K) == 1) { bs = bs + BIGV * cbl / (g.X[I + 1] - g.X[I]); pen = true; }
            if (g.MP > 8 && IBC(g, I - 1, J, K) == 1) { bs = bs + BIGV * cbl / (g.X[I] - g.X[I - 1]); pen = true; }
            if (g.NP > 8 && IBC(g, I, J + 1, K) == 1) { bs = bs + BIGV * cbl / (g.Rr[J + 1] - g.Rr[J]); pen = true; }
            if (g.NP > 8 && IBC(g, I, J - 1, K) == 1) { bs = bs + BIGV * cbl / (g.Rr[J] - g.Rr[J - 1]); pen = true; }
            if (g.LP > 8 && IBC(g, I, J, K + 1) == 1) { bs = bs + BIGV * cbl / (g.Z[K + 1] - g.Z[K]); pen = true; }
            if (g.LP > 8 && IBC(g, I, J, K - 1) == 1) { bs = bs + BIGV * cbl / (g.Z[K] - g.Z[K - 1]); pen = true; }
            if (pen) sfp = -BIGV;
            else {
                R bt = c.THETA[o];
                bs = R(c.p.ct1) * R(c.p.cmu) * bt / R(c.p.taur) * c.DNST[o] * c.GTE[o] * c.GF[kK][o];
                sfp = -(R(c.p.ct2) * R(c.p.taur) * bt * c.DNST[o] * c.GF[kEps][o] / (c.GF[kK][o] + R(kSmall20)));
            }
        }
        if (NELG == 8 && !blocked) {
            // radiation rate (Source.f90:437-447)
            if (rad_active) {
                R vol = vol_c(g, I, J, K);
                R q_rad = c.QA[o] - c.QE[o];
                bs = bs + q_rad / (vol * R(c.p.qr0));
            }
            // fixed-temperature wall sink, patches of this cell in patch order (Source.f90:473-509)
            if (c.p.wall_sink && c.cell_patch_start) {
                // CSR over the centre class: class 0 offset == linear index
                int b0 = c.cell_patch_start[o], b1 = c.cell_patch_start[o + 1];
                for (int b = b0; b < b1; ++b) {
                    int pn = c.cell_patch_list[b];
                    const Patch& q = c.patch[pn];
                    bs = bs - c.qconv[pn] / (R(q.ds_src) * R(c.p.r0) * R(c.p.qr0));
                }
            }
            if (itr_gas > 1) bs = R(c.p.rf_hsource) * bs + (R(1) - R(c.p.rf_hsource)) * c.BSH[o];
        }
        if (blocked) {
            // blocked cells keep AP=1, AS=0 and BS=FZ (GSLV3V reset / SOURCE)
            ap_out[o] = R(1);
            bs_out[o] = bs;
            continue;
        }
        if (NELG == 8) c.BSH[o] = bs;   // bs_hprev = bs (Source.f90:520)
        // ---- GSLV3G0: AP from the six coefficients (k_scalar_faces) ----------------
        R ap = zero;
        for (int q = 0; q < 6; ++q) ap = ap + as_set[q][o];
        // ---- relaxation (Gslv3g.f90:64-87) -----------------------------------------
        if (fabs(ap) <= R(1.0e-20)) { ap_out[o] = R(1); bs_out[o] = fz[o]; continue; }
        R vol = vol_c(g, I, J, K);
        bs = bs * vol;
        ap = ap - (sfp * vol);
        ap = ap / R(c.p.rfl[L - 1]);
        bs = bs + R(c.p.rflc[L - 1]) * fz[o] * ap;
        ap_out[o] = ap;
        bs_out[o] = bs;
    }
    if (NELG == 8) {
        double s = block_sum(qreact, sh);
        if (threadIdx.x == 0) c.partials[5 * kRedBlocks + blockIdx.x] = s;
    }
}

// ---------------------------------------------------------------------------
// GSLV3G0's six neighbour coefficients of the scalar equations (Gslv3g.f90:
// 30-47 with FLWD/FLW, Gslv3x.f90:292-329), evaluated once per face.  The
// reference forms them per cell, so every interior face's flux f and
// diffusion conductance, and the DA weight of the pair, are evaluated by
// both cells that share it; here one thread per face (blockIdx.y = direction
// IU) evaluates them once and writes the coefficient of the cell on each
// side: AS(C-, IU, +) = DA + max(0,-f), AS(C+, IU, -) = DA + max(0,f), or
// FLW at an inlet neighbour, or 0 at a blocked one, as each cell would.  The
// values are the cell-wise ones bit for bit.  Cells outside the solved range
// are not written; blocked cells in it get 0.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_scalar_faces(Ctx<R> c, Range cr, int set, R sgm) {
    const GeoT<R>& g = c.g;
    const int IU = (int)blockIdx.y + 1;
    R* const* as_set = c.ASs[set];
    // faces of direction IU: the cell range widened by one face on each end
    const int fi0 = IU == 1 ? cr.i0 - 1 : cr.i0, fi1 = IU == 1 ? cr.i1 + 1 : cr.i1;
    const int fj0 = IU == 2 ? cr.j0 - 1 : cr.j0, fj1 = IU == 2 ? cr.j1 + 1 : cr.j1;
    const int fk0 = IU == 3 ? cr.k0 - 1 : cr.k0, fk1 = IU == 3 ? cr.k1 + 1 : cr.k1;
    const Range fr{fi0, fi1, fj0, fj1, fk0, fk1};
    const int ex = IU == 1, ey = IU == 2, ez = IU == 3;
    const long long n = fr.count();
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int I, J, K;
        fr.at((int)t, I, J, K);
        const int Im = I - ex, Jm = J - ey, Km = K - ez, Ip = I + ex, Jp = J + ey, Kp = K + ez;
        const bool in_m = IU == 1 ? Im >= cr.i0 : IU == 2 ? Jm >= cr.j0 : Km >= cr.k0;
        const bool in_p = IU == 1 ? Ip <= cr.i1 : IU == 2 ? Jp <= cr.j1 : Kp <= cr.k1;
        const int ib_m = IBC(g, Im, Jm, Km), ib_p = IBC(g, Ip, Jp, Kp);
        const bool want_m = in_m && ib_m < 1, want_p = in_p && ib_p < 1;
        R dsum = R(0), f = R(0);
        if ((want_m && ib_p <= 0) || (want_p && ib_m <= 0)) {
            // FLWD's flux and conductance at the face, DA once
            const R area = area_c(g, I, J, K, IU);
            const R ddl = IU == 1 ? g.DX[I] : (IU == 2 ? g.DR[J] : g.DZ[K]);
            f = A(c.THETA, I, J, K) * A(c.DNST, I, J, K) * A(c.UG[IU - 1], I, J, K) * area;
            const R diff = A(c.THETA, I, J, K) * A(c.GAMA, I, J, K) / sgm * area / ddl;
            dsum = da<R>(diff, f);
        }
        // the cell on the - side: its + neighbour is the cell on the + side
        if (in_m) {
            R a = R(0);
            if (want_m) {
                if (ib_p <= 0) a = dsum + rmax(R(0), -f);
                else if (ib_p == 2) a = flw(c, Ip, Jp, Kp, IU, 2);
            }
            as_set[(IU - 1) * 2 + 1][pidx(g, Im, Jm, Km)] = a;
        }
        if (in_p) {
            R a = R(0);
            if (want_p) {
                if (ib_m <= 0) a = dsum + rmax(R(0), f);
                else if (ib_m == 2) a = flw(c, Im, Jm, Km, IU, 1);
            }
            as_set[(IU - 1) * 2][pidx(g, Ip, Jp, Kp)] = a;
        }
    }
}

// BOUND and GF(L) <- FZ after a scalar solve (Gslv3g.f90:100-106).  The solve
// runs on FZs[L-1], a copy of GF(L) (FZ=GF(L), Gslv3g.f90:51-55).
template <typename R>
__global__ void k_scalar_finish(Ctx<R> c, Range rg, int L) {
    const GeoT<R>& g = c.g;
    R* fz = c.FZs[L - 1];
    R* gf = c.GF[L - 1];
    long long n = rg.count();
    GFM_FOR(t, n) {
        int I, J, K;
        rg.at(t, I, J, K);
        long long o = pidx(g, I, J, K);
        if (g.ib[o] >= 1) continue;
        R f = fz[o];
        if (L == kK + 1) f = rmax(f, R(1.0e-6));
        else if (L == kEps + 1) f = rmax(f, R(1.0e-12));
        else if (L == kH + 1) {}
        else { f = rmin(f, R(1)); f = rmax(f, R(0)); }
        gf[o] = f;
    }
}

// FZ(L) <- GF(L) on all centres before the solve (Gslv3g.f90:51-55)
template <typename R>
__global__ void k_copy_centres(const R* __restrict__ src, R* __restrict__ dst, long long n) {
    GFM_FOR(t, n) dst[t] = src[t];
}

// ---------------------------------------------------------------------------
// Property update on open cell centres (Gflow.f90:302-382)
// ---------------------------------------------------------------------------
template <typename R>
__device__ void ther(Ctx<R>& c, long long o) {
    R eps = rmax(c.GF[kEps][o], R(1.0e-12));
    c.GF[kEps][o] = eps;
    R k = c.GF[kK][o];
    R g0 = R(c.p.cmu) * R(c.p.reyg) * R(c.p.epsr) / R(2.0 * c.p.taur) * (k * k) / eps * c.DNST[o];
    c.TMU[o] = g0;
    c.GAMA[o] = R(2) / R(c.p.reyg) * (g0 + r_pow(c.T[o] / R(c.p.trdg), R(c.p.amu)));
}

template <typename R>
__global__ void k_props(Ctx<R> c, Range rg) {
    const NistT<R>& nist = *c.nist;
    const GeoT<R>& g = c.g;
    long long n = rg.count();
    const R G0 = R(c.scal[S_G0]);
    const R t0 = R(c.p.t0), h0 = R(c.p.h_0), t_mx = R(c.p.t_mx), t_mn = R(c.p.t_mn);
    const R p_mx = R(c.p.p_mx), p_mn = R(c.p.p_mn), wt0 = R(c.p.wt0);
    GFM_FOR(t, n) {
        int I, J, K;
        rg.at(t, I, J, K);
        long long o = pidx(g, I, J, K);
        if (g.ib[o] >= 1) continue;
        R y[9];
        for (int l = 0; l < 9; ++l) y[l] = l == 7 ? R(0) : c.GF[l][o];
        conc(y, 1);
        R T = enth_to_t<R>(nist, y, 1, y[kH], c.T[o], t0, h0);
        if (T > t_mx) { T = t_mx; y[kH] = t_to_enth<R>(nist, y, 1, T, t0, h0); }
        else if (T < t_mn) { T = t_mn; y[kH] = t_to_enth<R>(nist, y, 1, T, t0, h0); }
        R pp = c.P[o] - G0;
        pp = pp < p_mx ? pp : p_mx;
        pp = pp > p_mn ? pp : p_mn;
        R rho = dnst_calc<R>(y, 1, pp, T, wt0);
        for (int l = 0; l < 9; ++l) if (l != 7) c.GF[l][o] = y[l];
        c.T[o] = T;
        c.P[o] = pp;
        c.DNST[o] = rho;
        ther(c, o);
    }
}

// Mass-weighted mean temperature (Utility.f90:1485-1510): slots 6 (T*rho*vol), 7 (rho*vol)
template <typename R>
__global__ void k_tave(Ctx<R> c, Range rg) {
    __shared__ double sh[32];
    const GeoT<R>& g = c.g;
    long long n = rg.count();
    double a = 0, b = 0;
    GFM_FOR(t, n) {
        int I, J, K;
        rg.at(t, I, J, K);
        long long o = pidx(g, I, J, K);
        if (g.ib[o] != 0) continue;
        double vol = vol_c(g, I, J, K);
        a += (double)c.T[o] * (double)c.DNST[o] * vol;
        b += (double)c.DNST[o] * vol;
    }
    double sa = block_sum(a, sh), sb = block_sum(b, sh);
    if (threadIdx.x == 0) { c.partials[6 * kRedBlocks + blockIdx.x] = sa; c.partials[7 * kRedBlocks + blockIdx.x] = sb; }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
inline int grid_for(long long n) {
    long long b = (n + kBlock - 1) / kBlock;
    if (b < 1) b = 1;
    if (b > kRedBlocks) b = kRedBlocks;
    return (int)b;
}
template <typename R> Range mom_range(const Ctx<R>& c, int iu) {
    const GeoT<R>& g = c.g;
    int nx1 = iu == 1;
    return Range{4 + nx1, g.MPM2 - nx1, g.NJY1V[iu], g.NJY2V[iu], g.LKZ1V[iu], g.LKZ2V[iu]};
}
template <typename R> Range cell_range(const Ctx<R>& c) {
    const GeoT<R>& g = c.g;
    return Range{4, g.MPM2, g.NJY1, g.NJY2, g.LKZ1, g.LKZ2};
}
template <typename R> Range all_centres(const Ctx<R>& c) {
    return Range{2, c.g.MP, 2, c.g.NP, 2, c.g.LP};
}

template <typename R> void launch_wallfn(const Ctx<R>& c, const int* wl, int n, cudaStream_t s) {
    if (n > 0) k_wallfn<R><<<grid_for(n), kBlock, 0, s>>>(c, wl, n);
}
template <typename R> void launch_copy_faces_to_fz(const Ctx<R>& c, cudaStream_t s) {
    k_copy_faces<R><<<grid_for(3 * c.g.CB), kBlock, 0, s>>>(c);
}
template <typename R> void launch_mom_assemble(const Ctx<R>& c, cudaStream_t s) {
    Range r1 = mom_range(c, 1), r2 = mom_range(c, 2), r3 = mom_range(c, 3);
    k_mom_assemble<R, 1><<<grid_for(r1.count()), kBlock, 0, s>>>(c, r1);
    k_mom_assemble<R, 2><<<grid_for(r2.count()), kBlock, 0, s>>>(c, r2);
    k_mom_assemble<R, 3><<<grid_for(r3.count()), kBlock, 0, s>>>(c, r3);
}
template <typename R> void launch_p_assemble(const Ctx<R>& c, cudaStream_t s) {
    Range r = cell_range(c);
    k_p_assemble<R><<<grid_for(r.count()), kBlock, 0, s>>>(c, r);
}
template <typename R> void launch_bound_p(const Ctx<R>& c, cudaStream_t s) {
    Range r = cell_range(c);
    k_bound_p<R><<<grid_for(r.count()), kBlock, 0, s>>>(c, r);
}
template <typename R> void launch_mom_prep(const Ctx<R>& c, cudaStream_t s) {
    Range r1 = mom_range(c, 1), r2 = mom_range(c, 2), r3 = mom_range(c, 3);
    k_mom_prep<R, 1><<<grid_for(r1.count()), kBlock, 0, s>>>(c, r1);
    k_mom_prep<R, 2><<<grid_for(r2.count()), kBlock, 0, s>>>(c, r2);
    k_mom_prep<R, 3><<<grid_for(r3.count()), kBlock, 0, s>>>(c, r3);
}
template <typename R> void launch_mom_finish(const Ctx<R>& c, cudaStream_t s) {
    for (int iu = 1; iu <= 3; ++iu) {
        Range r = mom_range(c, iu);
        k_mom_finish<R><<<grid_for(r.count()), kBlock, 0, s>>>(c, r, iu - 1);
    }
}
template <typename R> void launch_pcorr_source(const Ctx<R>& c, cudaStream_t s) {
    Range r = cell_range(c);
    k_pcorr_source<R><<<grid_for(r.count()), kBlock, 0, s>>>(c, r);
    k_zero_centres<R><<<grid_for(c.g.CB), kBlock, 0, s>>>(c);
}
template <typename R> void launch_velcorr(const Ctx<R>& c, cudaStream_t s) {
    Range r1 = mom_range(c, 1), r2 = mom_range(c, 2), r3 = mom_range(c, 3);
    k_velcorr<R, 1><<<grid_for(r1.count()), kBlock, 0, s>>>(c, r1);
    k_velcorr<R, 2><<<grid_for(r2.count()), kBlock, 0, s>>>(c, r2);
    k_velcorr<R, 3><<<grid_for(r3.count()), kBlock, 0, s>>>(c, r3);
}
template <typename R> void launch_qconv(const Ctx<R>& c, cudaStream_t s) {
    int nb = grid_for(c.n_patch > 0 ? c.n_patch : 1);
    k_qconv<R><<<nb, kBlock, 0, s>>>(c);
}
template <typename R> void launch_scalar_sources_first(const Ctx<R>& c, cudaStream_t s) {
    Range r = cell_range(c);
    k_fuel_source<R><<<grid_for(r.count()), kBlock, 0, s>>>(c, r);
}
// GSLV3G0's coefficients of the scalar range with sigma sgm into six given
// arrays (the minor species' set, SGM = SSIGMA, Gslv3m.f90:143-146)
template <typename R> void launch_scalar_faces_into(const Ctx<R>& c, R* const* as_out, double sgm, cudaStream_t s) {
    Ctx<R> cc = c;
    for (int q = 0; q < 6; ++q) cc.ASs[0][q] = as_out[q];
    Range r = cell_range(c);
    int nb = grid_for(r.count());
    k_scalar_faces<R><<<dim3(nb, 3), kBlock, 0, s>>>(cc, r, 0, R(sgm));
}
template <typename R> void launch_scalar_assemble(const Ctx<R>& c, int L, bool new_as, cudaStream_t s) {
    Range r = cell_range(c);
    int nb = grid_for(r.count());
    // the coefficient set of equal sigma, face by face, before its first equation
    if (new_as) k_scalar_faces<R><<<dim3(nb, 3), kBlock, 0, s>>>(c, r, c.as_set[L - 1], R(c.p.sigma[L - 1]));
    switch (L) {
        case 1: k_scalar_assemble<R, 1><<<nb, kBlock, 0, s>>>(c, r); break;
        case 2: k_scalar_assemble<R, 2><<<nb, kBlock, 0, s>>>(c, r); break;
        case 3: k_scalar_assemble<R, 3><<<nb, kBlock, 0, s>>>(c, r); break;
        case 4: k_scalar_assemble<R, 4><<<nb, kBlock, 0, s>>>(c, r); break;
        case 5: k_scalar_assemble<R, 5><<<nb, kBlock, 0, s>>>(c, r); break;
        case 6: k_scalar_assemble<R, 6><<<nb, kBlock, 0, s>>>(c, r); break;
        case 7: k_scalar_assemble<R, 7><<<nb, kBlock, 0, s>>>(c, r); break;
    }
    // FZ(L) <- GF(L) for the solve: class 0 block
    k_copy_centres<R><<<grid_for(c.g.CB), kBlock, 0, s>>>(c.GF[L - 1], c.FZs[L - 1], c.g.CB);
}
template <typename R> void launch_scalar_finish(const Ctx<R>& c, int L, cudaStream_t s) {
    Range r = cell_range(c);
    k_scalar_finish<R><<<grid_for(r.count()), kBlock, 0, s>>>(c, r, L);
}
template <typename R> void launch_props(const Ctx<R>& c, cudaStream_t s) {
    Range r = all_centres(c);
    k_props<R><<<grid_for(r.count()), kBlock, 0, s>>>(c, r);
}
template <typename R> void launch_tave(const Ctx<R>& c, cudaStream_t s) {
    Range r{4, c.g.MP - 2, 4, c.g.NP - 2, 4, c.g.LP - 2};
    k_tave<R><<<grid_for(r.count()), kBlock, 0, s>>>(c, r);
}

#define INST(R)                                                                              \
    template void launch_wallfn<R>(const Ctx<R>&, const int*, int, cudaStream_t);         \
    template void launch_copy_faces_to_fz<R>(const Ctx<R>&, cudaStream_t);                  \
    template void launch_mom_assemble<R>(const Ctx<R>&, cudaStream_t);                      \
    template void launch_p_assemble<R>(const Ctx<R>&, cudaStream_t);                        \
    template void launch_bound_p<R>(const Ctx<R>&, cudaStream_t);                           \
    template void launch_mom_prep<R>(const Ctx<R>&, cudaStream_t);                          \
    template void launch_mom_finish<R>(const Ctx<R>&, cudaStream_t);                        \
    template void launch_pcorr_source<R>(const Ctx<R>&, cudaStream_t);                      \
    template void launch_velcorr<R>(const Ctx<R>&, cudaStream_t);                           \
    template void launch_qconv<R>(const Ctx<R>&, cudaStream_t);                             \
    template void launch_scalar_sources_first<R>(const Ctx<R>&, cudaStream_t);              \
    template void launch_scalar_assemble<R>(const Ctx<R>&, int, bool, cudaStream_t);        \
    template void launch_scalar_faces_into<R>(const Ctx<R>&, R* const*, double, cudaStream_t); \
    template void launch_scalar_finish<R>(const Ctx<R>&, int, cudaStream_t);                \
    template void launch_tave<R>(const Ctx<R>&, cudaStream_t);                              \
    template void launch_props<R>(const Ctx<R>&, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace gfm
