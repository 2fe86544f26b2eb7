// pair.cu - real-space forces of force_real (src/forcem.f90:233-552).
//
//   k_pair_fp64   head-head pairs with the molecular cutoff, LJ/Buckingham on the heads,
//                 Ewald erfc on every site pair (src/forcem.f90:288-403)
//   k_wall_fp64   head-wall pairs: vdW on the head, erfc for each site of the head molecule
//                 against the frozen wall atom, wall reaction sums fws (src/forcem.f90:418-498)
//   k_surf_part   z forces of surface atoms booked to the wall they sit on (:408-413)
//   k_lr_tail     analytic wall long-range tail (:509-543, slab variant only)
//
// Layout: one warp per head atom i walks i's half list (partners j > i).  The i-side site
// forces stay in registers and are reduced with warp shuffles at the end (one atomic per
// component); j-side forces go out as FP64 atomics.  Energies are booked per head type pair
// (elj/eqq(ijt), src/forcem.f90:317,338,378) into shared memory, then once per block to HBM.
#include <algorithm>

#include "common.cuh"
#include "ctx.h"

namespace mdg {

namespace {

constexpr int kWarps = 8;
constexpr int kNT = kWarps * 32;

struct EAcc {
    int ijt = -1;
    double lj = 0.0, qq = 0.0;
};

__device__ __forceinline__ void e_flush(EAcc& e, double* s_e, int nijt) {
    if (e.ijt >= 0 && (e.lj != 0.0 || e.qq != 0.0)) {
        atomicAdd(&s_e[e.ijt], e.lj);
        atomicAdd(&s_e[nijt + e.ijt], e.qq);
    }
    e.lj = e.qq = 0.0;
}

// End of the loops: lanes holding the warp's (largest) pair type reduce with shuffles, one shared
// atomic per warp; lanes left with another type flush one by one.
__device__ __forceinline__ void e_final(EAcc& e, double* s_e, int nijt) {
    const int ij0 = __reduce_max_sync(0xffffffffu, e.ijt);
    if (ij0 < 0) return;
    const bool mine = e.ijt == ij0;
    const double lj = warp_sum(mine ? e.lj : 0.0);
    const double qq = warp_sum(mine ? e.qq : 0.0);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&s_e[ij0], lj);
        atomicAdd(&s_e[nijt + ij0], qq);
    }
    if (!mine) e_flush(e, s_e, nijt);
}

__device__ __forceinline__ void e_add(EAcc& e, int ijt, double lj, double qq, double* s_e, int nijt) {
    if (ijt != e.ijt) {
        e_flush(e, s_e, nijt);
        e.ijt = ijt;
    }
    e.lj += lj;
    e.qq += qq;
}

// Abramowitz-Stegun 7.1.26 erfc(alpha r) and the Ewald real-space force factor
// (src/forcem.f90:334-340):  returns erfx; *ff = (spii*alfar*exp2a + erfx)
__device__ __forceinline__ double ewald_erfc(double alfar, double* ff, double spii) {
    const double t = 1.0 / (1.0 + kP * alfar);
    const double exp2a = exp(-alfar * alfar);
    const double erfx = ((((kA5 * t + kA4) * t + kA3) * t + kA2) * t + kA1) * t * exp2a;
    *ff = spii * alfar * exp2a + erfx;
    return erfx;
}

__global__ void __launch_bounds__(kNT) k_pair_fp64(View v) {
    extern __shared__ double s_e[];  // 2 * nijt
    for (int k = threadIdx.x; k < 2 * v.nijt; k += blockDim.x) s_e[k] = 0.0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int nwarps = gridDim.x * kWarps;
    EAcc e;
    for (int h = warp; h < v.nheads; h += nwarps) {
        const int i = v.head_atom[CK(h, v.nheads, 101)];
        const int it = v.type[CK(i, v.ntota, 102)];
        const int nsi_i = v.nsi[CK(it, v.nit, 103)];
        const double xi0 = v.x[CK(i, v.ntota, 104)], yi0 = v.y[CK(i, v.ntota, 104)], zi0 = v.z[CK(i, v.ntota, 104)];
        double rix[3], riy[3], riz[3], qi[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const bool ok = a < nsi_i;
            rix[a] = ok ? v.rsx[CK(i + a, v.nmove, 105)] : 0.0;
            riy[a] = ok ? v.rsy[CK(i + a, v.nmove, 105)] : 0.0;
            riz[a] = ok ? v.rsz[CK(i + a, v.nmove, 105)] : 0.0;
            qi[a] = ok ? v.q[CK(i + a, v.ntota, 106)] : 0.0;
        }
        double fix[3] = {0, 0, 0}, fiy[3] = {0, 0, 0}, fiz[3] = {0, 0, 0};
        const int n = v.nbcnt[CK(h, v.nheads, 107)];
        const int* nb = v.nb + (size_t)CK(h, v.nheads, 120) * v.maxnb;
        for (int k = lane; k < n; k += 32) {
            const int j = nb[CK(k, v.maxnb, 108)];
            double xio = minimg(xi0 - v.x[CK(j, v.nmove, 109)], v.lx, v.lxi);
            double yio = minimg(yi0 - v.y[j], v.ly, v.lyi);
            double zio = zi0 - v.z[j];
            if (v.bulk) zio = minimg(zio, v.lz, v.lzi);
            const double rsq = xio * xio + yio * yio + zio * zio;
            if (rsq > v.rcutsq) continue;
            const int jt = v.type[CK(j, v.ntota, 110)];
            const int ijt = CK(v.ijt[CK(it * v.nit + jt, v.nit * v.nit, 111)], v.nijt, 112);
            const int nsi_j = v.nsi[CK(jt, v.nit, 113)];
            const double rsqi = 1.0 / rsq;
            const double rij = sqrt(rsq);
            double fij = 0.0, elj = 0.0;
            const int vk = v.vdw[ijt];
            if (vk == 1) {
                const double r6 = v.sig[ijt] * (rsqi * rsqi * rsqi);
                elj = v.eps[ijt] * r6 * (r6 - 1.0);
                fij = 6.0 * rsqi * v.eps[ijt] * r6 * (2.0 * r6 - 1.0);
            } else if (vk == 2) {
                const double r6 = v.cc[ijt] * (rsqi * rsqi * rsqi);
                const double aux = v.aa[ijt] * exp(-rij * v.rhoi[ijt]);
                elj = aux - r6;
                fij = aux * v.rhoi[ijt] / rij - 6.0 * rsqi * r6;
            }
            double ff;
            const double auxq = v.facq * qi[0] * v.q[CK(j, v.ntota, 114)] / rij;
            const double erfx = ewald_erfc(v.alfa * rij, &ff, v.spii);
            double eqq = erfx * auxq;
            fij = fij + ff * auxq * rsqi;
            double fjx[3], fjy[3], fjz[3];
            fix[0] += xio * fij; fiy[0] += yio * fij; fiz[0] += zio * fij;
            fjx[0] = -xio * fij; fjy[0] = -yio * fij; fjz[0] = -zio * fij;
            double rjx[3], rjy[3], rjz[3], qj[3];
#pragma unroll
            for (int b = 1; b < 3; ++b) {
                fjx[b] = fjy[b] = fjz[b] = 0.0;
                const bool ok = b < nsi_j;
                rjx[b] = ok ? v.rsx[CK(j + b, v.nmove, 115)] : 0.0;
                rjy[b] = ok ? v.rsy[CK(j + b, v.nmove, 115)] : 0.0;
                rjz[b] = ok ? v.rsz[CK(j + b, v.nmove, 115)] : 0.0;
                qj[b] = ok ? v.q[CK(j + b, v.ntota, 116)] : 0.0;
            }
            rjx[0] = v.rsx[CK(j, v.nmove, 117)]; rjy[0] = v.rsy[CK(j, v.nmove, 117)]; rjz[0] = v.rsz[CK(j, v.nmove, 117)]; qj[0] = v.q[CK(j, v.ntota, 117)];
            // remaining site pairs (src/forcem.f90:360-402): (head of i, sites 2.. of j), then
            // (sites 2.. of i, all sites of j)
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (a >= nsi_i) break;
                const double xa = xio + rix[a], ya = yio + riy[a], za = zio + riz[a];
                const double qx = v.facq * qi[a];
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    if (b >= nsi_j) break;
                    if (a == 0 && b == 0) continue;
                    const double xd = xa - rjx[b], yd = ya - rjy[b], zd = za - rjz[b];
                    const double r2 = xd * xd + yd * yd + zd * zd;
                    const double r2i = 1.0 / r2;
                    const double rr = sqrt(r2);
                    const double au = qx * qj[b] / rr;
                    double fq;
                    const double ef = ewald_erfc(v.alfa * rr, &fq, v.spii);
                    eqq += ef * au;
                    const double fs = fq * au * r2i;
                    fix[a] += xd * fs; fiy[a] += yd * fs; fiz[a] += zd * fs;
                    fjx[b] -= xd * fs; fjy[b] -= yd * fs; fjz[b] -= zd * fs;
                }
            }
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                if (b >= nsi_j) break;
                atomicAdd(&v.fx[CK(j + b, v.nmove, 118)], fjx[b]);
                atomicAdd(&v.fy[CK(j + b, v.nmove, 118)], fjy[b]);
                atomicAdd(&v.fz[CK(j + b, v.nmove, 118)], fjz[b]);
            }
            e_add(e, ijt, elj, eqq, s_e, v.nijt);
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (a >= nsi_i) break;
            const double sx = warp_sum(fix[a]), sy = warp_sum(fiy[a]), sz = warp_sum(fiz[a]);
            if (lane == 0) {
                atomicAdd(&v.fx[CK(i + a, v.nmove, 119)], sx);
                atomicAdd(&v.fy[CK(i + a, v.nmove, 119)], sy);
                atomicAdd(&v.fz[CK(i + a, v.nmove, 119)], sz);
            }
        }
    }
    e_final(e, s_e, v.nijt);
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * v.nijt; k += blockDim.x)
        if (s_e[k] != 0.0) atomicAdd(&v.acc[k], s_e[k]);
}

__global__ void __launch_bounds__(kNT) k_wall_fp64(View v) {
    extern __shared__ double s_e[];  // 2 * nijt + 6 (fws x,y,z for sgn -1 / +1)
    for (int k = threadIdx.x; k < 2 * v.nijt + 6; k += blockDim.x) s_e[k] = 0.0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int nwarps = gridDim.x * kWarps;
    // energy sums per wall site type (the last two site types alternate from partner to partner)
    EAcc ew[2];
    const int wt0 = v.nit - 2;
    double ws[6] = {0, 0, 0, 0, 0, 0};  // [sgn<0: x,y,z][sgn>0: x,y,z]
    for (int h = warp; h < v.nheads; h += nwarps) {
        const int i = v.head_atom[h];
        const int it = v.type[i];
        const int nsi_i = v.nsi[it];
        const bool book = (it + 1) <= v.nltype;  // `it <= nltype` on 1-based ids (src/forcem.f90:481)
        const double xi0 = v.x[i], yi0 = v.y[i], zi0 = v.z[i];
        double rix[3], riy[3], riz[3], qi[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const bool ok = a < nsi_i;
            rix[a] = ok ? v.rsx[i + a] : 0.0;
            riy[a] = ok ? v.rsy[i + a] : 0.0;
            riz[a] = ok ? v.rsz[i + a] : 0.0;
            qi[a] = ok ? v.q[i + a] : 0.0;
        }
        double fix[3] = {0, 0, 0}, fiy[3] = {0, 0, 0}, fiz[3] = {0, 0, 0};
        const int n = v.wnbcnt[h];
        const int* nb = v.wnb + (size_t)h * v.maxwnb;
        for (int k = lane; k < n; k += 32) {
            const int j = nb[k];
            const double xi = minimg(xi0 - v.x[j], v.lx, v.lxi);
            const double yi = minimg(yi0 - v.y[j], v.ly, v.lyi);
            double zi = zi0 - v.z[j];
            if (v.bulk) zi = minimg(zi, v.lz, v.lzi);
            const double rsq = xi * xi + yi * yi + zi * zi;
            if (rsq > v.rcutsq) continue;
            const int so = signbit(v.z[j]) ? 0 : 3;
            const int ijt = v.ijt[it * v.nit + v.type[j]];
            double fij = 0.0, elj = 0.0;
            const int vk = v.vdw[ijt];
            if (vk == 1) {
                const double rsqi = 1.0 / rsq;
                const double r6 = v.sig[ijt] * (rsqi * rsqi * rsqi);
                elj = v.eps[ijt] * r6 * (r6 - 1.0);
                fij = 6.0 * rsqi * v.eps[ijt] * r6 * (2.0 * r6 - 1.0);
            } else if (vk == 2) {
                const double rsqi = 1.0 / rsq;
                const double rij = sqrt(rsq);
                const double r6 = v.cc[ijt] * (rsqi * rsqi * rsqi);
                const double aux = v.aa[ijt] * exp(-rij * v.rhoi[ijt]);
                elj = aux - r6;
                fij = aux * v.rhoi[ijt] / rij - 6.0 * rsqi * r6;
            }
            const double qx = v.facq * v.q[j];
            double eqq = 0.0;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (a >= nsi_i) break;
                const double xd = xi + rix[a], yd = yi + riy[a], zd = zi + riz[a];
                const double r2 = xd * xd + yd * yd + zd * zd;
                const double rr = sqrt(r2);
                const double r2i = 1.0 / r2;
                const double au = qx * qi[a] / rr;
                double fq;
                const double ef = ewald_erfc(v.alfa * rr, &fq, v.spii);
                eqq += ef * au;
                fij = fij + fq * au * r2i;
                fix[a] += xd * fij; fiy[a] += yd * fij; fiz[a] += zd * fij;
                if (book) {
                    ws[so] -= xd * fij; ws[so + 1] -= yd * fij; ws[so + 2] -= zd * fij;
                }
                fij = 0.0;
            }
            e_add(ew[min(max(v.type[j] - wt0, 0), 1)], ijt, elj, eqq, s_e, v.nijt);
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (a >= nsi_i) break;
            const double sx = warp_sum(fix[a]), sy = warp_sum(fiy[a]), sz = warp_sum(fiz[a]);
            if (lane == 0) {
                atomicAdd(&v.fx[i + a], sx);
                atomicAdd(&v.fy[i + a], sy);
                atomicAdd(&v.fz[i + a], sz);
            }
        }
    }
    e_final(ew[0], s_e, v.nijt);
    e_final(ew[1], s_e, v.nijt);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const double s = warp_sum(ws[k]);
        if (lane == 0 && s != 0.0) atomicAdd(&s_e[2 * v.nijt + k], s);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * v.nijt; k += blockDim.x)
        if (s_e[k] != 0.0) atomicAdd(&v.acc[k], s_e[k]);
    if (threadIdx.x < 6) {
        // fws layout: [x(-1),x(0),x(1), y(-1),y(0),y(1), z(-1),z(0),z(1)]
        const int comp = threadIdx.x % 3, sg = threadIdx.x / 3;  // sg 0 -> -1, 1 -> +1
        const double s = s_e[2 * v.nijt + threadIdx.x];
        if (s != 0.0) atomicAdd(&v.acc[2 * v.nijt + ACC_FWS + comp * 3 + (sg ? 2 : 0)], s);
    }
}

// fwsz(sign(z0(i))) += fz(i) for surface atoms, right after the head-head loop.
__global__ void k_surf_part(View v) {
    double lo = 0.0, hi = 0.0;
    for (int i = v.nliqa + blockIdx.x * blockDim.x + threadIdx.x; i < v.nmove; i += gridDim.x * blockDim.x) {
        if (signbit(v.z[i])) lo += v.fz[i];
        else hi += v.fz[i];
    }
    block_atomic_sum<kNT>(lo, &v.acc[2 * v.nijt + ACC_FWS + 6 + 0]);
    block_atomic_sum<kNT>(hi, &v.acc[2 * v.nijt + ACC_FWS + 6 + 2]);
}

// Wall long-range tail, src/forcem.f90:509-543.  lr: [9][nit] tables.  Small blocks: the
// per-atom FP64 work is spread over as many SMs as the atom count allows.
constexpr int kLrNT = 64;
__global__ void k_lr_tail(View v, const double* lr) {
    double ulr = 0.0, fw[2] = {0.0, 0.0};
    const int nit = v.nit;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < v.nmove; i += gridDim.x * blockDim.x) {
        const int it = v.type[i];
        if (fabs(v.q[i]) < F32D(0.7)) continue;
        double fz = v.fz[i];
        for (int j = -1; j <= 1; j += 2) {
            double aux = 0.0;
            const double sgn = (double)j;
            const double dw = v.lwh - sgn * v.z[i];
            if (dw < v.rcut) {
                aux = aux + sgn * lr[1 * nit + it];
                ulr += lr[8 * nit + it];
            } else {
                aux = aux + sgn * lr[0 * nit + it];
                ulr += lr[7 * nit + it];
                const double dwa = 1.0 / (dw * dw);
                const double dwa2 = dwa * dwa;
                aux = aux + sgn * (lr[2 * nit + it] * (dwa2 * dwa2 * dwa) - lr[3 * nit + it] * dwa2);
                const double dw3 = dw * dw * dw;
                ulr += (lr[2 * nit + it] / (9.0 * (dw3 * dw3 * dw3)) - lr[3 * nit + it] / (3.0 * dw3));
                const double t = lr[6 * nit + it];
                const double exp2a = lr[4 * nit + it] * exp(-dw / t);
                aux = aux + sgn * ((t + dw) * exp2a - lr[5 * nit + it] * dwa2);
                ulr += (t * (2.0 * t + dw) * exp2a - lr[5 * nit + it] / (3.0 * dw3));
            }
            fz -= aux;
            if (it + 1 <= v.nltype) fw[(j + 1) / 2] += aux;
        }
        v.fz[i] = fz;
    }
    block_atomic_sum<kLrNT>(ulr, &v.acc[2 * v.nijt + ACC_ULR]);
    block_atomic_sum<kLrNT>(fw[0], &v.acc[2 * v.nijt + ACC_FWS + 6 + 0]);
    block_atomic_sum<kLrNT>(fw[1], &v.acc[2 * v.nijt + ACC_FWS + 6 + 2]);
}

int pair_blocks(int nheads) {
    return std::max(1, std::min((nheads + kWarps - 1) / kWarps, 152 * 16));
}

}  // namespace

void pair_forces_fp64(Ctx& c) {
    const View& v = c.v;
    if (v.nheads == 0) return;
    k_pair_fp64<<<pair_blocks(v.nheads), kNT, sizeof(double) * 2 * v.nijt, c.stream>>>(v);
}

void wall_forces_fp64(Ctx& c) {
    const View& v = c.v;
    if (v.nheads == 0 || v.nwall == 0) return;
    k_wall_fp64<<<pair_blocks(v.nheads), kNT, sizeof(double) * (2 * v.nijt + 6), c.stream>>>(v);
}

void surf_partition(Ctx& c) {
    const View& v = c.v;
    if (v.nmove <= v.nliqa) return;
    k_surf_part<<<std::min((v.nmove - v.nliqa + kNT - 1) / kNT, 64), kNT, 0, c.stream>>>(v);
}

void lr_tail(Ctx& c) {
    const View& v = c.v;
    if (c.variant != MDG_SLAB || v.nmove == 0) return;
    k_lr_tail<<<std::min((v.nmove + kLrNT - 1) / kLrNT, 152 * 8), kLrNT, 0, c.stream>>>(v, c.d_lr);
}

}  // namespace mdg
