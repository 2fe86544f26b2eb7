// epilogue.cu - the end of force_get.
//
//   k_dipz / k_dipforce   EW3DC slab correction (src/forcem.f90:923-928): M_z = sum q z over
//                         moving atoms, fz += 2 crf facq M_z q with crf = -2 pi/(Lx Ly Lz)
//   k_angles              harmonic bends of surface molecules (force_intra, src/forcem.f90:565-652)
//   k_force_sum           serial force_sum (src/forcem_3d.f90:1031-1062): forces of flexible atoms,
//                         centre-of-mass forces and torques of rigid molecules, sum of all forces,
//                         and rsx(1:3) left holding the last rigid molecule's offsets (:1056-1058)
#include <algorithm>

#include "common.cuh"
#include "ctx.h"
#include "merge.cuh"

namespace mdg {

namespace {

constexpr int kNT = 64;

__global__ void k_dipz(View v) {
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < v.nmove; i += gridDim.x * blockDim.x)
        s += v.q[i] * v.z[i];
    block_atomic_sum<kNT>(s, &v.acc[2 * v.nijt + ACC_DIPZ]);
}

__global__ void k_dipforce(View v, double crf0) {
    const double dipz = v.acc[2 * v.nijt + ACC_DIPZ];
    const double crf = 2.0 * crf0 * v.facq * dipz;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < v.nmove; i += gridDim.x * blockDim.x)
        v.fz[i] += crf * v.q[i];
}

// ang: per term (i, j, k, slot); kt/th per slot.  Forces on j and k only, as the reference.
__global__ void k_angles(View v, int nterm, const int4* ang, const double* kt, const double* th) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nterm) return;
    const int4 a = ang[t];
    const int i = a.x, j = a.y, k = a.z;
    const double ax = minimg(v.x[k] - v.x[j], v.lx, v.lxi);
    const double ay = minimg(v.y[k] - v.y[j], v.ly, v.lyi);
    double az = v.z[k] - v.z[j];
    const double bx = minimg(v.x[j] - v.x[i], v.lx, v.lxi);
    const double by = minimg(v.y[j] - v.y[i], v.ly, v.lyi);
    double bz = v.z[j] - v.z[i];
    if (v.bulk) {
        az = minimg(az, v.lz, v.lzi);
        bz = minimg(bz, v.lz, v.lzi);
    }
    const double ai = 1.0 / sqrt(ax * ax + ay * ay + az * az);
    const double bi = 1.0 / sqrt(bx * bx + by * by + bz * bz);
    const double ab = ax * bx + ay * by + az * bz;
    const double cang = -ab * ai * bi;
    double fij = kt[a.w] * (acos(cang) - th[a.w]) / sqrt(1.0 - cang * cang);
    fij = fij * ai * bi;
    const double bb = ab * bi * bi, aa = ab * ai * ai;
    double tmp = aa * ax - bx;
    if (k < v.nmove) atomicAdd(&v.fx[k], fij * tmp);
    if (j < v.nmove) atomicAdd(&v.fx[j], fij * (bb * bx - ax - tmp));
    tmp = aa * ay - by;
    if (k < v.nmove) atomicAdd(&v.fy[k], fij * tmp);
    if (j < v.nmove) atomicAdd(&v.fy[j], fij * (bb * by - ay - tmp));
    tmp = aa * az - bz;
    if (k < v.nmove) atomicAdd(&v.fz[k], fij * tmp);
    if (j < v.nmove) atomicAdd(&v.fz[j], fij * (bb * bz - az - tmp));
}

// ft: 3 x (nmove - nriga); fc, tq: 3 x nrig (component-major).
__global__ void k_force_sum(View v, double* ft, double* fc, double* tq) {
    double sx = 0.0, sy = 0.0, sz = 0.0;
    const int nflex = v.nmove - v.nriga;
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < v.nmove; i += stride) {
        sx += v.fx[i];
        sy += v.fy[i];
        sz += v.fz[i];
        if (i >= v.nriga) {
            const int k = i - v.nriga;
            ft[CK(k, nflex, 301)] = v.fx[i];
            ft[CK(nflex + k, 3 * nflex, 302)] = v.fy[i];
            ft[CK(2 * nflex + k, 3 * nflex, 303)] = v.fz[i];
        }
    }
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < v.nrig; m += stride) {
        const int j = CK(3 * m, v.nmove - 2, 304);
        const double f0x = v.fx[j], f1x = v.fx[j + 1], f2x = v.fx[j + 2];
        const double f0y = v.fy[j], f1y = v.fy[j + 1], f2y = v.fy[j + 2];
        const double f0z = v.fz[j], f1z = v.fz[j + 1], f2z = v.fz[j + 2];
        fc[m] = f0x + f1x + f2x;
        fc[v.nrig + m] = f0y + f1y + f2y;
        fc[2 * v.nrig + m] = f0z + f1z + f2z;
        const double cx = v.cx[m], cy = v.cy[m], cz = v.cz[m];
        const double r0x = v.x[j] - cx, r1x = v.x[j + 1] - cx, r2x = v.x[j + 2] - cx;
        const double r0y = v.y[j] - cy, r1y = v.y[j + 1] - cy, r2y = v.y[j + 2] - cy;
        const double r0z = v.z[j] - cz, r1z = v.z[j + 1] - cz, r2z = v.z[j + 2] - cz;
        tq[m] = (r0y * f0z - r0z * f0y) + (r1y * f1z - r1z * f1y) + (r2y * f2z - r2z * f2y);
        tq[v.nrig + m] = (r0z * f0x - r0x * f0z) + (r1z * f1x - r1x * f1z) + (r2z * f2x - r2x * f2z);
        tq[2 * v.nrig + m] = (r0x * f0y - r0y * f0x) + (r1x * f1y - r1y * f1x) + (r2x * f2y - r2y * f2x);
        if (m == v.nrig - 1) {
            v.rsx[0] = r0x; v.rsx[1] = r1x; v.rsx[2] = r2x;
            v.rsy[0] = r0y; v.rsy[1] = r1y; v.rsy[2] = r2y;
            v.rsz[0] = r0z; v.rsz[1] = r1z; v.rsz[2] = r2z;
        }
    }
    block_atomic_sum<kNT>(sx, &v.acc[2 * v.nijt + ACC_FWS0 + 0]);
    block_atomic_sum<kNT>(sy, &v.acc[2 * v.nijt + ACC_FWS0 + 1]);
    block_atomic_sum<kNT>(sz, &v.acc[2 * v.nijt + ACC_FWS0 + 2]);
}

// For systems without bend angles (and no histograms), the final merge of the mixed form fused
// with force_sum: per rigid molecule or flexible atom (merge.cuh), then the sum of all forces.
__global__ void k_merge_sum(View v, MergeArgs A) {
    const MergeArgs M = merge_begin(v, A);
    double sx = 0.0, sy = 0.0, sz = 0.0;
    const int nu = v.nrig + (v.nmove - v.nriga);
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += gridDim.x * blockDim.x) {
        if (u < v.nrig) merge_rigid(v, M, u, sx, sy, sz);
        else merge_flex(v, M, u - v.nrig, sx, sy, sz);
    }
    block_atomic_sum<kNT>(sx, &v.acc[2 * v.nijt + ACC_FWS0 + 0]);
    block_atomic_sum<kNT>(sy, &v.acc[2 * v.nijt + ACC_FWS0 + 1]);
    block_atomic_sum<kNT>(sz, &v.acc[2 * v.nijt + ACC_FWS0 + 2]);
}

}  // namespace

MergeArgs merge_args(const Ctx& c, const double* frc) {
    const View& v = c.v;
    MergeArgs A{};
    A.pk = c.pk;
    A.frc = frc;
    A.crf0 = c.variant == MDG_SLAB ? -2.0 * (double)3.1415926535898f * v.lzi * v.lxi * v.lyi : 0.0;
    A.ft = c.d_ft;
    A.fc = c.d_fc;
    A.tq = c.d_tq;
    return A;
}

void merge_force_sum(Ctx& c, const double* frc) {
    const View& v = c.v;
    const int n = std::max(v.nrig + (v.nmove - v.nriga), 1);
    const int nb = std::max(1, std::min((n + kNT - 1) / kNT, 152 * 8));
    k_merge_sum<<<nb, kNT, 0, c.stream>>>(v, merge_args(c, frc));
}

void dipole_correction(Ctx& c) {
    const View& v = c.v;
    if (c.variant != MDG_SLAB || v.nmove == 0) return;
    const double pi_r = (double)3.1415926535898f;
    const double crf0 = -2.0 * pi_r * v.lzi * v.lxi * v.lyi;
    const int nb = std::min((v.nmove + kNT - 1) / kNT, 152 * 8);
    k_dipz<<<nb, kNT, 0, c.stream>>>(v);
    k_dipforce<<<nb, kNT, 0, c.stream>>>(v, crf0);
}

void angle_forces(Ctx& c) {
    if (c.nang_terms == 0) return;
    k_angles<<<(c.nang_terms + 127) / 128, 128, 0, c.stream>>>(c.v, c.nang_terms,
                                                               reinterpret_cast<const int4*>(c.d_ang),
                                                               c.d_ang_kt, c.d_ang_th);
}

void force_sum(Ctx& c, double* d_ft, double* d_fc, double* d_tq) {
    const View& v = c.v;
    const int n = std::max(v.nmove, v.nrig);
    const int nb = std::max(1, std::min((n + kNT - 1) / kNT, 152 * 8));
    k_force_sum<<<nb, kNT, 0, c.stream>>>(v, d_ft, d_fc, d_tq);
}

}  // namespace mdg
