// merge.cuh - the last step of a mixed-precision force evaluation for one unit (a rigid molecule
// or a flexible atom): the FP32 accumulator F, the reciprocal forces frc and the slab dipole term
// join the FP64 site forces, which then give the unit's force_sum results (src/forcem_3d.f90:
// 1031-1062): ft of a flexible atom; centre-of-mass force and torque of a rigid molecule, and
// rsx(1:3) left holding the last molecule's offsets (:1056-1058).  Shared by k_merge_sum
// (epilogue.cu) and the corrector that fuses it (integrate.cu).
#pragma once

#include "common.cuh"
#include "ctx.h"

namespace mdg {

struct MergeArgs {
    Pk pk;
    const double* frc;  // reciprocal forces 3 x nmove, or nullptr
    double crf0;        // -2 pi / (Lx Ly Lz) for the slab dipole term, 0 without it
    double crf;         // 2 crf0 facq M_z, the dipole force per unit charge (merge_begin)
    int dip;            // slab dipole term on
    double* ft;         // 3 x (nmove - nriga)
    double* fc;         // 3 x nrig
    double* tq;         // 3 x nrig
};

// the arguments for this context's arrays and variant (epilogue.cu)
MergeArgs merge_args(const Ctx& c, const double* frc);

// a kernel's copy of the arguments, with the dipole force of this evaluation's M_z
__device__ __forceinline__ MergeArgs merge_begin(const View& v, const MergeArgs& A) {
    MergeArgs M = A;
    M.dip = A.crf0 != 0.0;
    M.crf = M.dip ? 2.0 * A.crf0 * v.facq * v.acc[2 * v.nijt + ACC_DIPZ] : 0.0;
    return M;
}

// FP64 force of atom a after the merge (also stored, and F cleared for the next evaluation)
__device__ __forceinline__ void merged_force(const View& v, const MergeArgs& M, int a, double& gx, double& gy,
                                             double& gz) {
    const float4 f = M.pk.F[a];
    double hx = (double)f.x, hy = (double)f.y, hz = (double)f.z;
    if (M.frc) {
        hx += M.frc[a];
        hy += M.frc[v.nmove + a];
        hz += M.frc[2 * v.nmove + a];
    }
    if (M.dip) hz += M.crf * v.q[a];
    gx = v.fx[a] + hx;
    gy = v.fy[a] + hy;
    gz = v.fz[a] + hz;
    v.fx[a] = gx;
    v.fy[a] = gy;
    v.fz[a] = gz;
    M.pk.F[a] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// rigid molecule m: fc, tq (and the stale offsets); adds its force to s
__device__ __forceinline__ void merge_rigid(const View& v, const MergeArgs& M, int m, double& sx, double& sy,
                                            double& sz) {
    const int j = 3 * m;
    double f0x, f0y, f0z, f1x, f1y, f1z, f2x, f2y, f2z;
    merged_force(v, M, j, f0x, f0y, f0z);
    merged_force(v, M, j + 1, f1x, f1y, f1z);
    merged_force(v, M, j + 2, f2x, f2y, f2z);
    sx += f0x + f1x + f2x;
    sy += f0y + f1y + f2y;
    sz += f0z + f1z + f2z;
    M.fc[m] = f0x + f1x + f2x;
    M.fc[v.nrig + m] = f0y + f1y + f2y;
    M.fc[2 * v.nrig + m] = f0z + f1z + f2z;
    const double cx = v.cx[m], cy = v.cy[m], cz = v.cz[m];
    const double r0x = v.x[j] - cx, r1x = v.x[j + 1] - cx, r2x = v.x[j + 2] - cx;
    const double r0y = v.y[j] - cy, r1y = v.y[j + 1] - cy, r2y = v.y[j + 2] - cy;
    const double r0z = v.z[j] - cz, r1z = v.z[j + 1] - cz, r2z = v.z[j + 2] - cz;
    M.tq[m] = (r0y * f0z - r0z * f0y) + (r1y * f1z - r1z * f1y) + (r2y * f2z - r2z * f2y);
    M.tq[v.nrig + m] = (r0z * f0x - r0x * f0z) + (r1z * f1x - r1x * f1z) + (r2z * f2x - r2x * f2z);
    M.tq[2 * v.nrig + m] = (r0x * f0y - r0y * f0x) + (r1x * f1y - r1y * f1x) + (r2x * f2y - r2y * f2x);
    if (m == v.nrig - 1) {
        v.rsx[0] = r0x; v.rsx[1] = r1x; v.rsx[2] = r2x;
        v.rsy[0] = r0y; v.rsy[1] = r1y; v.rsy[2] = r2y;
        v.rsz[0] = r0z; v.rsz[1] = r1z; v.rsz[2] = r2z;
    }
}

// The same on a pair of lanes (mask: the lanes of the pairs on rigid molecules): role 0 merges
// sites 0 and 1, role 1 site 2; role 0 receives site 2's force and torque term and forms fc and tq
// (returned, and stored) in the order of merge_rigid.
__device__ __forceinline__ void merge_rigid_pair(const View& v, const MergeArgs& M, int m, int role, unsigned mask,
                                                 double& sx, double& sy, double& sz, double* fc, double* tq) {
    const int j = 3 * m;
    const double cx = v.cx[m], cy = v.cy[m], cz = v.cz[m];
    double px, py, pz, tx, ty, tz;
    double r0x, r0y, r0z, r1x = 0.0, r1y = 0.0, r1z = 0.0;
    if (role == 0) {
        double f0x, f0y, f0z, f1x, f1y, f1z;
        merged_force(v, M, j, f0x, f0y, f0z);
        merged_force(v, M, j + 1, f1x, f1y, f1z);
        r0x = v.x[j] - cx;
        r1x = v.x[j + 1] - cx;
        r0y = v.y[j] - cy;
        r1y = v.y[j + 1] - cy;
        r0z = v.z[j] - cz;
        r1z = v.z[j + 1] - cz;
        px = f0x + f1x;
        py = f0y + f1y;
        pz = f0z + f1z;
        tx = (r0y * f0z - r0z * f0y) + (r1y * f1z - r1z * f1y);
        ty = (r0z * f0x - r0x * f0z) + (r1z * f1x - r1x * f1z);
        tz = (r0x * f0y - r0y * f0x) + (r1x * f1y - r1y * f1x);
    } else {
        double f2x, f2y, f2z;
        merged_force(v, M, j + 2, f2x, f2y, f2z);
        r0x = v.x[j + 2] - cx;  // site 2's offset in slot 0
        r0y = v.y[j + 2] - cy;
        r0z = v.z[j + 2] - cz;
        px = f2x;
        py = f2y;
        pz = f2z;
        tx = (r0y * f2z - r0z * f2y);
        ty = (r0z * f2x - r0x * f2z);
        tz = (r0x * f2y - r0y * f2x);
    }
    const double qx = __shfl_xor_sync(mask, px, 1), qy = __shfl_xor_sync(mask, py, 1),
                 qz = __shfl_xor_sync(mask, pz, 1);
    const double ux = __shfl_xor_sync(mask, tx, 1), uy = __shfl_xor_sync(mask, ty, 1),
                 uz = __shfl_xor_sync(mask, tz, 1);
    if (role == 0) {
        fc[0] = px + qx;
        fc[1] = py + qy;
        fc[2] = pz + qz;
        tq[0] = tx + ux;
        tq[1] = ty + uy;
        tq[2] = tz + uz;
        sx += fc[0];
        sy += fc[1];
        sz += fc[2];
        M.fc[m] = fc[0];
        M.fc[v.nrig + m] = fc[1];
        M.fc[2 * v.nrig + m] = fc[2];
        M.tq[m] = tq[0];
        M.tq[v.nrig + m] = tq[1];
        M.tq[2 * v.nrig + m] = tq[2];
    }
    if (m == v.nrig - 1) {
        if (role == 0) {
            v.rsx[0] = r0x; v.rsx[1] = r1x;
            v.rsy[0] = r0y; v.rsy[1] = r1y;
            v.rsz[0] = r0z; v.rsz[1] = r1z;
        } else {
            v.rsx[2] = r0x;
            v.rsy[2] = r0y;
            v.rsz[2] = r0z;
        }
    }
}

// flexible atom k (atom nriga + k): ft; adds its force to s
__device__ __forceinline__ void merge_flex(const View& v, const MergeArgs& M, int k, double& sx, double& sy,
                                           double& sz) {
    const int nflex = v.nmove - v.nriga;
    double gx, gy, gz;
    merged_force(v, M, v.nriga + k, gx, gy, gz);
    sx += gx;
    sy += gy;
    sz += gz;
    M.ft[k] = gx;
    M.ft[nflex + k] = gy;
    M.ft[2 * nflex + k] = gz;
}

}  // namespace mdg
