// pack.cuh - the per-atom records of a mixed-precision force evaluation and the block-level steps
// that close the packing: the slab dipole M_z = sum q z of the moving atoms (src/forcem.f90:924),
// the neighbour-list rebuild decision (src/forcem.f90:245-250: the maximum squared displacement of
// the centres of mass and flexible atoms since the last rebuild) and the energy sums cleared for
// the evaluation.  Used by k_pack (pair_mx.cu) for the drop-in calls and by the predictor of a
// resident step (integrate.cu), which has the new positions in registers.
#pragma once

#include "common.cuh"
#include "ctx.h"

namespace mdg {

constexpr int kPackParts = 152 * 16;  // per-block dipole shares: room for either kernel's grid

// round(t 2^32) mod 2^32 for |t| < 2^19: t + 1.5 2^20 lies in [2^20, 2^21), where the spacing of
// doubles is 2^-32, so the low 32 bits of its significand are the rounded fraction (two FP64
// operations per coordinate; the FP64 pipe is narrow on this part).
__device__ __forceinline__ uint32_t frac32(double t) {
    return (uint32_t)__double_as_longlong(t + 1572864.0);
}

// Records of atom a at (x, y, z): fixed-point x, y (and z when periodic) as fractions of the box
// edge with the site type, z as FP32 hi + lo otherwise, site offset and charge.  Moving atoms also
// get their forces cleared and the reciprocal sum's record.  Returns q z of a moving atom, else 0.
__device__ __forceinline__ double pack_atom(const View& v, const Pk& pk, int a, double x, double y, double z,
                                            double rx, double ry, double rz, bool moving) {
    uint4 p;
    p.x = frac32(x * v.lxi);
    p.y = frac32(y * v.lyi);
    const uint32_t uz = frac32(z * v.lzi);
    if (pk.zper) {
        p.z = uz;
    } else {
        const float zh = (float)z;
        p.z = __float_as_uint(zh);
        pk.zlo[a] = (float)(z - (double)zh);
    }
    p.w = (uint32_t)v.type[a] | (signbit(z) ? 0x80000000u : 0u);
    pk.P[a] = p;
    const double qa = v.q[a];
    float4 q = make_float4(0.f, 0.f, 0.f, (float)qa);
    double mz = 0.0;
    if (moving) {
        q.x = (float)rx;
        q.y = (float)ry;
        q.z = (float)rz;
        pk.F[a] = make_float4(0.f, 0.f, 0.f, 0.f);
        v.fx[a] = 0.0;
        v.fy[a] = 0.0;
        v.fz[a] = 0.0;
        mz = qa * z;
        if (pk.tc) pk.tc[a] = make_uint4(p.x, p.y, uz, __float_as_uint(q.w));
    }
    pk.Q[a] = q;
    return mz;
}

// Every thread of the block: its dipole share to pk.part[blockIdx.x], its maximum displacement
// into the accumulator slot (atomic max).  red: 8 doubles of shared memory.
__device__ __forceinline__ void pack_block(const View& v, const Pk& pk, double mz, double md, double* red) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    mz = warp_sum(mz);
    for (int o = 16; o > 0; o >>= 1) md = fmax(md, __shfl_xor_sync(0xffffffffu, md, o));
    if (l == 0) {
        red[w] = mz;
        atomic_max_nonneg(&v.acc[2 * v.nijt + ACC_MAXD], md);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int k = 0; k < nw; ++k) b += red[k];
        pk.part[blockIdx.x] = b;
    }
    __syncthreads();
}

// Every thread of the block that finished last (after the caller's fence and count): the dipole
// from the shares in block order (deterministic), the rebuild decision, and the energy sums of
// this evaluation cleared (reset_status: the list overflow words too).
__device__ __forceinline__ void pack_close(const View& v, const Pk& pk, int dip, int force, int reset_status,
                                           double* red) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    const int na = 2 * v.nijt + ACC_NSLOT, kmax = 2 * v.nijt + ACC_MAXD, kdip = 2 * v.nijt + ACC_DIPZ;
    __threadfence();
    // loads first (the tail of a kernel: one round trip to L2 instead of one per dependent load)
    double maxd = 0.0;
    int frb = 0;
    if (threadIdx.x == 0) {
        maxd = __ldcg(&v.acc[kmax]);
        frb = __ldcg(&v.status[ST_FORCE_RB]);
    }
    // the shares: several per thread, their loads unrolled ahead of the adds (a loop that adds
    // each before loading the next pays one L2 round trip per share)
    double s = 0.0;
#pragma unroll 16
    for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x) s += __ldcg(&pk.part[b]);
    s = warp_sum(s);
    if (l == 0) red[w] = s;
    __syncthreads();
    for (int k = threadIdx.x; k < na; k += blockDim.x)
        if (k != kmax && k != kdip) v.acc[k] = 0.0;
    if (reset_status && threadIdx.x < 2) v.status[ST_LIST_OVF + threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        double dz = 0.0;
        for (int k = 0; k < nw; ++k) dz += red[k];
        v.acc[kdip] = dip ? dz : 0.0;
        const double aux = fmax(maxd, v.dshsq);
        v.status[ST_REBUILD] = (force || frb || 4.0 * aux > v.skin * v.skin) ? 1 : 0;
        v.status[ST_FORCE_RB] = 0;
        v.acc[kmax] = 0.0;
    }
}

// The same close by one warp of a later kernel (no block barrier, so that another warp can run
// other work at the same time), over the nparts shares of the packing kernel; zero_acc: also clear
// the energy sums (else the packing kernel did).  Every lane of the warp calls it.
__device__ __forceinline__ void pack_close_warp(const View& v, const Pk& pk, int dip, int force, int reset_status,
                                                int nparts, bool zero_acc) {
    const int l = threadIdx.x & 31;
    const int na = 2 * v.nijt + ACC_NSLOT, kmax = 2 * v.nijt + ACC_MAXD, kdip = 2 * v.nijt + ACC_DIPZ;
    double maxd = 0.0;
    int frb = 0;
    if (l == 0) {
        maxd = __ldcg(&v.acc[kmax]);
        frb = __ldcg(&v.status[ST_FORCE_RB]);
    }
    double s = 0.0;
#pragma unroll 16
    for (int b = l; b < nparts; b += 32) s += __ldcg(&pk.part[b]);
    s = warp_sum(s);
    if (zero_acc)
        for (int k = l; k < na; k += 32)
            if (k != kmax && k != kdip) v.acc[k] = 0.0;
    if (reset_status && l < 2) v.status[ST_LIST_OVF + l] = 0;
    if (l == 0) {
        v.acc[kdip] = dip ? s : 0.0;
        const double aux = fmax(maxd, v.dshsq);
        v.status[ST_REBUILD] = (force || frb || 4.0 * aux > v.skin * v.skin) ? 1 : 0;
        v.status[ST_FORCE_RB] = 0;
        v.acc[kmax] = 0.0;
    }
}

}  // namespace mdg
