// common.cuh - device helpers shared by the md_sim GB300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

// Single-precision Fortran literals promoted to real*8 (src/global.f90:18-24, src/forcem.f90:11-13).
#define F32D(x) ((double)(x##f))

namespace mdg {

constexpr double kA1 = F32D(0.254829592), kA2 = F32D(-0.284496736), kA3 = F32D(1.421413741);
constexpr double kA4 = F32D(-1.453152027), kA5 = F32D(1.061405429), kP = F32D(0.3275911);

// status words written by kernels, read by the host after a phase
enum StatusWord {
    ST_LIST_OVF = 0,   // head-head list overflow (count stored)
    ST_WLIST_OVF = 1,  // head-wall list overflow
    ST_SHAKE_MAXIT = 2,
    ST_SHAKE_RPTOL = 3,  // 1 + first failing constraint (molecule * 8 + is)
    ST_FORCE_RB = 4,   // host request: rebuild the list at the next trigger
    ST_REBUILD = 5,    // 1 when the current step rebuilt the list
    ST_SWEEPS = 6,     // SHAKE sweeps of the last call
    ST_OOB = 7,        // debug builds: tag of the first out-of-range index seen
    ST_TC_TIMEOUT = 8, // a tensor-core phase gave up waiting on an mbarrier (tag of the wait)
    ST_PACK_DONE = 9,  // blocks of the packing kernel finished (its last block resets it)
    ST_NWORDS = 12
};

// Debug builds (-DMDG_DEBUG_BOUNDS) check indices on the force path: an index outside [0, n)
// records its site tag in status[ST_OOB] and is redirected to element 0, so the kernel reports
// instead of faulting.  Release builds compile the check away.
#ifdef MDG_DEBUG_BOUNDS
#define CK(i, n, tag) \
    (((unsigned)(i) < (unsigned)(n)) ? (int)(i) : (atomicCAS(&v.status[ST_OOB], 0, (tag)), 0))
#else
#define CK(i, n, tag) (i)
#endif

// Minimum image with the reference's rounding, no multiply-add contraction:
// d - l*anint(d*li)   (src/nnlist.f90:125, src/forcem.f90:293).  anint = round half away.
__device__ __forceinline__ double minimg(double d, double l, double li) {
    return __dsub_rn(d, __dmul_rn(l, round(__dmul_rn(d, li))));
}

// x*x + y*y + z*z evaluated as ((x*x + y*y) + z*z) with separately rounded products.
__device__ __forceinline__ double dist2_exact(double x, double y, double z) {
    return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum into *dst with one atomic per block; all threads must call.  Blocks smaller than
// a warp (used to spread FP64-heavy per-molecule work over more SMs) reduce within their lanes.
template <int NT>
__device__ __forceinline__ void block_atomic_sum(double v, double* dst) {
    if constexpr (NT <= 32) {
        constexpr unsigned mask = NT == 32 ? 0xffffffffu : (1u << (NT & 31)) - 1u;
#pragma unroll
        for (int o = NT / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
        if (threadIdx.x == 0) atomicAdd(dst, v);
        return;
    }
    __shared__ double red[NT >= 32 ? NT / 32 : 1];
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        double s = (l < NT / 32) ? red[l] : 0.0;
        s = warp_sum(s);
        if (l == 0) atomicAdd(dst, s);
    }
}

__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
    // non-negative doubles order like their bit patterns
    atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

// The dynamic shared memory limit of a kernel is a property of the function, shared by every
// context of the process: raise it to the device's opt-in maximum instead of one context's need,
// so that a context created later with smaller tiles cannot lower it under an earlier one.
// The kernel's static shared memory counts against the same limit.
template <typename F>
inline cudaError_t allow_max_smem(F* f) {
    int dev = 0, mx = 0;
    cudaGetDevice(&dev);
    cudaError_t e = cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, f);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, mx - (int)fa.sharedSizeBytes);
}

}  // namespace mdg
