// pair_mx.cu - mixed-precision real-space forces: the terms of force_real (src/forcem.f90:233-552)
// in FP32 arithmetic with no FP64 work inside the pair loops.
//
// Each force evaluation first packs per-atom records (k_pack):
//   P[a]   uint4  x and y (and z when z is periodic for the forces) as 32-bit fixed-point
//                 fractions of the box edge, so the wrapped integer difference of two records IS
//                 the minimum-image vector (src/forcem.f90:296-300, anint image) to 2^-32 of the
//                 edge; a non-periodic z is the FP32 value z_hi (remainder in zlo[a]); w = site
//                 type, bit 31 = sign of z (which wall a wall atom belongs to).
//   Q[a]   float4 site offset rs(a) and charge q(a)
//   F[a]   float4 j-side force accumulator, zeroed here
//   tc[a]  uint4  fixed-point fractions of x, y, z and the charge, for the tensor-core reciprocal
//                 sum of the same evaluation (recip_tc.cu)
// k_pair_mx walks the same per-head half lists as the FP64 kernel (one warp per head): i-side
// site forces in FP32 sums per lane (a lane holds ~n/32 partners), warp-reduced once per head;
// j-side site forces per pair; both leave as one vector FP32 reduction (red.global.add.v4.f32)
// per site into F, which k_merge_f adds into the FP64 forces (and clears) after the loops.
// Energies per lane are compensated FP32 sums.  k_wall_mx does the head-wall loop
// (src/forcem.f90:418-498) the same way over (head, segment) work items, with the wall reaction
// sums of each item added into FP64 per lane.  The pair loops issue no FP64 instructions (the
// FP64 pipe of GB300 is narrow).  k_pair_mx_batch and k_wall_mx_batch run the same loop bodies
// over the heads of many systems at once (replica batches), one persistent launch each.
#include <algorithm>

#include "common.cuh"
#include "ctx.h"
#include "pack.cuh"

namespace mdg {

namespace {

constexpr int kWarps = 8;
constexpr int kNT = kWarps * 32;
constexpr int kWSeg = 64;  // wall partners per work item of the head-wall loop
constexpr int kPackBlocks = 152 * 8;  // most blocks of the packing kernel
static_assert(kPackBlocks <= kPackParts, "dipole shares");
constexpr float kPf = (float)kP, kA1f = (float)kA1, kA2f = (float)kA2, kA3f = (float)kA3, kA4f = (float)kA4,
                kA5f = (float)kA5;

struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

__device__ __forceinline__ float warp_sumf(float x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// Energies of the current head type pair; flushed to shared FP64 sums when the pair type changes.
struct EAcc {
    int ijt = -1;
    Kahan lj, qq;
};

__device__ __forceinline__ void e_flush(EAcc& e, double* s_e, int nijt) {
    if (e.ijt >= 0) {
        const double a = e.lj.value(), b = e.qq.value();
        if (a != 0.0) atomicAdd(&s_e[e.ijt], a);
        if (b != 0.0) atomicAdd(&s_e[nijt + e.ijt], b);
    }
    e.lj = Kahan();
    e.qq = Kahan();
}

// End of the loops: lanes holding the warp's (largest) pair type reduce with shuffles in FP64 (a
// warp's total grows with the heads it took, and an FP32 reduction of it would round at that
// size), one shared atomic per warp; lanes left with another type (mixed-type systems) flush one
// by one.
__device__ __forceinline__ void e_final(EAcc& e, double* s_e, int nijt) {
    const int ij0 = __reduce_max_sync(0xffffffffu, e.ijt);
    if (ij0 < 0) return;
    const bool mine = e.ijt == ij0;
    const double lj = warp_sum(mine ? e.lj.value() : 0.0);
    const double qq = warp_sum(mine ? e.qq.value() : 0.0);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&s_e[ij0], lj);
        atomicAdd(&s_e[nijt + ij0], qq);
    }
    if (!mine) e_flush(e, s_e, nijt);
}

__device__ __forceinline__ void e_add(EAcc& e, int ijt, float lj, float qq, double* s_e, int nijt) {
    if (ijt != e.ijt) {
        e_flush(e, s_e, nijt);
        e.ijt = ijt;
    }
    e.lj.add(lj);
    e.qq.add(qq);
}

// Abramowitz-Stegun 7.1.26 erfc(alpha r) and the Ewald force factor (src/forcem.f90:334-340).
__device__ __forceinline__ float erfc_as(float alfar, float* ff, float spii) {
    const float t = __fdividef(1.0f, 1.0f + kPf * alfar);
    const float exp2a = __expf(-alfar * alfar);
    const float erfx = ((((kA5f * t + kA4f) * t + kA3f) * t + kA2f) * t + kA1f) * t * exp2a;
    *ff = spii * alfar * exp2a + erfx;
    return erfx;
}

__device__ __forceinline__ void red_v4(float4* p, float a, float b, float c) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c), "f"(0.f)
                 : "memory");
}

// Records of every atom for this evaluation (pack.cuh); also clears the FP64 forces, sums the slab
// dipole, takes the neighbour-list rebuild decision and clears the energy sums (its last block).
// defer_close: no last-block tail; block 0 clears the energy sums (all but the displacement
// maximum) and the overflow words first, and k_pack_close closes the packing on another stream
// while the reciprocal sum starts.
__global__ void k_pack(View v, Pk pk, int dip, int force, int reset_status, int defer_close) {
    __shared__ double red[8];
    __shared__ bool last;
    double mz = 0.0, md = 0.0;
    if (pk.cmax && blockIdx.x == 0 && threadIdx.x == 0) *pk.cmax = 0.f;
    if (defer_close && blockIdx.x == 0) {
        const int na = 2 * v.nijt + ACC_NSLOT, kmax = 2 * v.nijt + ACC_MAXD;
        for (int k = threadIdx.x; k < na; k += blockDim.x)
            if (k != kmax) v.acc[k] = 0.0;
        if (reset_status && threadIdx.x < 2) v.status[ST_LIST_OVF + threadIdx.x] = 0;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < v.nrig + (v.nmove - v.nriga);
         i += gridDim.x * blockDim.x) {
        double a, b, c;
        if (i < v.nrig) {
            a = v.ocx[i] - v.cx[i];
            b = v.ocy[i] - v.cy[i];
            c = v.ocz[i] - v.cz[i];
        } else {
            const int k = i - v.nrig, at = k + v.nriga;
            a = v.ox[k] - v.x[at];
            b = v.oy[k] - v.y[at];
            c = v.oz[k] - v.z[at];
        }
        md = fmax(md, a * a + b * b + c * c);
    }
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < v.ntota; a += gridDim.x * blockDim.x) {
        const bool mv = a < v.nmove;
        mz += pack_atom(v, pk, a, v.x[a], v.y[a], v.z[a], mv ? v.rsx[a] : 0.0, mv ? v.rsy[a] : 0.0,
                        mv ? v.rsz[a] : 0.0, mv);
    }
    pack_block(v, pk, mz, md, red);
    if (defer_close) return;
    __threadfence();
    if (threadIdx.x == 0) last = atomicAdd(&v.status[ST_PACK_DONE], 1) == (int)gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    pack_close(v, pk, dip, force, reset_status, red);
    if (threadIdx.x == 0) v.status[ST_PACK_DONE] = 0;
}

// Pair-type tables in shared memory: per ijt {kind, sig, eps, aa, rhoi, cc}, ijt[it*nit+jt], nsi[it].
struct Tables {
    float* par;
    int* ijt;
    int* nsi;
};

__device__ __forceinline__ Tables load_tables(const View& v, const Pk& pk, double* s_e, int nextra) {
    Tables t;
    t.par = reinterpret_cast<float*>(s_e + 2 * v.nijt + nextra);
    t.ijt = reinterpret_cast<int*>(t.par + 6 * v.nijt);
    t.nsi = t.ijt + v.nit * v.nit;
    for (int k = threadIdx.x; k < 2 * v.nijt + nextra; k += blockDim.x) s_e[k] = 0.0;
    for (int k = threadIdx.x; k < 6 * v.nijt; k += blockDim.x) t.par[k] = pk.par[k];
    for (int k = threadIdx.x; k < v.nit * v.nit; k += blockDim.x) t.ijt[k] = v.ijt[k];
    for (int k = threadIdx.x; k < v.nit; k += blockDim.x) t.nsi[k] = v.nsi[k];
    __syncthreads();
    return t;
}

// Head-head (or head-wall) separation from packed records.
template <int ZPER>
__device__ __forceinline__ void head_vec(const uint4& pi, float zli, const uint4& pj, const Pk& pk, int j, float& dx,
                                         float& dy, float& dz) {
    dx = __int2float_rn((int)(pi.x - pj.x)) * pk.sx;
    dy = __int2float_rn((int)(pi.y - pj.y)) * pk.sy;
    if (ZPER) dz = __int2float_rn((int)(pi.z - pj.z)) * pk.sz;
    else dz = (__uint_as_float(pi.z) - __uint_as_float(pj.z)) + (zli - pk.zlo[j]);
}

// vdW between heads (src/forcem.f90:303-327): returns the energy, adds f/r to *fij.
__device__ __forceinline__ float vdw_term(const float* par, float rsqi, float rinv, float rij, float* fij) {
    const int vk = __float_as_int(par[0]);
    if (vk == 1) {
        const float r6 = par[1] * (rsqi * rsqi * rsqi);
        const float ep = par[2];
        *fij = 6.0f * rsqi * ep * r6 * (2.0f * r6 - 1.0f);
        return ep * r6 * (r6 - 1.0f);
    }
    if (vk == 2) {
        const float r6 = par[5] * (rsqi * rsqi * rsqi);
        const float rh = par[4];
        const float aux = par[3] * __expf(-rij * rh);
        *fij = aux * rh * rinv - 6.0f * rsqi * r6;
        return aux - r6;
    }
    *fij = 0.f;
    return 0.f;
}

// The head-head loop of one warp over the heads h0, h0 + hs, ... below v.nheads.
template <int ZPER>
__device__ __forceinline__ void pair_heads(const View& v, const Pk& pk, const Tables& T, int h0, int hs, EAcc& e,
                                           double* s_e) {
    const int lane = threadIdx.x & 31;
    const float alfa = pk.alfa, spii = pk.spii, facq = pk.facq, rcutsq = pk.rcutsq;
    for (int h = h0; h < v.nheads; h += hs) {
        const int i = v.head_atom[h];
        const uint4 pi = pk.P[i];
        const int it = (int)(pi.w & 0x7fffffffu);
        const int nsi_i = T.nsi[it];
        const float zli = ZPER ? 0.f : pk.zlo[i];
        float4 si[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) si[a] = a < nsi_i ? pk.Q[i + a] : make_float4(0.f, 0.f, 0.f, 0.f);
        // i-side sums: a lane holds about n / 32 partners of the head, few enough for plain FP32
        float fix[3] = {0, 0, 0}, fiy[3] = {0, 0, 0}, fiz[3] = {0, 0, 0};
        const int n = v.nbcnt[h];
        const int* nb = v.nb + (size_t)h * v.maxnb;
        // software pipeline over the lane's partners: the record of the next partner and the
        // index of the one after are loaded while this one is computed (one warp per head and
        // one block per SM leave few warps to hide the dependent gathers otherwise)
        int j1 = lane < n ? nb[lane] : 0;
        int j2 = lane + 32 < n ? nb[lane + 32] : 0;
        uint4 p1 = lane < n ? pk.P[j1] : make_uint4(0u, 0u, 0u, 0u);
        for (int k = lane; k < n; k += 32) {
            const int j = j1;
            const uint4 pj = p1;
            j1 = j2;
            if (k + 32 < n) p1 = pk.P[j1];
            if (k + 64 < n) j2 = nb[k + 64];
            const int jt = (int)(pj.w & 0x7fffffffu);
            const int nsi_j = T.nsi[jt];
            float4 sj[3];  // the partner's sites, requested before the distance test
#pragma unroll
            for (int b = 0; b < 3; ++b) sj[b] = b < nsi_j ? pk.Q[j + b] : make_float4(0.f, 0.f, 0.f, 0.f);
            float xio, yio, zio;
            head_vec<ZPER>(pi, zli, pj, pk, j, xio, yio, zio);
            const float rsq = xio * xio + yio * yio + zio * zio;
            if (rsq > rcutsq) continue;
            const int ijt = T.ijt[it * v.nit + jt];
            const float rinv = rsqrtf(rsq);
            const float rsqi = rinv * rinv;
            const float rij = rsq * rinv;
            float fij;
            const float elj = vdw_term(T.par + 6 * ijt, rsqi, rinv, rij, &fij);
            float ff;
            const float auxq = facq * si[0].w * sj[0].w * rinv;
            float eqq = erfc_as(alfa * rij, &ff, spii) * auxq;
            fij = fij + ff * auxq * rsqi;
            float fjx[3], fjy[3], fjz[3];
            fix[0] = fmaf(xio, fij, fix[0]); fiy[0] = fmaf(yio, fij, fiy[0]); fiz[0] = fmaf(zio, fij, fiz[0]);
            fjx[0] = -xio * fij; fjy[0] = -yio * fij; fjz[0] = -zio * fij;
#pragma unroll
            for (int b = 1; b < 3; ++b) fjx[b] = fjy[b] = fjz[b] = 0.f;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (a >= nsi_i) break;
                const float xa = xio + si[a].x, ya = yio + si[a].y, za = zio + si[a].z;
                const float qx = facq * si[a].w;
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    if (b >= nsi_j) break;
                    if (a == 0 && b == 0) continue;
                    const float xd = xa - sj[b].x, yd = ya - sj[b].y, zd = za - sj[b].z;
                    const float r2 = xd * xd + yd * yd + zd * zd;
                    const float ri = rsqrtf(r2);
                    const float rr = r2 * ri;
                    const float au = qx * sj[b].w * ri;
                    float fq;
                    eqq += erfc_as(alfa * rr, &fq, spii) * au;
                    const float fs = fq * au * (ri * ri);
                    fix[a] = fmaf(xd, fs, fix[a]); fiy[a] = fmaf(yd, fs, fiy[a]); fiz[a] = fmaf(zd, fs, fiz[a]);
                    fjx[b] -= xd * fs; fjy[b] -= yd * fs; fjz[b] -= zd * fs;
                }
            }
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                if (b >= nsi_j) break;
                red_v4(&pk.F[j + b], fjx[b], fjy[b], fjz[b]);
            }
            e_add(e, ijt, elj, eqq, s_e, v.nijt);
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (a >= nsi_i) break;
            const float sx = warp_sumf(fix[a]), sy = warp_sumf(fiy[a]), sz = warp_sumf(fiz[a]);
            if (lane == 0) red_v4(&pk.F[i + a], sx, sy, sz);
        }
    }
}

// The block's energy sums into the system's accumulators (all threads; the shared sums are free
// for the next system's tables afterwards).
__device__ __forceinline__ void pair_flush(const View& v, EAcc& e, double* s_e) {
    e_final(e, s_e, v.nijt);
    e = EAcc();
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * v.nijt; k += blockDim.x)
        if (s_e[k] != 0.0) atomicAdd(&v.acc[k], s_e[k]);
    __syncthreads();
}

template <int ZPER>
__global__ void __launch_bounds__(kNT) k_pair_mx(View v, Pk pk) {
    extern __shared__ double s_e[];
    const Tables T = load_tables(v, pk, s_e, 0);
    EAcc e;
    pair_heads<ZPER>(v, pk, T, blockIdx.x * kWarps + (threadIdx.x >> 5), gridDim.x * kWarps, e, s_e);
    pair_flush(v, e, s_e);
}

// Head-wall work units of a system: (head, segment of seg wall partners), so that the few heads
// next to a wall with hundreds of partners are shared by several warps (seg = kWSeg for one
// system; a batch of systems has parallelism to spare and takes kWSegBatch, which halves the per-unit
// work of the head's loads and reductions).  A lane sees at most seg / 32 partners per unit, so its
// FP32 sums within a unit are short and need no compensation.
constexpr int kWSegBatch = 256;
__host__ __device__ __forceinline__ long wall_units(const View& v, int seg) {
    return (long)v.nheads * ((v.maxwnb + seg - 1) / seg);
}

// Energy sums per wall site type (the last two site types; the two alternate from partner to
// partner, and one accumulator per type avoids a flush on every change) and the wall reaction
// sums of the lane, added per work unit.
struct WAcc {
    EAcc ew[2];
    double ws[6] = {0, 0, 0, 0, 0, 0};
    double* s_e = nullptr;  // the block's shared energy sums
};

// The head-wall loop of one warp over the units u0, u0 + us, ... below wall_units(v, seg).
template <int ZPER>
__device__ __forceinline__ void wall_heads(const View& v, const Pk& pk, const Tables& T, long u0, long us, int seg,
                                           WAcc& w) {
    const int lane = threadIdx.x & 31;
    const float alfa = pk.alfa, spii = pk.spii, facq = pk.facq, rcutsq = pk.rcutsq;
    const int wt0 = v.nit - 2;
    const int nseg = (v.maxwnb + seg - 1) / seg;
    const long nitems = (long)v.nheads * nseg;
    for (long item = u0; item < nitems; item += us) {
        const int h = (int)(item / nseg), sg = (int)(item % nseg);
        const int n = min(v.wnbcnt[h], (sg + 1) * seg);
        if (sg * seg >= n) continue;
        const int i = v.head_atom[h];
        const uint4 pi = pk.P[i];
        const int it = (int)(pi.w & 0x7fffffffu);
        const int nsi_i = T.nsi[it];
        const bool book = (it + 1) <= v.nltype;
        const float zli = ZPER ? 0.f : pk.zlo[i];
        float4 si[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) si[a] = a < nsi_i ? pk.Q[i + a] : make_float4(0.f, 0.f, 0.f, 0.f);
        float fix[3] = {0, 0, 0}, fiy[3] = {0, 0, 0}, fiz[3] = {0, 0, 0};
        // wall reaction sums of this unit, lower wall (z < 0) in l*, upper in u*: plain registers
        // updated through selects (x - 0 is exact, so each sum is what a per-wall array gives)
        float lx = 0.f, ly = 0.f, lz = 0.f, ux = 0.f, uy = 0.f, uz = 0.f;
        const int* nb = v.wnb + (size_t)h * v.maxwnb;
        const float* qw = reinterpret_cast<const float*>(pk.Q) + 3;  // charges: Q[j].w = qw[4 j]
        // software pipeline as in the head-head loop: the next partner's record and charge and
        // the index after it load while this partner is computed
        const int k0 = sg * seg + lane;
        int j1 = k0 < n ? nb[k0] : 0;
        int j2 = k0 + 32 < n ? nb[k0 + 32] : 0;
        uint4 p1 = k0 < n ? pk.P[j1] : make_uint4(0u, 0u, 0u, 0u);
        float q1 = k0 < n ? qw[4 * (size_t)j1] : 0.f;
        for (int k = k0; k < n; k += 32) {
            const int j = j1;
            const uint4 pj = p1;
            const float qj = q1;
            j1 = j2;
            if (k + 32 < n) {
                p1 = pk.P[j1];
                q1 = qw[4 * (size_t)j1];
            }
            if (k + 64 < n) j2 = nb[k + 64];
            float xi, yi, zi;
            head_vec<ZPER>(pi, zli, pj, pk, j, xi, yi, zi);
            const float rsq = xi * xi + yi * yi + zi * zi;
            if (rsq > rcutsq) continue;
            const bool lower = (pj.w & 0x80000000u) != 0;
            const int jt = (int)(pj.w & 0x7fffffffu);
            const int ijt = T.ijt[it * v.nit + jt];
            const float rinv = rsqrtf(rsq);
            float fij;
            const float elj = vdw_term(T.par + 6 * ijt, rinv * rinv, rinv, rsq * rinv, &fij);
            const float qx = facq * qj;
            float eqq = 0.f;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (a >= nsi_i) break;
                const float xd = xi + si[a].x, yd = yi + si[a].y, zd = zi + si[a].z;
                const float r2 = xd * xd + yd * yd + zd * zd;
                const float ri = rsqrtf(r2);
                const float rr = r2 * ri;
                const float au = qx * si[a].w * ri;
                float fq;
                eqq += erfc_as(alfa * rr, &fq, spii) * au;
                fij = fij + fq * au * (ri * ri);
                fix[a] = fmaf(xd, fij, fix[a]);
                fiy[a] = fmaf(yd, fij, fiy[a]);
                fiz[a] = fmaf(zd, fij, fiz[a]);
                if (book) {
                    const float sx = xd * fij, sy = yd * fij, sz = zd * fij;
                    lx -= lower ? sx : 0.f; ly -= lower ? sy : 0.f; lz -= lower ? sz : 0.f;
                    ux -= lower ? 0.f : sx; uy -= lower ? 0.f : sy; uz -= lower ? 0.f : sz;
                }
                fij = 0.f;
            }
            // energy sums per wall site type (the last two site types)
            if (jt > wt0) e_add(w.ew[1], ijt, elj, eqq, w.s_e, v.nijt);
            else e_add(w.ew[0], ijt, elj, eqq, w.s_e, v.nijt);
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (a >= nsi_i) break;
            const float sx = warp_sumf(fix[a]), sy = warp_sumf(fiy[a]), sz = warp_sumf(fiz[a]);
            if (lane == 0) red_v4(&pk.F[i + a], sx, sy, sz);
        }
        if (book) {
            w.ws[0] += (double)lx; w.ws[1] += (double)ly; w.ws[2] += (double)lz;
            w.ws[3] += (double)ux; w.ws[4] += (double)uy; w.ws[5] += (double)uz;
        }
    }
}

// The block's energy and wall reaction sums into the system's accumulators (all threads).
__device__ __forceinline__ void wall_flush(const View& v, WAcc& w) {
    double* s_e = w.s_e;
    e_final(w.ew[0], s_e, v.nijt);
    e_final(w.ew[1], s_e, v.nijt);
    w.ew[0] = EAcc();
    w.ew[1] = EAcc();
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const double s = warp_sum(w.ws[k]);
        if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(&s_e[2 * v.nijt + k], s);
        w.ws[k] = 0.0;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * v.nijt; k += blockDim.x)
        if (s_e[k] != 0.0) atomicAdd(&v.acc[k], s_e[k]);
    if (threadIdx.x < 6) {
        const int comp = threadIdx.x % 3, sg = threadIdx.x / 3;
        const double s = s_e[2 * v.nijt + threadIdx.x];
        if (s != 0.0) atomicAdd(&v.acc[2 * v.nijt + ACC_FWS + comp * 3 + (sg ? 2 : 0)], s);
    }
    __syncthreads();
}

template <int ZPER>
__global__ void __launch_bounds__(kNT) k_wall_mx(View v, Pk pk) {
    extern __shared__ double s_e[];
    const Tables T = load_tables(v, pk, s_e, 6);
    WAcc w;
    w.s_e = s_e;
    wall_heads<ZPER>(v, pk, T, blockIdx.x * kWarps + (threadIdx.x >> 5), (long)gridDim.x * kWarps, kWSeg, w);
    wall_flush(v, w);
}

// ---- the same loops over several systems in one launch (replica batches) -------------------
// Each system's heads (or head-wall units) are cut into work items of about kItemUnits units; the
// items of system r are r's first item .. its next system's first item, and item k of a system with
// n items holds its units k, k + n, k + 2n, ... (a stride through the whole system, so that items
// near a wall and items in the middle of a film cost alike).  Block b walks the items
// [b N / G, (b + 1) N / G) of all N in order: its system changes only a few times, and then it
// flushes the finished system's energies and loads the next one's view and tables into shared
// memory.
constexpr int kItemUnits = 64;

struct alignas(16) RsRep {
    View v;
    Pk pk;
};

// View and Pk copied word by word into shared memory (plain data: pointers, sizes, scalars).
__device__ __forceinline__ void load_rep(const RsRep* __restrict__ src, RsRep* dst) {
    static_assert(sizeof(RsRep) % 8 == 0, "word copy");
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(dst);
    for (int k = threadIdx.x; k < (int)(sizeof(RsRep) / 8); k += blockDim.x) d[k] = s[k];
    __syncthreads();
}

// The system of item it: the first r with first[r + 1] > it, searched from r (items in order).
__device__ __forceinline__ int rep_of(const int* __restrict__ first, int nrep, int it, int r) {
    if (r < 0) {
        int lo = 0, hi = nrep - 1;  // first[0] = 0 <= it < first[nrep]
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (first[mid] <= it) lo = mid;
            else hi = mid - 1;
        }
        r = lo;
    }
    while (r < nrep - 1 && first[r + 1] <= it) ++r;
    return r;
}

template <int ZPER>
__global__ void __launch_bounds__(kNT) k_pair_mx_batch(const RsRep* __restrict__ reps, const int* __restrict__ first,
                                                        int nrep) {
    extern __shared__ double s_e[];
    __shared__ alignas(16) unsigned char sr_raw[sizeof(RsRep)];  // RsRep has member initialisers
    RsRep& sr = *reinterpret_cast<RsRep*>(sr_raw);
    const int nitems = first[nrep];
    const int b0 = (int)((long)nitems * blockIdx.x / gridDim.x);
    const int b1 = (int)((long)nitems * (blockIdx.x + 1) / gridDim.x);
    const int warp = threadIdx.x >> 5;
    int r = -1;
    Tables T{};
    EAcc e;
    for (int it = b0; it < b1; ++it) {
        const int rn = rep_of(first, nrep, it, r);
        if (rn != r) {
            if (r >= 0) pair_flush(sr.v, e, s_e);
            load_rep(reps + rn, &sr);
            T = load_tables(sr.v, sr.pk, s_e, 0);
            r = rn;
        }
        const int n = first[r + 1] - first[r], k = it - first[r];
        pair_heads<ZPER>(sr.v, sr.pk, T, k + n * warp, n * kWarps, e, s_e);
    }
    if (r >= 0) pair_flush(sr.v, e, s_e);
}

template <int ZPER>
__global__ void __launch_bounds__(kNT) k_wall_mx_batch(const RsRep* __restrict__ reps, const int* __restrict__ first,
                                                        int nrep) {
    extern __shared__ double s_e[];
    __shared__ alignas(16) unsigned char sr_raw[sizeof(RsRep)];  // RsRep has member initialisers
    RsRep& sr = *reinterpret_cast<RsRep*>(sr_raw);
    const int nitems = first[nrep];
    const int b0 = (int)((long)nitems * blockIdx.x / gridDim.x);
    const int b1 = (int)((long)nitems * (blockIdx.x + 1) / gridDim.x);
    const int warp = threadIdx.x >> 5;
    int r = -1;
    Tables T{};
    WAcc w;
    w.s_e = s_e;
    for (int it = b0; it < b1; ++it) {
        const int rn = rep_of(first, nrep, it, r);
        if (rn != r) {
            if (r >= 0) wall_flush(sr.v, w);
            load_rep(reps + rn, &sr);
            T = load_tables(sr.v, sr.pk, s_e, 6);
            r = rn;
        }
        const long n = first[r + 1] - first[r], k = it - first[r];
        wall_heads<ZPER>(sr.v, sr.pk, T, k + n * warp, n * kWarps, kWSegBatch, w);
    }
    if (r >= 0) wall_flush(sr.v, w);
}

// F (and the reciprocal forces frc, 3 x nmove, when given) into the FP64 forces; F cleared.
// crf0 != 0 adds the slab term fz += 2 crf0 facq M_z q (src/forcem.f90:925-928) with M_z from
// k_pack.
__global__ void k_merge_f(View v, Pk pk, const double* __restrict__ frc, double crf0) {
    const double crf = crf0 != 0.0 ? 2.0 * crf0 * v.facq * v.acc[2 * v.nijt + ACC_DIPZ] : 0.0;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < v.nmove; a += gridDim.x * blockDim.x) {
        const float4 f = pk.F[a];
        double gx = (double)f.x, gy = (double)f.y, gz = (double)f.z;
        if (frc) {
            gx += frc[a];
            gy += frc[v.nmove + a];
            gz += frc[2 * v.nmove + a];
        }
        if (crf0 != 0.0) gz += crf * v.q[a];
        v.fx[a] += gx;
        v.fy[a] += gy;
        v.fz[a] += gz;
        pk.F[a] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

int blocks(const Ctx& c, int nheads) {
    const int b = std::max(1, std::min((nheads + kWarps - 1) / kWarps, 152 * 16));
    return c.pair_blocks > 0 ? std::min(b, c.pair_blocks) : b;
}

size_t table_smem(const View& v, int nextra) {
    return sizeof(double) * (2 * v.nijt + nextra) + sizeof(float) * 6 * v.nijt + sizeof(int) * (v.nit * v.nit + v.nit);
}

}  // namespace

void pack_setup(Ctx& c) {
    const View& v = c.v;
    const int n = std::max(v.ntota, 1);
    c.pk.P = (uint4*)dalloc(c, sizeof(uint4) * n);
    c.pk.Q = (float4*)dalloc(c, sizeof(float4) * n);
    c.pk.zlo = (float*)dalloc(c, sizeof(float) * n);
    c.pk.F = (float4*)dalloc(c, sizeof(float4) * std::max(v.nmove, 1));
    c.pk.part = (double*)dalloc(c, sizeof(double) * kPackParts);
    c.pk.zper = v.bulk ? 1 : 0;
    c.pk.sx = (float)(v.lx / 4294967296.0);
    c.pk.sy = (float)(v.ly / 4294967296.0);
    c.pk.sz = (float)(v.lz / 4294967296.0);
    c.pk.alfa = (float)v.alfa;
    c.pk.spii = (float)v.spii;
    c.pk.facq = (float)v.facq;
    c.pk.rcutsq = (float)v.rcutsq;
}

double slab_crf0(const Ctx& c) {
    if (c.variant != MDG_SLAB) return 0.0;
    return -2.0 * (double)3.1415926535898f * c.v.lzi * c.v.lxi * c.v.lyi;
}

__global__ void __launch_bounds__(32) k_pack_close(View v, Pk pk, int dip, int force, int nparts) {
    pack_close_warp(v, pk, dip, force, 0, nparts, false);
}

void pack_mixed(Ctx& c, bool force_rebuild, bool reset_status, bool defer_close) {
    const View& v = c.v;
    const int n = std::max(std::max(v.ntota, v.nrig + (v.nmove - v.nriga)), 1);
    const int nb = std::min((n + 255) / 256, kPackBlocks);
    c.pack_parts = nb;
    c.pack_force = force_rebuild;
    k_pack<<<nb, 256, 0, c.stream>>>(v, c.pk, c.variant == MDG_SLAB ? 1 : 0, force_rebuild ? 1 : 0,
                                     reset_status ? 1 : 0, defer_close ? 1 : 0);
}

void pack_close_launch(Ctx& c) {
    k_pack_close<<<1, 32, 0, c.stream>>>(c.v, c.pk, c.variant == MDG_SLAB ? 1 : 0, c.pack_force ? 1 : 0,
                                         c.pack_parts);
}

void merge_mixed(Ctx& c, const double* frc, bool dipole) {
    const View& v = c.v;
    if (v.nmove == 0) return;
    k_merge_f<<<std::min((v.nmove + 255) / 256, 152 * 8), 256, 0, c.stream>>>(v, c.pk, frc,
                                                                              dipole ? slab_crf0(c) : 0.0);
}

void pairs_mixed(Ctx& c, bool merge) {
    const View& v = c.v;
    if (v.nheads == 0) return;
    // Beside the head-wall loop and the reciprocal sum (merge false: the concurrent form) the
    // head-head loop has time to spare; it keeps to one block per SM, leaving room for the
    // reciprocal branch's kernels (measured on the slab: its reduction 18 -> 13 us, the step 2 %).
    int nb = blocks(c, v.nheads);
    if (!merge) nb = std::min(nb, 152);
    if (c.pk.zper) k_pair_mx<1><<<nb, kNT, table_smem(v, 0), c.stream>>>(v, c.pk);
    else k_pair_mx<0><<<nb, kNT, table_smem(v, 0), c.stream>>>(v, c.pk);
    if (merge) merge_mixed(c, nullptr, false);
}

void walls_mixed(Ctx& c, bool concurrent) {
    const View& v = c.v;
    if (v.nheads == 0 || v.nwall == 0) return;
    // beside the head-head loop and the reciprocal sum, one block per SM, as the head-head loop
    // (measured on the slab: the reciprocal reduction gets the room, the step 2 % shorter)
    int nb = blocks(c, v.nheads);
    if (concurrent) nb = std::min(nb, 152);
    if (c.pk.zper) k_wall_mx<1><<<nb, kNT, table_smem(v, 6), c.stream>>>(v, c.pk);
    else k_wall_mx<0><<<nb, kNT, table_smem(v, 6), c.stream>>>(v, c.pk);
}

// ---- replica batches: host side ------------------------------------------------------------
int rs_batch_setup(RsBatch& rb, const std::vector<Ctx*>& cs, std::string& err) {
    std::vector<RsRep> reps[2];
    std::vector<int> fp[2], fw[2];
    size_t smem[2][2] = {{0, 0}, {0, 0}};
    for (Ctx* c : cs) {
        const int g = c->pk.zper ? 1 : 0;
        RsRep r;
        r.v = c->v;
        r.pk = c->pk;
        if (fp[g].empty()) {
            fp[g].push_back(0);
            fw[g].push_back(0);
        }
        const long nw = wall_units(c->v, kWSegBatch);
        fp[g].push_back(fp[g].back() + (c->v.nheads + kItemUnits - 1) / kItemUnits);
        fw[g].push_back(fw[g].back() + (int)((nw + kItemUnits - 1) / kItemUnits));
        reps[g].push_back(r);
        smem[g][0] = std::max(smem[g][0], table_smem(c->v, 0));
        smem[g][1] = std::max(smem[g][1], table_smem(c->v, 6));
    }
    size_t need = 0;
    size_t off[2][3];
    for (int g = 0; g < 2; ++g) {
        off[g][0] = need;
        need += (sizeof(RsRep) * reps[g].size() + 255) & ~size_t(255);
        off[g][1] = need;
        need += (sizeof(int) * fp[g].size() + 255) & ~size_t(255);
        off[g][2] = need;
        need += (sizeof(int) * fw[g].size() + 255) & ~size_t(255);
    }
    if (need > rb.cap) {
        if (rb.d_buf) cudaFree(rb.d_buf);
        rb.d_buf = nullptr;
        rb.cap = 0;
        if (cudaMalloc(&rb.d_buf, need) != cudaSuccess) {
            err = "replica batch: descriptor allocation failed";
            return MDG_E_CUDA;
        }
        rb.cap = need;
    }
    unsigned char* base = static_cast<unsigned char*>(rb.d_buf);
    for (int g = 0; g < 2; ++g) {
        RsBatch::Group& G = rb.g[g];
        G = RsBatch::Group();
        G.nrep = (int)reps[g].size();
        if (G.nrep == 0) continue;
        G.reps = base + off[g][0];
        G.first_p = reinterpret_cast<int*>(base + off[g][1]);
        G.first_w = reinterpret_cast<int*>(base + off[g][2]);
        G.items_p = fp[g].back();
        G.items_w = fw[g].back();
        G.smem_p = smem[g][0];
        G.smem_w = smem[g][1];
        if (cudaMemcpy(G.reps, reps[g].data(), sizeof(RsRep) * G.nrep, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(G.first_p, fp[g].data(), sizeof(int) * fp[g].size(), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(G.first_w, fw[g].data(), sizeof(int) * fw[g].size(), cudaMemcpyHostToDevice) != cudaSuccess) {
            err = "replica batch: descriptor upload failed";
            return MDG_E_CUDA;
        }
    }
    return MDG_OK;
}

void rs_batch_launch(const RsBatch& rb, cudaStream_t sp, cudaStream_t sw) {
    for (int g = 0; g < 2; ++g) {
        const RsBatch::Group& G = rb.g[g];
        if (G.nrep == 0) continue;
        const RsRep* reps = static_cast<const RsRep*>(G.reps);
        if (G.items_w > 0) {
            const int nb = std::max(1, std::min(rb.blocks_w, G.items_w));
            if (g) k_wall_mx_batch<1><<<nb, kNT, G.smem_w, sw>>>(reps, G.first_w, G.nrep);
            else k_wall_mx_batch<0><<<nb, kNT, G.smem_w, sw>>>(reps, G.first_w, G.nrep);
        }
        if (G.items_p > 0) {
            const int nb = std::max(1, std::min(rb.blocks_p, G.items_p));
            if (g) k_pair_mx_batch<1><<<nb, kNT, G.smem_p, sp>>>(reps, G.first_p, G.nrep);
            else k_pair_mx_batch<0><<<nb, kNT, G.smem_p, sp>>>(reps, G.first_p, G.nrep);
        }
    }
}

void rs_batch_free(RsBatch& rb) {
    if (rb.d_buf) cudaFree(rb.d_buf);
    rb = RsBatch();
}

}  // namespace mdg
