// recip_tc.cu - reciprocal-space Ewald sum on tcgen05 tensor cores (mixed precision path).
//
// The sum of force_fouri (src/forcem.f90:827-937) factorises over the k components:
//   S(l,m,n) = sum_j [q_j e^{i(l tx_j + m ty_j)}] e^{i n tz_j}                       (pass 1)
//   f_j      = q_j sum_{l,m} Im( e^{i(l tx_j + m ty_j)} T_j(l,m) ) (kx, ky) and
//              q_j kz sum_{l,m} Im( e^{i(l tx_j + m ty_j)} T'_j(l,m) ) with
//   T_j(l,m) = sum_n C(l,m,n) e^{i n tz_j},  T'_j(l,m) = sum_n n C(l,m,n) e^{i n tz_j}   (pass 2)
// with C = Ak conj(S + S_wall).  Both are complex matrix products written as real ones:
//   pass 1: D[(l,m) row, (re|im, n)] over K = atoms, A = [Re | Im] of the row factor, B = the
//           2x2 real block form of e^{i n tz}, M = 128 rows per CTA, split-K over atom chunks;
//   pass 2: D[atom, (row, T|T', re|im)] over K = (n, re|im), A = e^{i n tz} per atom (built once
//           per CTA), B = packed C chunks streamed with cp.async.bulk, two TMEM accumulators
//           double-buffered against the epilogue that forms Im(e T) per row.
// Operands are hi/lo splits (x = hi + lo, FP16 halves here; the self test exercises BF16) and every
// product is hi*hi + hi*lo + lo*hi with FP32 accumulation in TMEM.  Phases come from exact 32-bit fixed-point fractions of the box
// (u = frac(x/L) 2^32, so l*u wraps modulo one period) evaluated with __sincosf on [-pi, pi).
// Each thread block waits on mbarriers with bounded spins; a timeout sets status[ST_TC_TIMEOUT].
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "ctx.h"
#include "tc.cuh"

namespace mdg {

namespace {

constexpr int kG1 = 32;      // atoms per pass-1 group (two K steps)
constexpr int kT = 256;      // threads per CTA
constexpr float kPhase = 1.4629180792671596e-09f;  // 2 pi / 2^32

// Operand type of the hi/lo split.  FP16 keeps 11 + 11 significant bits (BF16: 8 + 8); all
// operands are O(1) (phase factors, charges, and C(k) scaled by the step's max |n C|).
typedef __half elem_t;
__device__ __forceinline__ uint32_t idesc_e(int M, int N) { return tc::idesc_f16(M, N); }
__device__ __forceinline__ uint16_t ebits(elem_t h) { return __half_as_ushort(h); }
__device__ __forceinline__ elem_t eneg(elem_t h) { return __hneg(h); }

struct TcDims {
    int KN, NN;      // n range -KN..KN, NN = 2 KN + 1
    int NP;          // pass-1 N (2 NN rounded up to 16)
    int KS;          // pass-2 K steps (2 NN rounded up to 16, / 16)
    int nrow, nchunk2;
    float px, py, pz;
};

__device__ __forceinline__ void phase(uint32_t u, float& c, float& s) {
    __sincosf((float)(int32_t)u * kPhase, &s, &c);
}

__device__ __forceinline__ uint32_t pack2(elem_t a, elem_t b) {
    return (uint32_t)ebits(a) | ((uint32_t)ebits(b) << 16);
}

// 32-bit fixed-point box fractions and the charge of each moving atom
__global__ void k_tc_prep_atoms(View v, uint4* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nmove) return;
    double f[3] = {v.x[i] * v.lxi, v.y[i] * v.lyi, v.z[i] * v.lzi};
    uint32_t u[3];
    for (int d = 0; d < 3; ++d) {
        const double fr = f[d] - floor(f[d]);
        u[d] = (uint32_t)(unsigned long long)llrint(fr * 4294967296.0);
    }
    out[i] = make_uint4(u[0], u[1], u[2], __float_as_uint((float)v.q[i]));
}

// ---------------------------------------------------------------------------------------------
// pass 1: structure factor
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kT, 1) k_tc_sfac(View v, const uint4* __restrict__ atoms, int chunk,
                                                   const int4* __restrict__ rows, const int* __restrict__ nlen,
                                                   TcDims d, double2* S, uint32_t ncols) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const uint32_t aBytes = 8 * 4096;                 // [p][h][ks] 128 x 16 tiles
    const uint32_t bTile = (uint32_t)d.NP * 32;       // NP x 16 tile
    const uint32_t stBytes = aBytes + 8 * bTile;
    unsigned char* stage0 = sm + 1024;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm);  // mma_done[2]
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 64);
    int* err = &v.status[ST_TC_TIMEOUT];
    const int a0 = blockIdx.y * chunk, a1 = min(v.nmove, a0 + chunk);
    const int ngroup = (a1 > a0) ? (a1 - a0 + kG1 - 1) / kG1 : 0;
    const int row_base = blockIdx.x * 128;
    if (t == 0) {
        tc::mbar_init(tc::smem_u32(&bars[0]), 1);
        tc::mbar_init(tc::smem_u32(&bars[1]), 1);
        tc::mbar_fence_init();
    }
    // zero both stages once (padding rows of B stay zero)
    for (uint32_t o = t * 16; o < 2 * stBytes; o += kT * 16) *reinterpret_cast<uint4*>(stage0 + o) = make_uint4(0, 0, 0, 0);
    if (warp == 0) tc::tmem_alloc(tc::smem_u32(tslot), ncols);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = idesc_e(128, d.NP);
    // this thread's row for the A operand
    const int r = t & 127, ksA = t >> 7;
    const int row = row_base + r;
    int l = 0, m = 0;
    const bool row_ok = row < d.nrow;
    if (row_ok) {
        const int4 rw = rows[row];
        l = rw.x;
        m = rw.y;
    }
    bool alive = true;
    for (int g = 0; g < ngroup && alive; ++g) {
        const int s = g & 1;
        unsigned char* st = stage0 + s * stBytes;
        if (g >= 2) alive = tc::mbar_wait(tc::smem_u32(&bars[s]), ((g >> 1) - 1) & 1, err, 11);
        if (!alive) break;
        const int gbase = a0 + g * kG1;
        // A: row r, atoms ksA*16 .. +15, parts re/im, hi/lo
        {
            uint32_t w[4][8];  // [p*2+h][pair]
#pragma unroll
            for (int i = 0; i < 16; i += 2) {
                float ar[2], ai[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const int at = gbase + ksA * 16 + i + e;
                    ar[e] = ai[e] = 0.f;
                    if (row_ok && at < a1) {
                        const uint4 rec = atoms[at];
                        float c, sn;
                        phase((uint32_t)l * rec.x + (uint32_t)m * rec.y, c, sn);
                        const float q = __uint_as_float(rec.w);
                        ar[e] = q * c;
                        ai[e] = q * sn;
                    }
                }
                elem_t h0, l0, h1, l1;
                tc::split(ar[0], h0, l0);
                tc::split(ar[1], h1, l1);
                w[0][i >> 1] = pack2(h0, h1);
                w[1][i >> 1] = pack2(l0, l1);
                tc::split(ai[0], h0, l0);
                tc::split(ai[1], h1, l1);
                w[2][i >> 1] = pack2(h0, h1);
                w[3][i >> 1] = pack2(l0, l1);
            }
#pragma unroll
            for (int ph = 0; ph < 4; ++ph) {
                unsigned char* tile = st + (ph * 2 + ksA) * 4096;  // [p][h][ks]
                *reinterpret_cast<uint4*>(tile + tc::tile_off(r, 0)) = make_uint4(w[ph][0], w[ph][1], w[ph][2], w[ph][3]);
                *reinterpret_cast<uint4*>(tile + tc::tile_off(r, 8)) = make_uint4(w[ph][4], w[ph][5], w[ph][6], w[ph][7]);
            }
        }
        // B: rows (re, n) and (im, n) for 16 atoms of one K step
        if (t < 2 * d.NN) {
            const int ni = t % d.NN, ks = t / d.NN;
            const int n = ni - d.KN;
            uint32_t wc[2][8], wsn[2][8], wns[2][8];  // [h][pair]: cos, sin, -sin
#pragma unroll
            for (int i = 0; i < 16; i += 2) {
                float c2[2], s2[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const int at = gbase + ks * 16 + i + e;
                    c2[e] = s2[e] = 0.f;
                    if (at < a1) phase((uint32_t)n * atoms[at].z, c2[e], s2[e]);
                }
                elem_t hc0, lc0, hc1, lc1, hs0, ls0, hs1, ls1;
                tc::split(c2[0], hc0, lc0);
                tc::split(c2[1], hc1, lc1);
                tc::split(s2[0], hs0, ls0);
                tc::split(s2[1], hs1, ls1);
                wc[0][i >> 1] = pack2(hc0, hc1);
                wc[1][i >> 1] = pack2(lc0, lc1);
                wsn[0][i >> 1] = pack2(hs0, hs1);
                wsn[1][i >> 1] = pack2(ls0, ls1);
                wns[0][i >> 1] = pack2(eneg(hs0), eneg(hs1));
                wns[1][i >> 1] = pack2(eneg(ls0), eneg(ls1));
            }
            unsigned char* bb = st + aBytes;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                // part 0: re row <- cos, im row <- sin ; part 1: re row <- -sin, im row <- cos
                unsigned char* t0 = bb + ((0 * 2 + h) * 2 + ks) * bTile;
                unsigned char* t1 = bb + ((1 * 2 + h) * 2 + ks) * bTile;
                const int rre = ni, rim = d.NN + ni;
                *reinterpret_cast<uint4*>(t0 + tc::tile_off(rre, 0)) = make_uint4(wc[h][0], wc[h][1], wc[h][2], wc[h][3]);
                *reinterpret_cast<uint4*>(t0 + tc::tile_off(rre, 8)) = make_uint4(wc[h][4], wc[h][5], wc[h][6], wc[h][7]);
                *reinterpret_cast<uint4*>(t0 + tc::tile_off(rim, 0)) = make_uint4(wsn[h][0], wsn[h][1], wsn[h][2], wsn[h][3]);
                *reinterpret_cast<uint4*>(t0 + tc::tile_off(rim, 8)) = make_uint4(wsn[h][4], wsn[h][5], wsn[h][6], wsn[h][7]);
                *reinterpret_cast<uint4*>(t1 + tc::tile_off(rre, 0)) = make_uint4(wns[h][0], wns[h][1], wns[h][2], wns[h][3]);
                *reinterpret_cast<uint4*>(t1 + tc::tile_off(rre, 8)) = make_uint4(wns[h][4], wns[h][5], wns[h][6], wns[h][7]);
                *reinterpret_cast<uint4*>(t1 + tc::tile_off(rim, 0)) = make_uint4(wc[h][0], wc[h][1], wc[h][2], wc[h][3]);
                *reinterpret_cast<uint4*>(t1 + tc::tile_off(rim, 8)) = make_uint4(wc[h][4], wc[h][5], wc[h][6], wc[h][7]);
            }
        }
        tc::fence_async_smem();
        __syncthreads();
        if (t == 0) {
            tc::fence_after();
            const uint32_t sbase = tc::smem_u32(st);
#pragma unroll
            for (int p = 0; p < 2; ++p)
#pragma unroll
                for (int ks = 0; ks < 2; ++ks) {
                    const uint64_t ah = tc::desc(sbase + ((p * 2 + 0) * 2 + ks) * 4096);
                    const uint64_t al = tc::desc(sbase + ((p * 2 + 1) * 2 + ks) * 4096);
                    const uint64_t bh = tc::desc(sbase + aBytes + ((p * 2 + 0) * 2 + ks) * bTile);
                    const uint64_t bl = tc::desc(sbase + aBytes + ((p * 2 + 1) * 2 + ks) * bTile);
                    const uint32_t first = (g == 0 && p == 0 && ks == 0) ? 0u : 1u;
                    tc::mma_bf16(tmem, ah, bh, idesc, first);
                    tc::mma_bf16(tmem, ah, bl, idesc, 1u);
                    tc::mma_bf16(tmem, al, bh, idesc, 1u);
                }
            tc::commit(tc::smem_u32(&bars[s]));
        }
    }
    // all MMAs of this block done
    if (ngroup > 0 && alive) alive = tc::mbar_wait(tc::smem_u32(&bars[(ngroup - 1) & 1]), ((ngroup - 1) >> 1) & 1, err, 12);
    __syncthreads();
    if (ngroup > 0 && t < 128) {
        tc::fence_after();
        int nf = 0, kf = 0, nl = 0;
        if (row_ok) {
            const int4 rw = rows[row];
            nf = rw.z;
            kf = rw.w;
            nl = nlen[row];
        }
        for (int cc = 0; cc < d.NP / 16; ++cc) {
            float val[16];
            tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + cc * 16, val);
            if (!row_ok || !alive) continue;
#pragma unroll
            for (int c = 0; c < 16; ++c) {
                const int col = cc * 16 + c;
                if (col >= 2 * d.NN) continue;
                const int comp = col >= d.NN ? 1 : 0;
                const int n = (comp ? col - d.NN : col) - d.KN;
                if (n < nf || n >= nf + nl) continue;
                double* dst = comp ? &S[kf + n - nf].y : &S[kf + n - nf].x;
                atomicAdd(dst, (double)val[c]);
            }
        }
        tc::fence_before();
    }
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, ncols);
    }
    (void)lane;
}

// ---------------------------------------------------------------------------------------------
// C(k) packed as the pass-2 B operand: chunk c holds rows 32c..32c+31, columns
// col = 4 r_local + 2 t + comp (t: T or T', comp: re or im), K = 2 (n + KN) + part.
// ---------------------------------------------------------------------------------------------
// max |C| * max(1, |n|) over the k set (non-negative floats order like their bits)
__global__ void k_tc_cmax(const double2* __restrict__ C, const int3* __restrict__ kv, int nk, float* cmax) {
    float m = 0.f;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nk; k += gridDim.x * blockDim.x) {
        const double2 c = C[k];
        const double w = fmax(1.0, fabs((double)kv[k].z));
        m = fmaxf(m, (float)(fmax(fabs(c.x), fabs(c.y)) * w));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned int*>(cmax), __float_as_uint(m));
}

__global__ void k_tc_prep_c(const double2* __restrict__ C, const int4* __restrict__ rows,
                            const int* __restrict__ nlen, TcDims d, unsigned char* img, const float* cmax) {
    const double inv = cmax[0] > 0.f ? 1.0 / (double)cmax[0] : 1.0;
    const long total = (long)d.nchunk2 * d.KS * 128 * 16;
    const long chunkBytes = 2L * d.KS * 4096;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        const int kk = e & 15;
        const int col = (e >> 4) & 127;
        const long rest = e >> 11;
        const int ks = (int)(rest % d.KS);
        const int c = (int)(rest / d.KS);
        const int row = c * 32 + (col >> 2), tt = (col >> 1) & 1, comp = col & 1;
        const int k2 = ks * 16 + kk, ni = k2 >> 1, part = k2 & 1;
        float val = 0.f;
        if (row < d.nrow && ni < d.NN) {
            const int4 rw = rows[row];
            const int n = ni - d.KN;
            if (n >= rw.z && n < rw.z + nlen[row]) {
                const double2 cv = C[rw.w + n - rw.z];
                const double sc = (tt ? (double)n : 1.0) * inv;
                const double cr = cv.x * sc, ci = cv.y * sc;
                const double vv = comp == 0 ? (part == 0 ? cr : -ci) : (part == 0 ? ci : cr);
                val = (float)vv;
            }
        }
        elem_t h, lo;
        tc::split(val, h, lo);
        unsigned char* base = img + c * chunkBytes;
        const uint32_t off = tc::tile_off(col, kk);
        *reinterpret_cast<elem_t*>(base + (0 * d.KS + ks) * 4096 + off) = h;
        *reinterpret_cast<elem_t*>(base + (1 * d.KS + ks) * 4096 + off) = lo;
    }
}

// ---------------------------------------------------------------------------------------------
// pass 2: forces
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kT, 1) k_tc_force(View v, const uint4* __restrict__ atoms,
                                                    const unsigned char* __restrict__ img,
                                                    const int4* __restrict__ rows, TcDims d, const float* cmax) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const uint32_t tileB = 4096;
    const uint32_t halfBytes = d.KS * tileB;   // one of hi / lo
    const uint32_t imgBytes = 2 * halfBytes;   // a chunk image
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm);  // full[2], mma_done[2], acc_free[2]
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 64);
    unsigned char* Asm = sm + 1024;            // [h][ks] 128 x 16
    unsigned char* Bsm = Asm + imgBytes;       // [s][h][ks]
    int* err = &v.status[ST_TC_TIMEOUT];
    const int atom0 = blockIdx.x * 128;
    if (t == 0) {
        for (int b = 0; b < 6; ++b) tc::mbar_init(tc::smem_u32(&bars[b]), b >= 4 ? 4 : 1);
        tc::mbar_fence_init();
    }
    if (warp == 0) tc::tmem_alloc(tc::smem_u32(tslot), 256);
    // A: e^{i n tz} of this block's atoms, K = 2 (n + KN) + part
    {
        const int mrow = t & 127, half = t >> 7;
        const int at = atom0 + mrow;
        const uint32_t uz = at < v.nmove ? atoms[at].z : 0u;
        const int ksplit = (d.KS + 1) / 2;
        const int ks0 = half ? ksplit : 0, ks1 = half ? d.KS : ksplit;
        for (int ks = ks0; ks < ks1; ++ks) {
            uint32_t wh[8], wl[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int ni = ks * 8 + i;
                float c = 0.f, s = 0.f;
                if (at < v.nmove && ni < d.NN) phase((uint32_t)(ni - d.KN) * uz, c, s);
                elem_t hc, lc, hs, ls;
                tc::split(c, hc, lc);
                tc::split(s, hs, ls);
                wh[i] = pack2(hc, hs);
                wl[i] = pack2(lc, ls);
            }
            unsigned char* th = Asm + (0 * d.KS + ks) * tileB;
            unsigned char* tl = Asm + (1 * d.KS + ks) * tileB;
            *reinterpret_cast<uint4*>(th + tc::tile_off(mrow, 0)) = make_uint4(wh[0], wh[1], wh[2], wh[3]);
            *reinterpret_cast<uint4*>(th + tc::tile_off(mrow, 8)) = make_uint4(wh[4], wh[5], wh[6], wh[7]);
            *reinterpret_cast<uint4*>(tl + tc::tile_off(mrow, 0)) = make_uint4(wl[0], wl[1], wl[2], wl[3]);
            *reinterpret_cast<uint4*>(tl + tc::tile_off(mrow, 8)) = make_uint4(wl[4], wl[5], wl[6], wl[7]);
        }
    }
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = idesc_e(128, 128);
    const int NC = d.nchunk2;
    if (warp == 4) {
        if (lane == 0) {
            const uint32_t abase = tc::smem_u32(Asm), bbase = tc::smem_u32(Bsm);
            bool alive = true;
            for (int c = 0; c < NC && alive; ++c) {
                const int s = c & 1;
                if (c >= 2) alive = tc::mbar_wait(tc::smem_u32(&bars[2 + s]), ((c >> 1) - 1) & 1, err, 21);
                if (!alive) break;
                const uint32_t full = tc::smem_u32(&bars[s]);
                tc::mbar_expect_tx(full, imgBytes);
                tc::bulk_g2s(bbase + s * imgBytes, img + (size_t)c * imgBytes, halfBytes, full);
                tc::bulk_g2s(bbase + s * imgBytes + halfBytes, img + (size_t)c * imgBytes + halfBytes, halfBytes, full);
                alive = tc::mbar_wait(full, (c >> 1) & 1, err, 22);
                if (!alive) break;
                if (c >= 2) alive = tc::mbar_wait(tc::smem_u32(&bars[4 + s]), ((c >> 1) - 1) & 1, err, 23);
                if (!alive) break;
                tc::fence_after();
                const uint32_t dcol = tmem + s * 128;
                for (int ks = 0; ks < d.KS; ++ks) {
                    const uint64_t ah = tc::desc(abase + (0 * d.KS + ks) * tileB);
                    const uint64_t al = tc::desc(abase + (1 * d.KS + ks) * tileB);
                    const uint64_t bh = tc::desc(bbase + s * imgBytes + (0 * d.KS + ks) * tileB);
                    const uint64_t bl = tc::desc(bbase + s * imgBytes + (1 * d.KS + ks) * tileB);
                    tc::mma_bf16(dcol, ah, bh, idesc, ks > 0 ? 1u : 0u);
                    tc::mma_bf16(dcol, ah, bl, idesc, 1u);
                    tc::mma_bf16(dcol, al, bh, idesc, 1u);
                }
                tc::commit(tc::smem_u32(&bars[2 + s]));
            }
            // on a timeout, let issued work drain (bounded) before the block frees its TMEM
            if (!alive && NC > 0) tc::mbar_wait(tc::smem_u32(&bars[2 + ((NC - 1) & 1)]), ((NC - 1) >> 1) & 1, nullptr, 0);
        }
    } else if (warp < 4) {
        const int at = atom0 + t;
        const bool ok = at < v.nmove;
        uint4 rec = ok ? atoms[at] : make_uint4(0, 0, 0, 0);
        float fx = 0.f, fy = 0.f, fz = 0.f;
        bool alive = true;
        for (int c = 0; c < NC && alive; ++c) {
            const int s = c & 1;
            alive = tc::mbar_wait(tc::smem_u32(&bars[2 + s]), (c >> 1) & 1, err, 24);
            if (!alive) break;
            tc::fence_after();
            for (int half = 0; half < 2; ++half) {
                float val[64];
#pragma unroll
                for (int cc = 0; cc < 4; ++cc)
                    tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + s * 128 + half * 64 + cc * 16, val + cc * 16);
#pragma unroll
                for (int rr = 0; rr < 16; ++rr) {
                    const int row = c * 32 + half * 16 + rr;
                    const int4 rw = row < d.nrow ? rows[row] : make_int4(0, 0, 0, 0);
                    float ec, es;
                    phase((uint32_t)rw.x * rec.x + (uint32_t)rw.y * rec.y, ec, es);
                    const float s0 = ec * val[rr * 4 + 1] + es * val[rr * 4 + 0];
                    const float s1 = ec * val[rr * 4 + 3] + es * val[rr * 4 + 2];
                    fx += (d.px * (float)rw.x) * s0;
                    fy += (d.py * (float)rw.y) * s0;
                    fz += s1;
                }
            }
            tc::fence_before();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(tc::smem_u32(&bars[4 + s]));
        }
        if (ok && alive) {
            const double q = (double)__uint_as_float(rec.w) * (double)cmax[0];
            v.fx[at] += q * (double)fx;
            v.fy[at] += q * (double)fy;
            v.fz[at] += q * (double)d.pz * (double)fz;
        }
    }
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, 256);
    }
}

// ---------------------------------------------------------------------------------------------
// self test: D (128 x N) = A (128 x K) B^T (N x K) on one block, bf16 operands, fp32 out
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128, 1) k_umma_selftest(const float* A, const float* B, float* D, int N, int K,
                                                          int* err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 64);
    unsigned char* At = sm + 1024;
    unsigned char* Bt = At + 4096;
    const int t = threadIdx.x, warp = t >> 5;
    if (t == 0) {
        tc::mbar_init(tc::smem_u32(bar), 1);
        tc::mbar_fence_init();
    }
    if (warp == 0) tc::tmem_alloc(tc::smem_u32(tslot), 256);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    bool alive = true;
    for (int k0 = 0; k0 < K && alive; k0 += 16) {
        for (int e = t; e < 128 * 16; e += 128) {
            const int r = e >> 4, kk = e & 15;
            *reinterpret_cast<__nv_bfloat16*>(At + tc::tile_off(r, kk)) = __float2bfloat16_rn(A[r * K + k0 + kk]);
        }
        for (int e = t; e < N * 16; e += 128) {
            const int r = e >> 4, kk = e & 15;
            *reinterpret_cast<__nv_bfloat16*>(Bt + tc::tile_off(r, kk)) = __float2bfloat16_rn(B[r * K + k0 + kk]);
        }
        tc::fence_async_smem();
        __syncthreads();
        if (t == 0) {
            tc::fence_after();
            tc::mma_bf16(tmem, tc::desc(tc::smem_u32(At)), tc::desc(tc::smem_u32(Bt)), tc::idesc_bf16(128, N),
                         k0 > 0 ? 1u : 0u);
            tc::commit(tc::smem_u32(bar));
        }
        alive = tc::mbar_wait(tc::smem_u32(bar), (k0 >> 4) & 1, err, 31);
        __syncthreads();
    }
    tc::fence_after();
    for (int cc = 0; cc < N / 16; ++cc) {
        float val[16];
        tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + cc * 16, val);
        if (alive)
            for (int c = 0; c < 16; ++c) D[t * N + cc * 16 + c] = val[c];
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, 256);
    }
}

}  // namespace

int recip_tc_setup(Ctx& c) {
    View& v = c.v;
    KSet& ks = c.ks;
    TcPlan& p = c.tcp;
    p.KN = ks.knmax;
    p.NN = 2 * ks.knmax + 1;
    p.NP = (2 * p.NN + 15) / 16 * 16;
    p.KS = (2 * p.NN + 15) / 16;
    if (p.NP > 256) return set_err(&c, MDG_E_UNSUPPORTED, "knmax too large for the tensor-core reciprocal sum");
    p.ncols1 = p.NP <= 128 ? 128 : 256;
    p.mtiles = (ks.nrow + 127) / 128;
    p.nchunk2 = (ks.nrow + 31) / 32;
    const long want = (long)v.nmove * p.mtiles / (2 * 152);
    p.chunk1 = (int)std::max<long>(kG1, (want + kG1 - 1) / kG1 * kG1);
    p.nsplit1 = (v.nmove + p.chunk1 - 1) / p.chunk1;
    p.smem1 = 1024 + 2 * (8 * 4096 + 8 * p.NP * 32);
    p.smem2 = 1024 + 3 * 2 * p.KS * 4096;
    if (p.smem1 > 227 * 1024 || p.smem2 > 227 * 1024)
        return set_err(&c, MDG_E_UNSUPPORTED, "knmax too large for the tensor-core shared-memory tiles");
    c.d_tc_atoms = (uint4*)dalloc(c, sizeof(uint4) * std::max(v.nmove, 1));
    c.d_tc_img = (unsigned char*)dalloc(c, (size_t)std::max(p.nchunk2, 1) * 2 * p.KS * 4096);
    c.d_tc_cmax = (float*)dalloc(c, sizeof(float) * 4);
    if (c.alloc_failed) return set_err(&c, MDG_E_CUDA, "out of device memory for the tensor-core reciprocal sum");
    MDG_CUDA(cudaFuncSetAttribute(k_tc_sfac, cudaFuncAttributeMaxDynamicSharedMemorySize, p.smem1));
    MDG_CUDA(cudaFuncSetAttribute(k_tc_force, cudaFuncAttributeMaxDynamicSharedMemorySize, p.smem2));
    p.ready = true;
    return MDG_OK;
}

void recip_tc(Ctx& c) {
    const View& v = c.v;
    KSet& ks = c.ks;
    const TcPlan& p = c.tcp;
    if (ks.nk == 0 || v.nmove == 0) return;
    TcDims d{p.KN, p.NN, p.NP, p.KS, ks.nrow, p.nchunk2, (float)ks.pipix, (float)ks.pipiy, (float)ks.pipiz};
    k_tc_prep_atoms<<<(v.nmove + 255) / 256, 256, 0, c.stream>>>(v, c.d_tc_atoms);
    cudaMemsetAsync(ks.s, 0, sizeof(double2) * ks.nk, c.stream);
    k_tc_sfac<<<dim3(p.mtiles, p.nsplit1), kT, p.smem1, c.stream>>>(v, c.d_tc_atoms, p.chunk1, ks.row, ks.row_nlen, d,
                                                                    ks.s, (uint32_t)p.ncols1);
    recip_energy_launch(c);
    cudaMemsetAsync(c.d_tc_cmax, 0, sizeof(float), c.stream);
    k_tc_cmax<<<std::min((ks.nk + 255) / 256, 152), 256, 0, c.stream>>>(ks.c, ks.kvec, ks.nk, c.d_tc_cmax);
    const long total = (long)p.nchunk2 * p.KS * 128 * 16;
    k_tc_prep_c<<<(int)std::min<long>((total + 255) / 256, 152 * 8), 256, 0, c.stream>>>(ks.c, ks.row, ks.row_nlen, d,
                                                                                         c.d_tc_img, c.d_tc_cmax);
    k_tc_force<<<(v.nmove + 127) / 128, kT, p.smem2, c.stream>>>(v, c.d_tc_atoms, c.d_tc_img, ks.row, d, c.d_tc_cmax);
}

int umma_selftest(int n, int k, const float* a, const float* b, float* dout, std::string& err) {
    if (n < 16 || n > 256 || n % 16 || k < 16 || k % 16) {
        err = "selftest: n must be 16..256 (multiple of 16), k a multiple of 16";
        return MDG_E_ARG;
    }
    float *da = nullptr, *db = nullptr, *dd = nullptr;
    int* de = nullptr;
    auto fin = [&](int rc, const char* m) {
        if (da) cudaFree(da);
        if (db) cudaFree(db);
        if (dd) cudaFree(dd);
        if (de) cudaFree(de);
        if (rc) err = m;
        return rc;
    };
    if (cudaMalloc(&da, sizeof(float) * 128 * k) || cudaMalloc(&db, sizeof(float) * n * k) ||
        cudaMalloc(&dd, sizeof(float) * 128 * n) || cudaMalloc(&de, sizeof(int)))
        return fin(MDG_E_CUDA, "selftest: cudaMalloc failed");
    cudaMemcpy(da, a, sizeof(float) * 128 * k, cudaMemcpyHostToDevice);
    cudaMemcpy(db, b, sizeof(float) * n * k, cudaMemcpyHostToDevice);
    cudaMemset(de, 0, sizeof(int));
    const int smem = 1024 + 4096 + 256 * 32;
    if (cudaFuncSetAttribute(k_umma_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return fin(MDG_E_CUDA, "selftest: attribute");
    k_umma_selftest<<<1, 128, smem>>>(da, db, dd, n, k, de);
    if (cudaDeviceSynchronize() != cudaSuccess) return fin(MDG_E_CUDA, "selftest: kernel failed");
    int h = 0;
    cudaMemcpy(&h, de, sizeof(int), cudaMemcpyDeviceToHost);
    if (h) return fin(MDG_E_CUDA, "selftest: mbarrier wait timed out");
    cudaMemcpy(dout, dd, sizeof(float) * 128 * n, cudaMemcpyDeviceToHost);
    return fin(MDG_OK, "");
}

}  // namespace mdg
