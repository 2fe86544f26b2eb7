// recip_tc.cu - reciprocal-space Ewald sum on tcgen05 tensor cores (mixed precision path).
//
// The sum of force_fouri (src/forcem.f90:827-937) factorises over the k components:
//   S(l,m,n) = sum_j [q_j e^{i(l tx_j + m ty_j)}] e^{i n tz_j}                       (pass 1)
//   f_j      = q_j sum_{l,m} Im( e^{i(l tx_j + m ty_j)} T_j(l,m) ) (kx, ky) and
//              q_j kz sum_{l,m} Im( e^{i(l tx_j + m ty_j)} T'_j(l,m) ) with
//   T_j(l,m) = sum_n C(l,m,n) e^{i n tz_j},  T'_j(l,m) = sum_n n C(l,m,n) e^{i n tz_j}   (pass 2)
// with C = Ak conj(S + S_wall).  Both are complex matrix products written as real ones:
//   pass 1: the structure factor over K = atoms, split-K over atom chunks, in one of two forms:
//           n-side (k_tc_sfac2, used when 2 (2 KN + 1) <= 128): D[(re|im, n) lane, (l, m) row],
//           A = q e^{i n tz} in the 2x2 real block form, B = e^{i(l tx + m ty)}, N = 256 rows per
//           CTA; row-side (k_tc_sfac): D[(l, m) row, (re|im, n)], A = [Re | Im] of the row factor,
//           B = the 2x2 block form of e^{i n tz}, M = 128 rows per tile;
//   pass 2: D[atom, (row, T|T', re|im)] over K = (n, re|im), A = e^{i n tz} per atom (built once
//           per CTA), B = packed C chunks streamed with cp.async.bulk through a ring of K-step
//           slots, two TMEM accumulators double-buffered against the epilogue that forms
//           Im(e T) per row.
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

constexpr float kPhase = 1.4629180792671596e-09f;  // 2 pi / 2^32

// Operands are FP16 hi/lo splits (11 + 11 significant bits; BF16 would give 8 + 8); all are O(1)
// (phase factors, charges, and C(k) scaled per (l, m) row by the row's max |C| max(1, |n|)).
__device__ __forceinline__ uint32_t idesc_e(int M, int N) { return tc::idesc_f16(M, N); }

struct TcDims {
    int KN, NN;      // n range -KN..KN, NN = 2 KN + 1
    int NP;          // pass-1 N (2 NN rounded up to 16)
    int KS;          // pass-2 K steps (2 NN rounded up to 16, / 16)
    int nrow, nchunk2;
    float px, py, pz;
    int nst2;        // pass-2 slot groups of kPer2 K steps in shared memory (as many as fit)
};

__device__ __forceinline__ void phase(uint32_t u, float& c, float& s) {
    __sincosf((float)(int32_t)u * kPhase, &s, &c);
}


// ---------------------------------------------------------------------------------------------
// pass 1: structure factor
//
// One CTA owns TPC row tiles (TPC * 128 (l, m) rows; TPC = 4 when the accumulators fit TMEM) and a
// contiguous chunk of atoms, walked in groups of kGA = 16 atoms (one K step) through a 2-3 deep
// shared-memory ring:
//   producer warps (one thread per row): per group, phase tables e^{i m ty_j} (all m) and q_j e^{i l tx_j}
//       (the l values of the CTA's rows) by __sincosf of exact fixed-point phases, the B tiles
//       e^{i n tz_j} in the 2x2 real block form, then each thread its row's A entries
//       q_j e^{i l tx_j} e^{i m ty_j} = table products, split hi/lo and stored in the UMMA
//       canonical layout; arrive on full[s];
//   last warp, lane 0 (issuer): waits full[s], issues 3 (hi/lo) x 2 (re/im part) MMAs per tile,
//       commits to empty[s], which frees the stage for the producers.
// The accumulators (one per tile, N = NP columns) are written once, as FP32 partial sums per
// atom chunk, to part[split][col][row]; k_tc_sreduce adds the chunks in compensated FP32 and
// forms S(k), the energy terms, C(k) and the scale of the pass-2 operand (src/forcem.f90:879-917).
// ---------------------------------------------------------------------------------------------
constexpr int kGA = 16;                  // atoms per group (one K step)
constexpr int kMaxNL = 64;               // l values per CTA (table width; the last slot stays 0)
constexpr int kMaxItems = 4;             // table entries per producer thread and group

template <int TPC>
struct P1 {
    static constexpr int kProd = 128 * TPC;      // producer threads: one per CTA row
    static constexpr int kThreads = kProd + 32;  // + issuer warp
    static constexpr int kS = TPC >= 4 ? 2 : 3;  // ring depth
};

struct P1Layout {
    uint32_t a_bytes, b_tile, stage, tab_m, tab_l, off_stage, off_tab, total;
};

// tables: e^{i m ty} as float2 [atom][NM + 1] (slot NM = 0), q e^{i l tx} as float2 [atom][kMaxNL]
__host__ __device__ inline P1Layout p1_layout(int tpc, int stages, int NP, int NM) {
    P1Layout L;
    L.a_bytes = tpc * 4 * 4096;                         // [tile][p][h] 128 x 16 halves
    L.b_tile = (uint32_t)NP * 32;                       // NP x 16 halves
    L.stage = L.a_bytes + 4 * L.b_tile;                 // + [p][h] B tiles
    L.tab_m = (uint32_t)kGA * (NM + 1) * 8;
    L.tab_l = (uint32_t)kGA * kMaxNL * 8;
    L.off_stage = 1024;
    L.off_tab = L.off_stage + stages * L.stage;
    L.total = L.off_tab + 2 * (L.tab_m + L.tab_l);
    return L;
}

// Named barrier 1 over the producer warps with an AND of their flags (every producer reaches it on
// every group, so a timeout seen by one producer stops all of them together).
template <int NPROD>
__device__ __forceinline__ bool producers_all(bool ok) {
    uint32_t res;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.and.pred p, 1, %2, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(res)
        : "r"((uint32_t)ok), "n"(NPROD)
        : "memory");
    return res != 0;
}

__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// hi/lo FP16 split of two floats into packed halves
__device__ __forceinline__ void split2(float a, float b, uint32_t& hi, uint32_t& lo) {
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = pack_h2(a - hf.x, b - hf.y);
}

template <int TPC>
__global__ void __launch_bounds__(P1<TPC>::kThreads, 1)
    k_tc_sfac(View v, const uint4* __restrict__ atoms, int chunk, const int4* __restrict__ rows, TcDims d, int NM,
              int KM, float* __restrict__ part, int rtot, uint32_t ncols, float* __restrict__ rowsc) {
    constexpr int kProd = P1<TPC>::kProd, kS = P1<TPC>::kS;
    extern __shared__ __align__(1024) unsigned char sm[];
    const P1Layout L = p1_layout(TPC, kS, d.NP, NM);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    uint64_t* full = reinterpret_cast<uint64_t*>(sm);
    uint64_t* empty = full + kS;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 512);
    int* err = &v.status[ST_TC_TIMEOUT];
    const int a0 = blockIdx.y * chunk, a1 = min(v.nmove, a0 + chunk);
    const int ngroup = a1 > a0 ? (a1 - a0 + kGA - 1) / kGA : 0;
    const int row0 = blockIdx.x * (TPC * 128);
    const int rlast = min(row0 + TPC * 128, d.nrow) - 1;
    const int l_lo = rows[row0].x, nl = min(rows[rlast].x - l_lo + 1, kMaxNL - 1);
    const int NM1 = NM + 1;
    if (t == 0) {
        for (int i = 0; i < kS; ++i) {
            tc::mbar_init(tc::smem_u32(&full[i]), kProd);
            tc::mbar_init(tc::smem_u32(&empty[i]), 1);
        }
        tc::mbar_fence_init();
    }
    // zero the ring (B rows beyond 2 NN stay zero) and both table buffers (padding slots stay zero)
    for (uint32_t o = t * 16; o < L.total - L.off_stage; o += P1<TPC>::kThreads * 16)
        *reinterpret_cast<uint4*>(sm + L.off_stage + o) = make_uint4(0, 0, 0, 0);
    if (warp == 0) tc::tmem_alloc(tc::smem_u32(tslot), ncols);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t tcols = ncols / TPC;
    bool alive = true;
    if (warp == kProd / 32) {
        // ---------------- issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_e(128, d.NP);
            const uint64_t dS0 = tc::desc(tc::smem_u32(sm + L.off_stage));
            int committed = -1;
            for (int g = 0; g < ngroup && alive; ++g) {
                const int s = g % kS;
                alive = tc::mbar_wait(tc::smem_u32(&full[s]), (g / kS) & 1, err, 11);
                if (!alive) break;
                tc::fence_after();
                const uint64_t ds = dS0 + (uint64_t)((s * L.stage) >> 4);
                const uint64_t db = ds + (uint64_t)(L.a_bytes >> 4);
                // all products of one accumulator back to back: switching the accumulator between
                // consecutive MMAs roughly halves the issue rate
#pragma unroll
                for (int tile = 0; tile < TPC; ++tile) {
                    const uint32_t dcol = tmem + tile * tcols;
#pragma unroll
                    for (int p = 0; p < 2; ++p) {
                        const uint64_t bh = db + (uint64_t)(((p * 2 + 0) * L.b_tile) >> 4);
                        const uint64_t bl = db + (uint64_t)(((p * 2 + 1) * L.b_tile) >> 4);
                        const uint64_t ah = ds + (uint64_t)(((tile * 2 + p) * 2 + 0) * 256);
                        const uint64_t al = ds + (uint64_t)(((tile * 2 + p) * 2 + 1) * 256);
                        tc::mma_bf16(dcol, ah, bh, idesc, (g > 0 || p > 0) ? 1u : 0u);
                        tc::mma_bf16(dcol, ah, bl, idesc, 1u);
                        tc::mma_bf16(dcol, al, bh, idesc, 1u);
                    }
                }
                tc::commit(tc::smem_u32(&empty[s]));
                committed = g;
            }
            // on a timeout, let the issued MMAs drain (bounded) before the block frees its TMEM
            if (!alive && committed >= 0)
                tc::mbar_wait(tc::smem_u32(&empty[committed % kS]), (committed / kS) & 1, nullptr, 0);
        }
    } else {
        // ---------------- producers
        const int r = t;                                 // CTA row (tile = r / 128)
        const int row = row0 + r;
        if (blockIdx.y == 0 && row < d.nrow) rowsc[row] = 0.f;  // k_tc_sreduce takes the maximum
        int li = kMaxNL - 1, mi = NM;                    // zero slots for padding rows
        if (row < d.nrow) {
            const int4 rw = rows[row];
            li = min(rw.x - l_lo, kMaxNL - 2);
            mi = rw.y + KM;
        }
        const int tile = r >> 7, rr = r & 127;
        // this thread's table entries (the same every group): e^{i m ty} items, q e^{i l tx} items,
        // and B items (n, atom pair)
        const int nm_items = kGA * NM, nl_items = kGA * nl, nb_items = d.NN * (kGA / 2);
        // items packed as (atom << 16) | index, -1 when the thread has no such item
        int im_i[kMaxItems], il_i[kMaxItems], ib_i[kMaxItems];
#pragma unroll
        for (int k = 0; k < kMaxItems; ++k) {
            const int e = t + k * kProd;
            im_i[k] = e < nm_items ? ((e / NM) << 16) | (e % NM) : -1;
            il_i[k] = e < nl_items ? ((e / nl) << 16) | (e % nl) : -1;
            ib_i[k] = e < nb_items ? (((e / d.NN) * 2) << 16) | (e % d.NN) : -1;
        }
#define IM_J(k) (im_i[k] >> 16)
#define IM_M(k) (im_i[k] & 0xffff)
#define IL_J(k) (il_i[k] >> 16)
#define IL_L(k) (il_i[k] & 0xffff)
#define IB_J(k) (ib_i[k] >> 16)
#define IB_N(k) (ib_i[k] & 0xffff)
        // the atom fractions this thread's items need, loaded one group ahead so that the global
        // load latency overlaps the barrier and the A fill of the current group
        uint32_t pm[kMaxItems], plx[kMaxItems], plq[kMaxItems], pb0[kMaxItems], pb1[kMaxItems];
        auto prefetch = [&](int gb) {
#pragma unroll
            for (int k = 0; k < kMaxItems; ++k) {
                pm[k] = (im_i[k] >= 0 && gb + IM_J(k) < a1) ? __ldg(&atoms[gb + IM_J(k)].y) : 0u;
                plx[k] = plq[k] = 0u;
                if (il_i[k] >= 0 && gb + IL_J(k) < a1) {
                    const uint4 rec = __ldg(&atoms[gb + IL_J(k)]);
                    plx[k] = rec.x;
                    plq[k] = rec.w;
                }
                pb0[k] = (ib_i[k] >= 0 && gb + IB_J(k) < a1) ? __ldg(&atoms[gb + IB_J(k)].z) : 0u;
                pb1[k] = (ib_i[k] >= 0 && gb + IB_J(k) + 1 < a1) ? __ldg(&atoms[gb + IB_J(k) + 1].z) : 0u;
            }
        };
        if (ngroup > 0) prefetch(a0);
        for (int g = 0; g < ngroup; ++g) {
            const int s = g % kS;
            const int gb = a0 + g * kGA;
            float2* tm = reinterpret_cast<float2*>(sm + L.off_tab + (g & 1) * (L.tab_m + L.tab_l));
            float2* tl = reinterpret_cast<float2*>(reinterpret_cast<unsigned char*>(tm) + L.tab_m);
            bool ok = true;
            if (g >= kS) ok = tc::mbar_wait_warp(tc::smem_u32(&empty[s]), ((g / kS) - 1) & 1, err, 12);
            unsigned char* st = sm + L.off_stage + s * L.stage;
            unsigned char* bb = st + L.a_bytes;
            if (ok) {
#pragma unroll
                for (int k = 0; k < kMaxItems; ++k) {
                    if (im_i[k] >= 0) {
                        const int at = gb + IM_J(k);
                        float c = 0.f, sn = 0.f;
                        if (at < a1) phase((uint32_t)(IM_M(k) - KM) * pm[k], c, sn);
                        tm[IM_J(k) * NM1 + IM_M(k)] = make_float2(c, sn);
                    }
                    if (il_i[k] >= 0) {
                        const int at = gb + IL_J(k);
                        float c = 0.f, sn = 0.f;
                        if (at < a1) {
                            phase((uint32_t)(IL_L(k) + l_lo) * plx[k], c, sn);
                            const float q = __uint_as_float(plq[k]);
                            c *= q;
                            sn *= q;
                        }
                        tl[IL_J(k) * kMaxNL + IL_L(k)] = make_float2(c, sn);
                    }
                    if (ib_i[k] >= 0) {
                        const int jp = IB_J(k), ni = IB_N(k);
                        const uint32_t n = (uint32_t)(ni - d.KN);
                        float c0 = 0.f, s0 = 0.f, c1 = 0.f, s1 = 0.f;
                        if (gb + jp < a1) phase(n * pb0[k], c0, s0);
                        if (gb + jp + 1 < a1) phase(n * pb1[k], c1, s1);
                        uint32_t ch, cl, sh, sl;
                        split2(c0, c1, ch, cl);
                        split2(s0, s1, sh, sl);
                        const uint32_t ore = tc::tile_off(ni, jp), oim = tc::tile_off(d.NN + ni, jp);
                        // part 0: re row <- cos, im row <- sin ; part 1: re row <- -sin, im row <- cos
                        *reinterpret_cast<uint32_t*>(bb + 0 * L.b_tile + ore) = ch;
                        *reinterpret_cast<uint32_t*>(bb + 1 * L.b_tile + ore) = cl;
                        *reinterpret_cast<uint32_t*>(bb + 0 * L.b_tile + oim) = sh;
                        *reinterpret_cast<uint32_t*>(bb + 1 * L.b_tile + oim) = sl;
                        *reinterpret_cast<uint32_t*>(bb + 2 * L.b_tile + ore) = sh ^ 0x80008000u;
                        *reinterpret_cast<uint32_t*>(bb + 3 * L.b_tile + ore) = sl ^ 0x80008000u;
                        *reinterpret_cast<uint32_t*>(bb + 2 * L.b_tile + oim) = ch;
                        *reinterpret_cast<uint32_t*>(bb + 3 * L.b_tile + oim) = cl;
                    }
                }
            }
            if (g + 1 < ngroup) prefetch(gb + kGA);
            if (!producers_all<kProd>(ok)) {
                alive = false;
                break;
            }
            // A: this row's 16 entries q e^{i l tx} e^{i m ty} (zero for padding rows)
            uint32_t wrh[8], wrl[8], wih[8], wil[8];
#pragma unroll
            for (int j = 0; j < kGA; j += 2) {
                const float2 el0 = tl[j * kMaxNL + li], em0 = tm[j * NM1 + mi];
                const float2 el1 = tl[(j + 1) * kMaxNL + li], em1 = tm[(j + 1) * NM1 + mi];
                const float re0 = el0.x * em0.x - el0.y * em0.y, im0 = el0.x * em0.y + el0.y * em0.x;
                const float re1 = el1.x * em1.x - el1.y * em1.y, im1 = el1.x * em1.y + el1.y * em1.x;
                split2(re0, re1, wrh[j >> 1], wrl[j >> 1]);
                split2(im0, im1, wih[j >> 1], wil[j >> 1]);
            }
            unsigned char* ta = st + (tile * 2) * 2 * 4096;   // [tile][p][h]
            const uint32_t o0 = tc::tile_off(rr, 0), o8 = tc::tile_off(rr, 8);
            *reinterpret_cast<uint4*>(ta + 0 * 4096 + o0) = make_uint4(wrh[0], wrh[1], wrh[2], wrh[3]);
            *reinterpret_cast<uint4*>(ta + 0 * 4096 + o8) = make_uint4(wrh[4], wrh[5], wrh[6], wrh[7]);
            *reinterpret_cast<uint4*>(ta + 1 * 4096 + o0) = make_uint4(wrl[0], wrl[1], wrl[2], wrl[3]);
            *reinterpret_cast<uint4*>(ta + 1 * 4096 + o8) = make_uint4(wrl[4], wrl[5], wrl[6], wrl[7]);
            *reinterpret_cast<uint4*>(ta + 2 * 4096 + o0) = make_uint4(wih[0], wih[1], wih[2], wih[3]);
            *reinterpret_cast<uint4*>(ta + 2 * 4096 + o8) = make_uint4(wih[4], wih[5], wih[6], wih[7]);
            *reinterpret_cast<uint4*>(ta + 3 * 4096 + o0) = make_uint4(wil[0], wil[1], wil[2], wil[3]);
            *reinterpret_cast<uint4*>(ta + 3 * 4096 + o8) = make_uint4(wil[4], wil[5], wil[6], wil[7]);
            tc::fence_async_smem();
            tc::mbar_arrive(tc::smem_u32(&full[s]));
        }
#undef IM_J
#undef IM_M
#undef IL_J
#undef IL_L
#undef IB_J
#undef IB_N
        // all MMAs done -> accumulators to the partial-sum buffer
        if (ngroup > 0 && alive)
            alive = tc::mbar_wait_warp(tc::smem_u32(&empty[(ngroup - 1) % kS]), ((ngroup - 1) / kS) & 1, err, 13);
        tc::fence_after();
        const uint32_t tbase = tmem + ((uint32_t)((warp & 3) * 32) << 16) + tile * tcols;
        float* dst = part + (size_t)blockIdx.y * d.NP * rtot;
        for (int cc = 0; cc < d.NP / 16; ++cc) {
            float val[16];
            tc::tmem_ld16(tbase + cc * 16, val);
            if (!alive) continue;
#pragma unroll
            for (int c = 0; c < 16; ++c) dst[(size_t)(cc * 16 + c) * rtot + row] = ngroup > 0 ? val[c] : 0.f;
        }
        tc::fence_before();
    }
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, ncols);
    }
}

// ---------------------------------------------------------------------------------------------
// pass 1, n-side form (2 NN <= 128): the same structure factor with the roles of the operands
// swapped, D[(re|im, n) lane, (l, m) row] over K = atoms:
//   A (M = 128 lanes): q e^{i n tz} in the 2x2 real block form (part 0: cos / sin, part 1: -sin /
//     cos), lanes n (re) and NN + n (im), zero beyond 2 NN;
//   B (N = 256 rows): the real (part 0) and imaginary (part 1) parts of e^{i(l tx + m ty)}.
// Every tcgen05.mma is M = 128, N = 256 (128 cycles at the dense rate), 6 per group of 16 atoms
// (2 parts x hi*hi, hi*lo, lo*hi).  The CTA's atom records (a contiguous chunk, at most
// kMaxChunk1b atoms) arrive in shared memory by one bulk copy; then 16 producer warps (two
// threads per CTA row, 8 atoms each) write, group after group,
//   the B entries of their rows, each by one __sincosf of the exact fixed-point phase
//     l ux + m uy (mod 2^32), split hi/lo and stored in the UMMA layout, and
//   one A item (n, atom pair) per thread of the first 14 warps,
// and arrive on the stage's barrier.  A separate issuer warp (lane 0) waits for the 16 arrivals
// and issues the group's 6 MMAs: an issue waits for room in the tensor core's queue (about 640
// cycles of work), which stalled whichever producer warp issued.  Thread mappings keep the
// shared stores free of bank conflicts: a quarter warp writes 8 consecutive rows of one atom half
// (128 contiguous bytes); an A item warp covers 8 lanes x 4 atom pairs of one core matrix column.
// Accumulation: the tensor core's FP32 accumulation loses magnitude in every step (measured on
// this GPU: about 1.5e-8 of the running sum per accumulating MMA, always towards zero), so long
// chains bias S(k).  The chain is cut every G groups: it accumulates in TMEM columns 0-255, and
// one group into the next chain the producers add it in FP32 (round to nearest, unbiased) to the
// sums in TMEM columns 256-511; the issuer starts a chain only after all have done so.  At the
// end the sums are this CTA's partial [split][lane][row].
// Every wait is bounded; a timeout anywhere sets a shared abort flag that ends all waits.
// ---------------------------------------------------------------------------------------------
constexpr int kW1b = 16;                 // producer warps
constexpr int kT1b = kW1b * 32 + 32;     // + the MMA issuer warp (warp 16, lane 0)
constexpr int kS1b = 3;                  // stages (A and B of one group)
constexpr uint32_t kBSt = 4 * 8192;      // B: [p][h] tiles of 256 x 16 halves
constexpr uint32_t kASt = 4 * 4096;      // A: [p][h] tiles of 128 x 16 halves
constexpr uint32_t kSt1b = kBSt + kASt;
constexpr int kMaxChunk1b = 3072;        // atoms per CTA (records in shared memory: 48 KB)

struct P1bLayout {
    uint32_t off_st, off_rec, total;
};
__host__ __device__ inline P1bLayout p1b_layout() {
    P1bLayout L;
    L.off_st = 1024;
    L.off_rec = L.off_st + kS1b * kSt1b;
    L.total = L.off_rec + kMaxChunk1b * 16;
    return L;
}

// bounded mbarrier wait that also ends when another thread of the CTA has given up (*ab != 0)
__device__ __forceinline__ bool wait_ab(uint32_t addr, uint32_t parity, volatile int* ab, int* err, int tag) {
    for (int it = 0; it < (1 << 22); ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(addr), "r"(parity)
            : "memory");
        if (ok) return true;
        if (*ab) return false;
        if (it > 32) __nanosleep(it < 2048 ? 32 : 256);
    }
    *ab = 1;
    if (err) atomicCAS(err, 0, tag);
    return false;
}

// bounded mbarrier wait by a whole warp: every lane polls (one instruction, so the lanes agree),
// which keeps the warp converged; false once the abort flag is set or the limit is reached
__device__ __forceinline__ bool wait_all(uint32_t addr, uint32_t parity, volatile int* ab, int* err, int tag) {
    for (int it = 0; it < (1 << 22); ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(addr), "r"(parity)
            : "memory");
        if (__all_sync(0xffffffffu, ok != 0)) return true;
        if (*ab) return false;
        if (it > 32) __nanosleep(it < 2048 ? 32 : 256);
    }
    *ab = 1;
    if (err && (threadIdx.x & 31) == 0) atomicCAS(err, 0, tag);
    return false;
}

typedef unsigned long long f2t;  // two packed floats (f32x2)
__device__ __forceinline__ f2t f2pk(float a, float b) {
    f2t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 f2up(f2t r) {
    float2 v;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
    return v;
}
__device__ __forceinline__ f2t f2sub(f2t a, f2t b) {
    f2t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// hi/lo FP16 split of two floats with one packed subtraction
__device__ __forceinline__ void split2p(float a, float b, uint32_t& hi, uint32_t& lo) {
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    const float2 r = f2up(f2sub(f2pk(a, b), f2pk(hf.x, hf.y)));
    lo = pack_h2(r.x, r.y);
}

__global__ void __launch_bounds__(kT1b, 1)
    k_tc_sfac2(View v, const uint4* __restrict__ atoms, int chunk, const int4* __restrict__ rows, TcDims d,
               float* __restrict__ part, int rtot, int G, float* __restrict__ rowsc) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const P1bLayout L = p1b_layout();
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    uint64_t* full = reinterpret_cast<uint64_t*>(sm);          // [kS1b] stage written (16 warps)
    uint64_t* empty = full + kS1b;                              // [kS1b] stage's MMAs done
    uint64_t* chainDone = empty + kS1b;                         // accumulation chain's MMAs done
    uint64_t* drained = chainDone + 1;                          // chain added to the sums (16 warps)
    uint64_t* recbar = drained + 1;                             // records landed
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 512);
    volatile int* ab = reinterpret_cast<volatile int*>(sm + 520);
    int* err = &v.status[ST_TC_TIMEOUT];
    const int a0 = blockIdx.y * chunk, a1 = min(v.nmove, a0 + chunk);
    const int ngroup = a1 > a0 ? (a1 - a0 + kGA - 1) / kGA : 0;
    const int nchain = (ngroup + G - 1) / G;
    const int row0 = blockIdx.x * 256;
    if (t == 0) {
        for (int i = 0; i < kS1b; ++i) {
            tc::mbar_init(tc::smem_u32(&full[i]), kW1b);
            tc::mbar_init(tc::smem_u32(&empty[i]), 1);
        }
        tc::mbar_init(tc::smem_u32(chainDone), 1);
        tc::mbar_init(tc::smem_u32(drained), kW1b);
        tc::mbar_init(tc::smem_u32(recbar), 1);
        *ab = 0;
        tc::mbar_fence_init();
    }
    // zero the stages (A lanes beyond 2 NN stay zero) and the records (padding atoms: zero
    // charge, so zero A entries)
    for (uint32_t o = t * 16; o < L.total - L.off_st; o += kT1b * 16)
        *reinterpret_cast<uint4*>(sm + L.off_st + o) = make_uint4(0, 0, 0, 0);
    if (warp == 0) tc::tmem_alloc(tc::smem_u32(tslot), 512);
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    if (t == 0 && a1 > a0) {
        const uint32_t bytes = (uint32_t)(a1 - a0) * 16u;
        tc::mbar_expect_tx(tc::smem_u32(recbar), bytes);
        tc::bulk_g2s(tc::smem_u32(sm + L.off_rec), atoms + a0, bytes, tc::smem_u32(recbar));
    }
    if (warp < kW1b) {
        const uint4* recs = reinterpret_cast<const uint4*>(sm + L.off_rec);
        // B entries: a warp holds 16 consecutive rows, its half warps the two atom halves (a half
        // warp reads one record; a quarter warp stores 8 rows of one atom half, 128 contiguous bytes)
        const int h = (t >> 4) & 1;                   // atoms 8 h .. 8 h + 7 of each group
        const int r = ((t >> 5) << 4) | (t & 15);     // CTA row
        const int row = row0 + r;
        if (blockIdx.y == 0 && h == 0 && row < d.nrow) rowsc[row] = 0.f;  // k_tc_sreduce takes the maximum
        uint32_t lu = 0, mu = 0;                      // padding rows: phase 0 (their sums are not read)
        if (row < d.nrow) {
            const int4 rw = rows[row];
            lu = (uint32_t)rw.x;
            mu = (uint32_t)rw.y;
        }
        const uint32_t o8 = tc::tile_off(r, 8 * h);
        // A item: lane n (of a group of 8) and atom pair jp; a warp covers 8 lanes x 4 pairs of
        // one core matrix column
        const int ijp = (t & 3) | (((t >> 5) & 1) << 2);
        const int ini = ((t >> 6) << 3) | ((t >> 2) & 7);
        const bool has_item = ini < d.NN;
        const bool warp_items = __any_sync(0xffffffffu, has_item);  // warp-uniform
        const uint32_t ore = tc::tile_off(ini, 2 * ijp), oim = tc::tile_off(d.NN + ini, 2 * ijp);
        const uint32_t nfac = (uint32_t)(ini - d.KN);
        const int q = warp & 3, wq = warp >> 2;       // TMEM lane quarter, column block of the drains
        const uint32_t tq = tmem + ((uint32_t)(q * 32) << 16) + wq * 64;  // this warp's TMEM block
        bool alive = a1 <= a0 || wait_all(tc::smem_u32(recbar), 0, ab, err, 40);
        int nd = 0;                                    // chains added to the sums
        // chain c (columns 0-255) added in FP32 to the sums (columns 256-511), then the chain
        // accumulator is free for the next chain
        auto drain = [&](int c) {
            alive = wait_all(tc::smem_u32(chainDone), (uint32_t)(c & 1), ab, err, 41);
            if (!alive) return;
            tc::fence_after();
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) {
                uint32_t raw[16], sum[16];
                tc::tmem_ld16_nw(tq + cc * 16, raw);
                if (c > 0) tc::tmem_ld16_nw(tq + 256 + cc * 16, sum);
                tc::tmem_wait_ld();
                if (c > 0) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) raw[i] = __float_as_uint(__uint_as_float(raw[i]) + __uint_as_float(sum[i]));
                }
                tc::tmem_st16(tq + 256 + cc * 16, raw);
            }
            tc::tmem_wait_st();
            tc::fence_before();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(tc::smem_u32(drained));
        };
        int s = 0, gi = 0;                             // stage, group within the chain
        uint32_t rnd = 0;                             // parity of the stage's use
        for (int g = 0; g < ngroup && alive; ++g) {
            if (gi == 1 && g > G) {  // one group into chain c + 1: chain c's MMAs are (nearly) done
                drain(nd++);
                if (!alive) break;
            }
            if (g >= kS1b) alive = wait_all(tc::smem_u32(&empty[s]), rnd ^ 1u, ab, err, 43);
            if (!alive) break;
            unsigned char* st = sm + L.off_st + s * kSt1b;
            const uint4* rc = recs + g * kGA;
            uint32_t rh[4], rl[4], ih[4], il[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint2 r0 = *reinterpret_cast<const uint2*>(&rc[8 * h + 2 * k]);
                const uint2 r1 = *reinterpret_cast<const uint2*>(&rc[8 * h + 2 * k + 1]);
                float c0, s0, c1, s1;
                phase(lu * r0.x + mu * r0.y, c0, s0);
                phase(lu * r1.x + mu * r1.y, c1, s1);
                split2p(c0, c1, rh[k], rl[k]);
                split2p(s0, s1, ih[k], il[k]);
            }
            *reinterpret_cast<uint4*>(st + 0 * 8192 + o8) = make_uint4(rh[0], rh[1], rh[2], rh[3]);
            *reinterpret_cast<uint4*>(st + 1 * 8192 + o8) = make_uint4(rl[0], rl[1], rl[2], rl[3]);
            *reinterpret_cast<uint4*>(st + 2 * 8192 + o8) = make_uint4(ih[0], ih[1], ih[2], ih[3]);
            *reinterpret_cast<uint4*>(st + 3 * 8192 + o8) = make_uint4(il[0], il[1], il[2], il[3]);
            if (warp_items) {  // A: q e^{i n tz} of two atoms, lanes n and NN + n
                const uint2 z0 = *reinterpret_cast<const uint2*>(&rc[2 * ijp].z);
                const uint2 z1 = *reinterpret_cast<const uint2*>(&rc[2 * ijp + 1].z);
                float c0, s0, c1, s1;
                phase(nfac * z0.x, c0, s0);
                phase(nfac * z1.x, c1, s1);
                const float q0 = __uint_as_float(z0.y), q1 = __uint_as_float(z1.y);
                uint32_t ch, cl, sh, sl;
                split2p(q0 * c0, q1 * c1, ch, cl);
                split2p(q0 * s0, q1 * s1, sh, sl);
                if (has_item) {
                    unsigned char* as = st + kBSt;
                    *reinterpret_cast<uint32_t*>(as + 0 * 4096 + ore) = ch;  // part 0: cos / sin
                    *reinterpret_cast<uint32_t*>(as + 0 * 4096 + oim) = sh;
                    *reinterpret_cast<uint32_t*>(as + 1 * 4096 + ore) = cl;
                    *reinterpret_cast<uint32_t*>(as + 1 * 4096 + oim) = sl;
                    *reinterpret_cast<uint32_t*>(as + 2 * 4096 + ore) = sh ^ 0x80008000u;  // part 1: -sin / cos
                    *reinterpret_cast<uint32_t*>(as + 2 * 4096 + oim) = ch;
                    *reinterpret_cast<uint32_t*>(as + 3 * 4096 + ore) = sl ^ 0x80008000u;
                    *reinterpret_cast<uint32_t*>(as + 3 * 4096 + oim) = cl;
                }
            }
            tc::fence_async_smem();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(tc::smem_u32(&full[s]));
            alive = *ab == 0;  // one shared load for the warp: the same value in every lane
            if (++s == kS1b) {
                s = 0;
                rnd ^= 1u;
            }
            if (++gi == G) gi = 0;
        }
        while (alive && nd < nchain) drain(nd++);
        // this CTA's partial: lane (re|im, n) of the quarter, 64 consecutive rows
        const int lanei = q * 32 + lane;
        if (__shfl_sync(0xffffffffu, (alive && !*ab) ? 1 : 0, 0)) {  // warp-uniform: the loads are collective
            tc::fence_after();
            float4* dst = reinterpret_cast<float4*>(part + (size_t)blockIdx.y * d.NP * rtot + (size_t)lanei * rtot +
                                                    row0 + wq * 64);
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) {
                float sum[16];
                tc::tmem_ld16(tq + 256 + cc * 16, sum);
                if (lanei < 2 * d.NN)
#pragma unroll
                    for (int i = 0; i < 4; ++i)
                        dst[cc * 4 + i] = make_float4(sum[4 * i], sum[4 * i + 1], sum[4 * i + 2], sum[4 * i + 3]);
            }
        }
    } else if (lane == 0) {
        // the issuer: group g's 6 MMAs once the 16 producer warps have written its stage (and,
        // at a chain's start, added the previous chain to the sums); it produces nothing, so an
        // issue that waits for room in the MMA queue delays no entries
        const uint32_t idesc = idesc_e(128, 256);
        const uint64_t dS0 = tc::desc(tc::smem_u32(sm + L.off_st));
        int s = 0, gi = 0, c = 0, ls = -1;
        uint32_t rnd = 0, lr = 0;
        for (int g = 0; g < ngroup; ++g) {
            if (!wait_ab(tc::smem_u32(&full[s]), rnd, ab, err, 47)) break;
            if (gi == 0 && c > 0 && !wait_ab(tc::smem_u32(drained), (uint32_t)((c - 1) & 1), ab, err, 48)) break;
            tc::fence_after();
            const bool first = gi == 0, last = gi == G - 1 || g == ngroup - 1;
            const uint64_t ds = dS0 + (uint64_t)((s * kSt1b) >> 4);
#pragma unroll
            for (int p = 0; p < 2; ++p) {
                const uint64_t bh = ds + (uint64_t)(((p * 2 + 0) * 8192) >> 4);
                const uint64_t bl = ds + (uint64_t)(((p * 2 + 1) * 8192) >> 4);
                const uint64_t ah = ds + (uint64_t)((kBSt + (p * 2 + 0) * 4096) >> 4);
                const uint64_t al = ds + (uint64_t)((kBSt + (p * 2 + 1) * 4096) >> 4);
                tc::mma_bf16(tmem, ah, bh, idesc, (first && p == 0) ? 0u : 1u);
                tc::mma_bf16(tmem, ah, bl, idesc, 1u);
                tc::mma_bf16(tmem, al, bh, idesc, 1u);
            }
            tc::commit(tc::smem_u32(&empty[s]));
            if (last) tc::commit(tc::smem_u32(chainDone));
            ls = s;
            lr = rnd;
            if (++s == kS1b) {
                s = 0;
                rnd ^= 1u;
            }
            if (++gi == G) {
                gi = 0;
                ++c;
            }
        }
        // let the issued MMAs and the record copy finish (bounded) before the block frees its TMEM
        if (ls >= 0) tc::mbar_wait(tc::smem_u32(&empty[ls]), lr, nullptr, 0);
        if (a1 > a0) tc::mbar_wait(tc::smem_u32(recbar), 0, nullptr, 0);
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, 512);
    }
}

// Split-K reduction of pass 1 fused with the energy (src/forcem.f90:880-885,917), C(k) = Ak
// conj(S + S_wall) and the scale max |C| max(1, |n|) of the pass-2 operand.  A block takes 32
// consecutive (row, n) entries (row fastest, so each warp's loads are coalesced); warp g adds the
// partial sums of splits g, g + 8, ... in compensated FP32, and the eight partials are combined
// in a fixed order (deterministic), the result kept in FP64.
constexpr int kRedG = 8;
__global__ void __launch_bounds__(32 * kRedG) k_tc_sreduce(View v, const float* __restrict__ part, int nsplit,
                                                          int rtot, TcDims d, const int4* __restrict__ rows,
                                                          const int* __restrict__ nlen,
                                                          const double* __restrict__ ak,
                                                          const double2* __restrict__ qw, double2* S, double2* C,
                                                          float2* Cf, float* cmax, float* rowsc) {
    __shared__ float4 sh[kRedG][32];
    const int le = threadIdx.x & 31, g = threadIdx.x >> 5;
    const long total = (long)d.nrow * d.NN;
    const long e = (long)blockIdx.x * 32 + le;
    bool valid = e < total;
    int row = 0, ni = 0, n = 0;
    int4 rw = make_int4(0, 0, 0, 0);
    if (valid) {
        row = (int)(e % d.nrow);
        ni = (int)(e / d.nrow);
        rw = rows[row];
        n = ni - d.KN;
        valid = n >= rw.z && n < rw.z + nlen[row];
    }
    float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f;
    if (valid) {
#pragma unroll 4
        for (int sp = g; sp < nsplit; sp += kRedG) {
            const float* pp = part + (size_t)sp * d.NP * rtot;
            const float xr = pp[(size_t)ni * rtot + row] - cr;
            const float tr = sr + xr;
            cr = (tr - sr) - xr;
            sr = tr;
            const float xi = pp[(size_t)(d.NN + ni) * rtot + row] - ci;
            const float ti = si + xi;
            ci = (ti - si) - xi;
            si = ti;
        }
    }
    sh[g][le] = make_float4(sr, cr, si, ci);
    __syncthreads();
    double ew = 0.0, ll = 0.0;
    float mx = 0.f;
    if (g == 0 && valid) {
        double dr = 0.0, di = 0.0;
#pragma unroll
        for (int q = 0; q < kRedG; ++q) {
            const float4 p4 = sh[q][le];
            dr += (double)p4.x - (double)p4.y;
            di += (double)p4.z - (double)p4.w;
        }
        const int k = rw.w + n - rw.z;
        const double2 sv = make_double2(dr, di);
        S[k] = sv;
        const double2 st = make_double2(sv.x + qw[k].x, sv.y + qw[k].y);
        const double a = ak[k];
        ll = a * (sv.x * sv.x + sv.y * sv.y);
        ew = a * (st.x * st.x + st.y * st.y);
        const double2 cv = make_double2(a * st.x, -a * st.y);
        C[k] = cv;
        Cf[k] = make_float2((float)cv.x, (float)cv.y);
        const float w = (float)max(1, abs(n));
        mx = fmaxf(fabsf((float)cv.x), fabsf((float)cv.y)) * w;
        atomicMax(reinterpret_cast<unsigned int*>(&rowsc[row]), __float_as_uint(mx));
    }
    if (g == 0) {  // warp 0 holds the block's entries
        ew = warp_sum(ew);
        ll = warp_sum(ll);
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (le == 0) {
            if (ew != 0.0) atomicAdd(&v.acc[2 * v.nijt + ACC_UEWA], ew);
            if (ll != 0.0) atomicAdd(&v.acc[2 * v.nijt + ACC_EWQLL], ll);
            atomicMax(reinterpret_cast<unsigned int*>(cmax), __float_as_uint(mx));
        }
    }
}

// ---------------------------------------------------------------------------------------------
// C(k) packed as the pass-2 B operand, each row scaled by its own maximum (the epilogue
// multiplies it back).  Pass 2 takes the rows sorted by the K steps their n range
// covers (row2, nlen2), so that chunk c (rows kRC c .. kRC c + kRC - 1 of that order) multiplies
// only the K steps ks_lo .. ks_lo + nks - 1 its rows use (chunk2[c] = image byte offset, ks_lo,
// nks).  Columns col = 4 r_local + 2 t + comp (t: T or T', comp: re or im), K = 2 (n + KN) + part;
// the image of a chunk is [nks][hi | lo] tiles of N x 16, so that one K step (its hi and lo tiles)
// is one contiguous copy.  One thread per (K step, column, n).
// ---------------------------------------------------------------------------------------------
constexpr int kRC = 64;                 // rows per pass-2 chunk
constexpr int kNC2 = 4 * kRC;           // pass-2 MMA N
constexpr uint32_t kTile2 = kNC2 * 32;  // one N x 16 B tile (bytes)

__global__ void k_tc_prep_c(const float2* __restrict__ Cf, const int4* __restrict__ rows,
                            const int* __restrict__ nlen, const int4* __restrict__ chunks, TcDims d,
                            unsigned char* img, const float* __restrict__ rowsc, const int* __restrict__ rorig,
                            float* __restrict__ rsc2, double* frc, int zero_from, int nmove) {
    if (blockIdx.y == 0)  // forces of the atoms whose pass-2 tiles are cut into pieces
        for (int i = zero_from + blockIdx.x * blockDim.x + threadIdx.x; i < nmove; i += gridDim.x * blockDim.x) {
            frc[i] = 0.0;
            frc[nmove + i] = 0.0;
            frc[2 * nmove + i] = 0.0;
        }
    const int c = blockIdx.y;
    if (blockIdx.x == 0 && threadIdx.x < kRC) {  // the chunk's row scales, for the force epilogue
        const int ro = rorig[c * kRC + threadIdx.x];
        rsc2[c * kRC + threadIdx.x] = ro >= 0 ? rowsc[ro] : 0.f;
    }
    const int4 ch = chunks[c];
    const int nks = ch.z;
    const int total = nks * kNC2 * 8;
    unsigned char* base = img + ch.x;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int i8 = e & 7;
        const int col = (e >> 3) % kNC2;
        const int ksl = (e >> 3) / kNC2;
        const int row = c * kRC + (col >> 2), tt = (col >> 1) & 1, comp = col & 1;
        const int ni = (ch.y + ksl) * 8 + i8;
        float v0 = 0.f, v1 = 0.f;
        const int nl = nlen[row];
        if (nl > 0 && ni < d.NN) {
            const int4 rw = rows[row];
            const int n = ni - d.KN;
            if (n >= rw.z && n < rw.z + nl) {
                // each row's C scaled by its own max |n C|: under one scale for all rows the
                // large-k rows' C would fall below FP16's normal range
                const float sr = rowsc[rorig[row]];
                const float inv = sr > 0.f ? 1.0f / sr : 1.0f;
                const float2 cv = Cf[rw.w + n - rw.z];
                const float sc = (tt ? (float)n : 1.0f) * inv;
                const float cr = cv.x * sc, ci = cv.y * sc;
                v0 = comp == 0 ? cr : ci;   // part 0
                v1 = comp == 0 ? -ci : cr;  // part 1
            }
        }
        uint32_t hi, lo;
        split2(v0, v1, hi, lo);
        const uint32_t off = tc::tile_off(col, 2 * i8);
        *reinterpret_cast<uint32_t*>(base + (2 * ksl) * kTile2 + off) = hi;
        *reinterpret_cast<uint32_t*>(base + (2 * ksl + 1) * kTile2 + off) = lo;
    }
}

// ---------------------------------------------------------------------------------------------
// pass 2: forces
//
// One CTA per 128 atoms (M = 128).  The CTA builds A = e^{i n tz} of its atoms (K = 2 (n + KN) +
// part) once and walks the chunks of C: 64 rows each, N = 256 columns = T and T' x re/im of the 64
// rows, so an MMA reads 12 KB of shared memory per 128 cycles; with N = 128 (32-row chunks) it
// read 8 KB per 64 cycles, the whole shared-memory bandwidth, and with the image copies beside it
// ran at about half its rate.  A chunk's K steps stream through a ring of 16 KB slots (one K
// step's hi and lo tiles): a copier warp fills each slot as soon as the 3 MMAs that read it before
// are done, an issuer warp issues the 3 (hi/lo) products per K step into one of two TMEM
// accumulators (the issuer does nothing else: an issue waits for room in the tensor core's queue
// of about 640 cycles of work), and 16 epilogue warps (four per TMEM lane quarter, 16 rows of a
// chunk each) drain the accumulator of chunk c while chunk c + 1 runs.  Per row the epilogue forms
// Im(e^{i(l tx + m ty)} T) with the row phase advanced along m by a complex multiply (recomputed by
// __sincosf at rows flagged in the row table: every 8th row and each change of l).
// ---------------------------------------------------------------------------------------------
constexpr int kEW2 = 16;                  // epilogue warps
constexpr int kT2 = (kEW2 + 2) * 32;      // + the issuer warp (16) and the copier warp (17)
constexpr int kSlot2 = 2 * (int)kTile2;   // one K step of a chunk image: hi and lo tiles
constexpr int kPer2 = 3;                  // K steps per copy (a 1-D bulk copy costs about 400 ns
                                          // whatever its size up to tens of KB, and one thread's
                                          // copies run one after another: few large copies)

struct P2Layout {
    uint32_t a_bytes, off_a, off_ring, off_rows, off_rsc, off_red, off_ch, total;
    int nslot;
};

// A (hi, lo), the ring of K-step slots (groups of kPer2, as many groups as fit), the row table,
// the force partials of row parts 1-3, the chunk table
__host__ __device__ inline P2Layout p2_layout(int KS, int nrow_pad, int nslot) {
    P2Layout L;
    L.a_bytes = 2 * KS * 4096;                 // [h][ks] 128 x 16
    L.off_a = 1024;
    L.off_ring = L.off_a + L.a_bytes;
    L.nslot = nslot;
    L.off_rows = L.off_ring + nslot * kPer2 * kSlot2;
    L.off_rsc = L.off_rows + nrow_pad * 16;    // rows: (float l, float m, l | restart << 31, m)
    L.off_red = L.off_rsc + nrow_pad * 4;      // row scales of this evaluation
    L.off_ch = L.off_red + 3 * 3 * 128 * 4;
    L.total = L.off_ch + 16 * (nrow_pad / kRC);
    return L;
}
constexpr int kMaxSlot2 = 12;

__global__ void __launch_bounds__(kT2, 1) k_tc_force(View v, const uint4* __restrict__ atoms,
                                                     const unsigned char* __restrict__ img,
                                                     const int4* __restrict__ rows, const int4* __restrict__ chunks,
                                                     const int4* __restrict__ items, TcDims d,
                                                     const float* __restrict__ rsc_g, double* __restrict__ frc) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const P2Layout L = p2_layout(d.KS, d.nchunk2 * kRC, d.nst2);
    const int R = L.nslot;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    uint64_t* full = reinterpret_cast<uint64_t*>(sm);   // [R] slot group landed
    uint64_t* empty = full + kMaxSlot2;                  // [R] the group's MMAs done
    uint64_t* mdone = empty + kMaxSlot2;                 // [2] MMAs of the chunk done (accumulator ready)
    uint64_t* afree = mdone + 2;                         // [2] accumulator read out (16 epilogue warps)
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 512);
    float4* rlm = reinterpret_cast<float4*>(sm + L.off_rows);
    float* rsc = reinterpret_cast<float*>(sm + L.off_rsc);
    int4* chs = reinterpret_cast<int4*>(sm + L.off_ch);  // this item's chunks
    int* err = &v.status[ST_TC_TIMEOUT];
    const int4 item = items[blockIdx.x];  // atom tile, chunks [c0, c0 + NC), whole tile or piece
    const int atom0 = item.x * 128;
    const int c0 = item.y, NC = item.z - item.y;
    const int NCT = d.nchunk2;
    if (t == 0) {
        for (int b = 0; b < R; ++b) {
            tc::mbar_init(tc::smem_u32(&full[b]), 1);
            tc::mbar_init(tc::smem_u32(&empty[b]), 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(tc::smem_u32(&mdone[b]), 1);
            tc::mbar_init(tc::smem_u32(&afree[b]), kEW2);
        }
        tc::mbar_fence_init();
    }
    for (int c = t; c < NC; c += kT2) chs[c] = chunks[c0 + c];
    __syncthreads();
    if (warp == kEW2 + 1) {
        if (lane == 0) {
            // the copier: the item's chunk images are one contiguous byte range of U K steps; it
            // streams through R slot groups of kPer2 K steps, one bulk copy per group as soon as
            // the MMAs that read the group before are done; the first copies overlap the other
            // warps' set-up
            const uint32_t ring = tc::smem_u32(sm + L.off_ring);
            int U = 0;
            for (int c = 0; c < NC; ++c) U += chs[c].z;
            const unsigned char* src = NC > 0 ? img + chs[0].x : img;
            int grp = 0, ls = -1;
            uint32_t ph = 0, lph = 0;                // parity of the group's use
            for (int u0 = 0, j = 0; u0 < U; u0 += kPer2, ++j) {
                if (j >= R && !tc::mbar_wait(tc::smem_u32(&empty[grp]), ph ^ 1u, err, 21)) break;
                const uint32_t bytes = (uint32_t)(min(kPer2, U - u0) * kSlot2);
                const uint32_t fb = tc::smem_u32(&full[grp]);
                tc::mbar_expect_tx(fb, bytes);
                tc::bulk_g2s(ring + grp * (kPer2 * kSlot2), src + (size_t)u0 * kSlot2, bytes, fb);
                ls = grp;
                lph = ph;
                if (++grp == R) {
                    grp = 0;
                    ph ^= 1u;
                }
            }
            // the last copy lands (bounded) before the block can exit
            if (ls >= 0) tc::mbar_wait(tc::smem_u32(&full[ls]), lph, nullptr, 0);
        }
    } else {
        constexpr int kTS = (kEW2 + 1) * 32;  // threads of the set-up: all warps but the copier
        for (int r = t; r < NCT * kRC; r += kTS) {
            const int4 rw = r < d.nrow ? rows[r] : make_int4(0, 0, 0, 0);
            int restart = (r & 7) == 0 || r >= d.nrow;
            if (!restart) {
                const int4 pw = rows[r - 1];  // 0 < r < nrow here
                restart = pw.x != rw.x || pw.y + 1 != rw.y;
            }
            rlm[r] = make_float4((float)rw.x, (float)rw.y, __int_as_float(rw.x | (restart << 31)), __int_as_float(rw.y));
            rsc[r] = rsc_g[r];
        }
        if (warp == 0) tc::tmem_alloc(tc::smem_u32(tslot), 512);
        // A: e^{i n tz} of this block's atoms, K = 2 (n + KN) + part (the epilogue warps, a
        // quarter of the K steps each)
        if (t < kEW2 * 32) {
            const int mrow = t & 127, kq = t >> 7;
            const int at = atom0 + mrow;
            const uint32_t uz = at < v.nmove ? atoms[at].z : 0u;
            for (int ks = kq; ks < d.KS; ks += 4) {
                uint32_t wh[8], wl[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int ni = ks * 8 + i;
                    float c = 0.f, s = 0.f;
                    if (at < v.nmove && ni < d.NN) phase((uint32_t)(ni - d.KN) * uz, c, s);
                    split2(c, s, wh[i], wl[i]);
                }
                unsigned char* th = sm + L.off_a + (0 * d.KS + ks) * 4096;
                unsigned char* tlo = sm + L.off_a + (1 * d.KS + ks) * 4096;
                *reinterpret_cast<uint4*>(th + tc::tile_off(mrow, 0)) = make_uint4(wh[0], wh[1], wh[2], wh[3]);
                *reinterpret_cast<uint4*>(th + tc::tile_off(mrow, 8)) = make_uint4(wh[4], wh[5], wh[6], wh[7]);
                *reinterpret_cast<uint4*>(tlo + tc::tile_off(mrow, 0)) = make_uint4(wl[0], wl[1], wl[2], wl[3]);
                *reinterpret_cast<uint4*>(tlo + tc::tile_off(mrow, 8)) = make_uint4(wl[4], wl[5], wl[6], wl[7]);
            }
        }
        tc::fence_async_smem();
        tc::fence_before();
        tc::named_sync(2, kTS);
        tc::fence_after();
        const uint32_t tmem = *tslot;
        if (warp == kEW2) {
            if (lane == 0) {
                const uint32_t idesc = idesc_e(128, kNC2);
                const uint64_t dA0 = tc::desc(tc::smem_u32(sm + L.off_a)), dR0 = tc::desc(tc::smem_u32(sm + L.off_ring));
                bool alive = true;
                int grp = 0, pos = 0, u = 0, U = 0;   // slot group, K step within it, K steps issued, all
                uint32_t ph = 0;
                for (int c = 0; c < NC; ++c) U += chs[c].z;
                for (int c = 0; c < NC && alive; ++c) {
                    const int s = c & 1;              // accumulator
                    if (c >= 2) alive = tc::mbar_wait(tc::smem_u32(&afree[s]), ((c >> 1) - 1) & 1, err, 23);
                    if (!alive) break;
                    const uint32_t dcol = tmem + s * kNC2;
                    const int4 ch = chs[c];
                    for (int ksl = 0; ksl < ch.z; ++ksl) {
                        if (pos == 0) {
                            alive = tc::mbar_wait(tc::smem_u32(&full[grp]), ph, err, 22);
                            if (!alive) break;
                            tc::fence_after();
                        }
                        const int ks = ch.y + ksl;
                        const uint64_t ah = dA0 + (uint64_t)(ks * 256), al = dA0 + (uint64_t)((d.KS + ks) * 256);
                        const uint64_t bh = dR0 + (uint64_t)(((grp * kPer2 + pos) * kSlot2) >> 4), bl = bh + (uint64_t)(kTile2 >> 4);
                        tc::mma_bf16(dcol, ah, bh, idesc, ksl > 0 ? 1u : 0u);
                        tc::mma_bf16(dcol, ah, bl, idesc, 1u);
                        tc::mma_bf16(dcol, al, bh, idesc, 1u);
                        ++u;
                        if (++pos == kPer2 || u == U) {  // the group's last K step: free it once read
                            tc::commit(tc::smem_u32(&empty[grp]));
                            pos = 0;
                            if (++grp == R) {
                                grp = 0;
                                ph ^= 1u;
                            }
                        }
                    }
                    if (alive) tc::commit(tc::smem_u32(&mdone[s]));
                }
                // let the issued work finish (bounded) before the block frees its TMEM
                if (NC > 0) tc::mbar_wait(tc::smem_u32(&mdone[(NC - 1) & 1]), ((NC - 1) >> 1) & 1, nullptr, 0);
            }
        } else {
            // warp w reads TMEM lanes 32 (w & 3) .. + 31 (its atoms) and rows 16 (w >> 2) .. + 15 of
            // each chunk, 8 rows (32 columns) at a time
            const int quad = warp & 3, hf = warp >> 2;
            const int at = atom0 + quad * 32 + lane;
            const bool ok = at < v.nmove;
            const uint4 rec = ok ? atoms[at] : make_uint4(0, 0, 0, 0);
            float dyc, dys;
            phase(rec.y, dyc, dys);
            float fx = 0.f, fy = 0.f, fz = 0.f;
            bool alive = true;
            for (int c = 0; c < NC && alive; ++c) {
                const int s = c & 1;
                alive = tc::mbar_wait_warp(tc::smem_u32(&mdone[s]), (c >> 1) & 1, err, 24);
                if (!alive) break;
                tc::fence_after();
                float ec = 0.f, es = 0.f;
                const int cid = c0 + c;
#pragma unroll
                for (int half = 0; half < 2; ++half) {
                    uint32_t raw[32];
                    const uint32_t ta = tmem + ((uint32_t)(quad * 32) << 16) + s * kNC2 + hf * 64 + half * 32;
                    tc::tmem_ld16_nw(ta, raw);
                    tc::tmem_ld16_nw(ta + 16, raw + 16);
                    tc::tmem_wait_ld();
                    if (half == 1) {  // the accumulator is read out: chunk c + 2 may use it
                        tc::fence_before();
                        __syncwarp();
                        if (lane == 0) tc::mbar_arrive(tc::smem_u32(&afree[s]));
                    }
#pragma unroll
                    for (int rr = 0; rr < 8; ++rr) {
                        const int row = cid * kRC + hf * 16 + half * 8 + rr;
                        const float4 lm = rlm[row];
                        const float scr = rsc[row];
                        const int lb = __float_as_int(lm.z);
                        if (rr == 0 || lb < 0) {
                            phase((uint32_t)(lb & 0x7fffffff) * rec.x + (uint32_t)__float_as_int(lm.w) * rec.y, ec, es);
                        } else {
                            const float nc = ec * dyc - es * dys;
                            es = ec * dys + es * dyc;
                            ec = nc;
                        }
                        const float v0 = __uint_as_float(raw[rr * 4 + 0]), v1 = __uint_as_float(raw[rr * 4 + 1]);
                        const float v2 = __uint_as_float(raw[rr * 4 + 2]), v3 = __uint_as_float(raw[rr * 4 + 3]);
                        const float s0 = (ec * v1 + es * v0) * scr;
                        fx = fmaf(lm.x, s0, fx);
                        fy = fmaf(lm.y, s0, fy);
                        fz = fmaf(ec * v3 + es * v2, scr, fz);
                    }
                }
            }
            // the warps of row parts 1-3 hand their partial sums to those of part 0 through shared memory
            float* red = reinterpret_cast<float*>(sm + L.off_red);
            const int ra = quad * 32 + lane;
            if (hf > 0) {
                float* rp = red + (hf - 1) * 384;
                rp[ra] = alive ? fx : 0.f;
                rp[128 + ra] = alive ? fy : 0.f;
                rp[256 + ra] = alive ? fz : 0.f;
            }
            tc::named_sync(1, kEW2 * 32);
            if (hf == 0 && ok) {  // a whole tile's atoms have one writer: plain stores; pieces add
#pragma unroll
                for (int pp = 0; pp < 3; ++pp) {  // (a timed-out block leaves zeros and its status)
                    fx += red[pp * 384 + ra];
                    fy += red[pp * 384 + 128 + ra];
                    fz += red[pp * 384 + 256 + ra];
                }
                const double q = alive ? (double)__uint_as_float(rec.w) : 0.0;
                const double gx = q * (double)d.px * (double)fx, gy = q * (double)d.py * (double)fy,
                             gz = q * (double)d.pz * (double)fz;
                if (item.w) {
                    frc[at] = gx;
                    frc[v.nmove + at] = gy;
                    frc[2 * v.nmove + at] = gz;
                } else {
                    atomicAdd(&frc[at], gx);
                    atomicAdd(&frc[v.nmove + at], gy);
                    atomicAdd(&frc[2 * v.nmove + at], gz);
                }
            }
        }
    }
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_dealloc(*tslot, 512);
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

// Pass-1 launch plan: tpc row tiles per CTA (2 or 4) and mult x (152 / row-tile groups) atom
// splits (mult 2 is the default; the autotuner tries the others).  Returns nonzero when the
// combination does not fit (TMEM columns or table capacity).
// mult: CTAs about 76 mult per launch (one system alone: fill the GPU), or 0 for the fewest
// CTAs of about kThroughputChunk atoms each (a system among many in one graph, where the GPU is
// full anyway and each CTA's set-up is paid in SM time).
constexpr int kThroughputChunk = 1024;

int tc_plan_pass1(Ctx& c, int tpc, int mult) {
    View& v = c.v;
    KSet& ks = c.ks;
    TcPlan& p = c.tcp;
    const int nthr = std::max(1, (v.nmove + kThroughputChunk - 1) / kThroughputChunk);
    if (tpc == 1) {
        // n-side form: 2 NN lanes in one 128-lane accumulator, 256 rows per CTA, at most
        // kMaxChunk1b atoms per CTA (their records in shared memory)
        if (2 * p.NN > 128) return 1;
        const size_t smem = p1b_layout().total;
        if (smem > 227 * 1024) return 1;
        p.smem1 = (int)smem;
        p.tpc1 = 1;
        p.ncols1 = 512;
        p.grid1x = (ks.nrow + 255) / 256;
        p.rtot = p.grid1x * 256;
        p.nsplit1 = mult > 0 ? std::max(1, std::min(std::max(1, 76 * mult / p.grid1x), (v.nmove + kGA - 1) / kGA))
                             : nthr;
        p.nsplit1 = std::max(p.nsplit1, (v.nmove + kMaxChunk1b - 1) / kMaxChunk1b);
        p.chunk1 = (v.nmove + p.nsplit1 - 1) / p.nsplit1;
        p.chunk1 = std::max(kGA, (p.chunk1 + kGA - 1) / kGA * kGA);
        if (p.chunk1 > kMaxChunk1b) return 1;
        p.nsplit1 = std::max(1, (v.nmove + p.chunk1 - 1) / p.chunk1);
        p.mult1 = mult;
        p.G1 = 8;
        return 0;
    }
    if (tpc == 4 && p.NP > 128) return 1;
    if (kGA * p.NM > kMaxItems * 128 * tpc || kGA * (kMaxNL - 1) > kMaxItems * 128 * tpc ||
        p.NN * (kGA / 2) > kMaxItems * 128 * tpc)
        return 1;
    const size_t smem = tpc == 4 ? p1_layout(4, P1<4>::kS, p.NP, p.NM).total : p1_layout(2, P1<2>::kS, p.NP, p.NM).total;
    if (smem > 227 * 1024) return 1;
    p.smem1 = (int)smem;
    p.tpc1 = tpc;
    p.ncols1 = tpc * (p.NP <= 128 ? 128 : 256);
    p.grid1x = (ks.nrow + tpc * 128 - 1) / (tpc * 128);
    p.rtot = p.grid1x * tpc * 128;
    p.nsplit1 = mult > 0 ? std::max(1, std::min(std::max(1, 76 * mult / p.grid1x), (v.nmove + 127) / 128)) : nthr;
    p.chunk1 = (v.nmove + p.nsplit1 - 1) / p.nsplit1;
    p.chunk1 = std::max(kGA, (p.chunk1 + kGA - 1) / kGA * kGA);
    p.nsplit1 = std::max(1, (v.nmove + p.chunk1 - 1) / p.chunk1);
    p.mult1 = mult;
    return 0;
}

// Work items of pass 2 (one CTA each): whole atom tiles; with pieces, the tiles of the last,
// partial wave (all tiles when there are fewer than one per SM) are cut into pieces of about equal
// K-step work, so that the wave fills the SMs (a system alone); pieces add their forces
// atomically into forces zeroed by the operand-packing kernel before.
static std::vector<int4> tc_items2(const Ctx& c, bool pieces, int& zero) {
    const View& v = c.v;
    const TcPlan& p = c.tcp;
    const std::vector<int>& cks = p.h_chunk_ks;
    const int ntile = (v.nmove + 127) / 128, tail = ntile % 152;
    int ksum = 0;
    for (int cc = 0; cc < p.nchunk2; ++cc) ksum += cks[cc];
    const int S = pieces && tail > 0 ? std::min(152 / tail, std::max(1, p.nchunk2 / 2)) : 1;
    const int first = S >= 2 ? ntile - tail : ntile;
    std::vector<int4> items;
    for (int t = 0; t < first; ++t) items.push_back(make_int4(t, 0, p.nchunk2, 1));
    for (int t = first; t < ntile; ++t) {
        int c0 = 0, acc = 0;
        for (int piece = 1; piece <= S && c0 < p.nchunk2; ++piece) {
            int c1 = c0;
            const long target = (long)ksum * piece / S;
            while (c1 < p.nchunk2 && (acc + cks[c1] <= target || c1 == c0)) acc += cks[c1++];
            if (piece == S) {
                while (c1 < p.nchunk2) acc += cks[c1++];
            }
            items.push_back(make_int4(t, c0, c1, 0));
            c0 = c1;
        }
    }
    zero = std::min(first * 128, v.nmove);
    return items;
}

// Both item tables (pieces for the system alone, whole tiles for throughput) go to the device once,
// so that switching plans is host bookkeeping only.
static int tc_plan_items2(Ctx& c) {
    TcPlan& p = c.tcp;
    for (int k = 0; k < 2; ++k) {
        int zero = 0;
        const std::vector<int4> items = tc_items2(c, k == 0, zero);
        p.items2_k[k] = (int4*)dalloc(c, sizeof(int4) * std::max(items.size(), (size_t)1));
        if (c.alloc_failed) return set_err(&c, MDG_E_CUDA, "out of device memory for the tensor-core reciprocal sum");
        p.nitems2_k[k] = (int)items.size();
        p.zero2_k[k] = zero;
        if (!items.empty())
            MDG_CUDA(cudaMemcpy(p.items2_k[k], items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice));
    }
    p.items2 = p.items2_k[0];
    p.nitems2 = p.nitems2_k[0];
    p.zero2 = p.zero2_k[0];
    return MDG_OK;
}

int recip_tc_throughput(Ctx& c, bool on) {
    TcPlan& p = c.tcp;
    if (!p.ready || on == p.throughput) return MDG_OK;
    if (on) p.mult_alone = p.mult1;
    if (tc_plan_pass1(c, p.tpc1, on ? 0 : p.mult_alone))
        return set_err(&c, MDG_E_UNSUPPORTED, "tensor-core plan");
    const int k = on ? 1 : 0;
    p.items2 = p.items2_k[k];
    p.nitems2 = p.nitems2_k[k];
    p.zero2 = p.zero2_k[k];
    p.throughput = on;
    drop_graphs(c);
    return MDG_OK;
}

int recip_tc_setup(Ctx& c) {
    View& v = c.v;
    KSet& ks = c.ks;
    TcPlan& p = c.tcp;
    p.KN = ks.knmax;
    p.NN = 2 * ks.knmax + 1;
    p.NP = (2 * p.NN + 15) / 16 * 16;
    p.KS = (2 * p.NN + 15) / 16;
    p.KM = ks.kmmax;
    p.NM = 2 * ks.kmmax + 1;
    if (p.NP > 256) return set_err(&c, MDG_E_UNSUPPORTED, "knmax too large for the tensor-core reciprocal sum");
    if (ks.klmax + 1 > kMaxNL - 1) return set_err(&c, MDG_E_UNSUPPORTED, "klmax too large for the tensor-core reciprocal sum");
    // the n-side form where it applies, else the row-side form with 4 or 2 row tiles per CTA
    const int tpc0 = !tc_plan_pass1(c, 1, 2) ? 1 : p.NP <= 128 ? 4 : 2;
    if (tc_plan_pass1(c, tpc0, 2) && tc_plan_pass1(c, 2, 2))
        return set_err(&c, MDG_E_UNSUPPORTED, "k range too large for the tensor-core table fill");
    // the partial-sum buffer is sized for the largest split the autotuner may choose
    size_t part_max = 0;
    for (int tpc : {1, 2, 4})
        for (int m : {0, 1, 2, 4})
            if (!tc_plan_pass1(c, tpc, m)) part_max = std::max(part_max, (size_t)p.nsplit1 * p.NP * p.rtot);
    if (tc_plan_pass1(c, tpc0, 2) && tc_plan_pass1(c, 2, 2)) return set_err(&c, MDG_E_UNSUPPORTED, "tensor-core plan");
    p.mtiles = (ks.nrow + 127) / 128;
    p.nchunk2 = (ks.nrow + kRC - 1) / kRC;
    p.nst2 = kMaxSlot2;  // slot groups of the pass-2 ring: as many as fit
    while (p.nst2 > 2 && p2_layout(p.KS, p.nchunk2 * kRC, p.nst2).total > 227 * 1024) --p.nst2;
    p.smem2 = (int)p2_layout(p.KS, p.nchunk2 * kRC, p.nst2).total;
    if (p.smem2 > 227 * 1024)
        return set_err(&c, MDG_E_UNSUPPORTED, "k range too large for the tensor-core shared-memory tiles");
    // pass-2 row order: rows sorted by the K steps of their n range, so that a chunk of kRC rows
    // runs only the K steps its rows need (the n range shrinks towards the edge of the k sphere)
    {
        const int nr = ks.nrow, nrp = p.nchunk2 * kRC;
        std::vector<int> klo(nr), khi(nr), order(nr);
        for (int r = 0; r < nr; ++r) {
            const int n0 = ks.h_row[r].z, n1 = n0 + ks.h_nlen[r] - 1;
            klo[r] = (2 * (n0 + p.KN)) / 16;
            khi[r] = (2 * (n1 + p.KN) + 1) / 16;
            order[r] = r;
        }
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            const int wa = khi[a] - klo[a], wb = khi[b] - klo[b];
            return wa != wb ? wa > wb : klo[a] < klo[b];
        });
        std::vector<int4> row2(nrp, make_int4(0, 0, 0, 0)), chunk2(p.nchunk2);
        std::vector<int> nlen2(nrp, 0), rorig2(nrp, -1);
        size_t off = 0;
        for (int cc = 0; cc < p.nchunk2; ++cc) {
            int lo = 1 << 30, hi = -1;
            for (int k = cc * kRC; k < std::min(nr, (cc + 1) * kRC); ++k) {
                const int r = order[k];
                row2[k] = ks.h_row[r];
                nlen2[k] = ks.h_nlen[r];
                rorig2[k] = r;
                lo = std::min(lo, klo[r]);
                hi = std::max(hi, khi[r]);
            }
            const int nks = hi - lo + 1;
            chunk2[cc] = make_int4((int)off, lo, nks, 0);
            off += (size_t)2 * nks * kTile2;
        }
        p.img_bytes = off;
        p.h_chunk_ks.resize(p.nchunk2);
        for (int cc = 0; cc < p.nchunk2; ++cc) p.h_chunk_ks[cc] = chunk2[cc].z;
        const int rc = tc_plan_items2(c);
        if (rc) return rc;
        p.rorig2 = (int*)dalloc(c, sizeof(int) * std::max(nrp, 1));
        p.rsc2 = (float*)dalloc(c, sizeof(float) * std::max(nrp, 1));
        p.rowsc = (float*)dalloc(c, sizeof(float) * std::max(nr, 1));
        p.row2 = (int4*)dalloc(c, sizeof(int4) * std::max(nrp, 1));
        p.nlen2 = (int*)dalloc(c, sizeof(int) * std::max(nrp, 1));
        p.chunk2 = (int4*)dalloc(c, sizeof(int4) * std::max(p.nchunk2, 1));
        if (c.alloc_failed) return set_err(&c, MDG_E_CUDA, "out of device memory for the tensor-core reciprocal sum");
        if (nrp > 0) {
            MDG_CUDA(cudaMemcpy(p.row2, row2.data(), sizeof(int4) * nrp, cudaMemcpyHostToDevice));
            MDG_CUDA(cudaMemcpy(p.nlen2, nlen2.data(), sizeof(int) * nrp, cudaMemcpyHostToDevice));
            MDG_CUDA(cudaMemcpy(p.chunk2, chunk2.data(), sizeof(int4) * p.nchunk2, cudaMemcpyHostToDevice));
            MDG_CUDA(cudaMemcpy(p.rorig2, rorig2.data(), sizeof(int) * nrp, cudaMemcpyHostToDevice));
            MDG_CUDA(cudaMemset(p.rsc2, 0, sizeof(float) * nrp));
        }
    }
    c.d_tc_atoms = (uint4*)dalloc(c, sizeof(uint4) * std::max(v.nmove, 1));
    c.d_tc_img = (unsigned char*)dalloc(c, std::max<size_t>(p.img_bytes, 16));
    c.d_tc_cmax = (float*)dalloc(c, sizeof(float) * 4);
    c.d_tc_part = (float*)dalloc(c, sizeof(float) * std::max<size_t>(part_max, 1));
    c.d_tc_cf = (float2*)dalloc(c, sizeof(float2) * std::max(ks.nk, 1));
    c.d_frc = (double*)dalloc(c, sizeof(double) * 3 * std::max(v.nmove, 1));
    if (c.alloc_failed) return set_err(&c, MDG_E_CUDA, "out of device memory for the tensor-core reciprocal sum");
    MDG_CUDA(allow_max_smem(k_tc_sfac2));
    MDG_CUDA(allow_max_smem(k_tc_sfac<4>));
    MDG_CUDA(allow_max_smem(k_tc_sfac<2>));
    MDG_CUDA(allow_max_smem(k_tc_force));
    p.ready = true;
    return MDG_OK;
}

void recip_tc(Ctx& c) {
    const View& v = c.v;
    KSet& ks = c.ks;
    const TcPlan& p = c.tcp;
    if (ks.nk == 0 || v.nmove == 0) return;
    TcDims d{p.KN, p.NN, p.NP, p.KS, ks.nrow, p.nchunk2, (float)ks.pipix, (float)ks.pipiy, (float)ks.pipiz, p.nst2};
    // c.d_tc_atoms was filled, and c.d_tc_cmax cleared, by the packing kernel of this evaluation
    if (p.tpc1 == 1)
        k_tc_sfac2<<<dim3(p.grid1x, p.nsplit1), kT1b, p.smem1, c.stream>>>(
            v, c.d_tc_atoms, p.chunk1, ks.row, d, c.d_tc_part, p.rtot, p.G1, p.rowsc);
    else if (p.tpc1 == 4)
        k_tc_sfac<4><<<dim3(p.grid1x, p.nsplit1), P1<4>::kThreads, p.smem1, c.stream>>>(
            v, c.d_tc_atoms, p.chunk1, ks.row, d, p.NM, p.KM, c.d_tc_part, p.rtot, (uint32_t)p.ncols1, p.rowsc);
    else
        k_tc_sfac<2><<<dim3(p.grid1x, p.nsplit1), P1<2>::kThreads, p.smem1, c.stream>>>(
            v, c.d_tc_atoms, p.chunk1, ks.row, d, p.NM, p.KM, c.d_tc_part, p.rtot, (uint32_t)p.ncols1, p.rowsc);
    const long nred = (long)ks.nrow * p.NN;
    k_tc_sreduce<<<(int)((nred + 31) / 32), 32 * kRedG, 0, c.stream>>>(
        v, c.d_tc_part, p.nsplit1, p.rtot, d, ks.row, ks.row_nlen, ks.ak, ks.qw, ks.s, ks.c, c.d_tc_cf, c.d_tc_cmax,
        p.rowsc);
    const int per_chunk = p.KS * kNC2 * 8;  // elements of the widest chunk image
    k_tc_prep_c<<<dim3((per_chunk + 255) / 256, p.nchunk2), 256, 0, c.stream>>>(
        c.d_tc_cf, p.row2, p.nlen2, p.chunk2, d, c.d_tc_img, p.rowsc, p.rorig2, p.rsc2, c.d_frc, p.zero2, v.nmove);
    k_tc_force<<<p.nitems2, kT2, p.smem2, c.stream>>>(v, c.d_tc_atoms, c.d_tc_img, p.row2, p.chunk2, p.items2, d,
                                                      p.rsc2, c.d_frc);
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
    if (allow_max_smem(k_umma_selftest) != cudaSuccess)
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
