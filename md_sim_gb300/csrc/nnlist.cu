// nnlist.cu - Verlet list rebuild on the GPU (replaces nnlist_init/nnlist_make,
// src/nnlist.f90:14-165) and the rebuild trigger of force_real (src/forcem.f90:245-250).
//
// The reference filters a stored O(heads^2) candidate list.  Here heads are binned into a cell
// grid whose cells are at least rskin wide, so every pair the reference keeps lies in the same
// or a neighbouring cell.  Candidates from the 27 (or fewer) cells pass a conservative FP32
// test on wrapped coordinates and then the reference's own FP64 test, evaluated with the same
// roundings (separate multiplies and adds, anint = round half away from zero), so the kept set
// is identical to the reference's.  Pairs are stored under the lower atom index as in
// list1/list2 (i < j); head-wall pairs under the head.  The *_b kernels run the same block bodies
// for many systems in one launch each (replica batches).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "ctx.h"

namespace mdg {

namespace {

constexpr int kNT = 256;

__device__ __forceinline__ int cell_coord(double w, int d, const Grid& g) {
    int c = (int)floor((w - g.org[d]) / g.cs[d]);
    return min(max(c, 0), g.nc[d] - 1);
}

__device__ __forceinline__ double wrap(double x, double l, int periodic) {
    return periodic ? x - l * floor(x / l) : x;
}

// Max squared displacement since the last rebuild; sets the rebuild flag.
__global__ void k_trigger(View v, int force) {
    double m = 0.0;
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
        m = fmax(m, a * a + b * b + c * c);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&v.acc[2 * v.nijt + ACC_MAXD], m);
    (void)force;
}

__global__ void k_trigger_decide(View v, int force) {
    const double aux = fmax(v.acc[2 * v.nijt + ACC_MAXD], v.dshsq);
    v.status[ST_REBUILD] = (force || v.status[ST_FORCE_RB] || 4.0 * aux > v.skin * v.skin) ? 1 : 0;
    v.status[ST_FORCE_RB] = 0;
    v.acc[2 * v.nijt + ACC_MAXD] = 0.0;
}

// The list build's kernels are written as block bodies with an explicit block index and block
// count, so that one launch can serve several systems (replica batches: each block finds its system
// and its block within that system's grid, the same grid a launch for that system alone has).

// Bin heads: cell index + count; saves the reference positions of the rebuild.
__device__ __forceinline__ void bin_heads(const View& v, const Grid& g, int* head_cell, int* cell_count,
                                          double4* hpos, int bid, int nblk) {
    if (!v.status[ST_REBUILD]) return;
    const int h = bid * blockDim.x + threadIdx.x;
    if (h < v.nheads) {
        const int a = v.head_atom[h];
        const double wx = wrap(v.x[a], v.lx, g.periodic[0]);
        const double wy = wrap(v.y[a], v.ly, g.periodic[1]);
        const double wz = wrap(v.z[a], v.lz, g.periodic[2]);
        const int c = (cell_coord(wz, 2, g) * g.nc[1] + cell_coord(wy, 1, g)) * g.nc[0] + cell_coord(wx, 0, g);
        head_cell[h] = c;
        hpos[h] = make_double4(wx, wy, wz, 0.0);
        atomicAdd(&cell_count[c], 1);
    }
    // reference positions (src/nnlist.f90:99-119)
    for (int i = h; i < v.nrig; i += nblk * blockDim.x) {
        v.ocx[i] = v.cx[i];
        v.ocy[i] = v.cy[i];
        v.ocz[i] = v.cz[i];
    }
    for (int i = h; i < v.nmove - v.nriga; i += nblk * blockDim.x) {
        v.ox[i] = v.x[i + v.nriga];
        v.oy[i] = v.y[i + v.nriga];
        v.oz[i] = v.z[i + v.nriga];
    }
}

__global__ void k_bin_heads(View v, Grid g, int* head_cell, int* cell_count, double4* hpos) {
    bin_heads(v, g, head_cell, cell_count, hpos, blockIdx.x, gridDim.x);
}

// Exclusive scan of the cell counts (one block) -> cell_start; resets counts to use as cursors.
__device__ __forceinline__ void scan_cells(const View& v, int ncell, int* cell_count, int* cell_start) {
    if (!v.status[ST_REBUILD]) return;
    __shared__ int carry;
    __shared__ int part[kNT];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < ncell; base += kNT) {
        const int i = base + threadIdx.x;
        const int val = i < ncell ? cell_count[i] : 0;
        part[threadIdx.x] = val;
        __syncthreads();
        for (int o = 1; o < kNT; o <<= 1) {
            int t = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
            __syncthreads();
            part[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < ncell) {
            cell_start[i] = carry + part[threadIdx.x] - val;
            cell_count[i] = 0;
        }
        __syncthreads();
        if (threadIdx.x == kNT - 1) carry += part[kNT - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) cell_start[ncell] = carry;
}

__global__ void k_scan_cells(View v, int ncell, int* cell_count, int* cell_start) {
    scan_cells(v, ncell, cell_count, cell_start);
}

__device__ __forceinline__ void scatter_heads(const View& v, const int* head_cell, int* cell_count,
                                              const int* cell_start, const double4* hpos, float4* cpos, int bid) {
    if (!v.status[ST_REBUILD]) return;
    const int h = bid * blockDim.x + threadIdx.x;
    if (h >= v.nheads) return;
    const int c = head_cell[h];
    const int slot = cell_start[c] + atomicAdd(&cell_count[c], 1);
    const double4 p = hpos[h];
    cpos[slot] = make_float4((float)p.x, (float)p.y, (float)p.z, __int_as_float(v.head_atom[h]));
}

__global__ void k_scatter_heads(View v, const int* head_cell, int* cell_count, const int* cell_start,
                                const double4* hpos, float4* cpos) {
    scatter_heads(v, head_cell, cell_count, cell_start, hpos, cpos, blockIdx.x);
}

__device__ __forceinline__ bool excluded(const View& v, int i, int j) {
    for (int k = v.excl_off[i]; k < v.excl_off[i + 1]; ++k)
        if (v.excl[k] == j) return true;
    return false;
}

// Reference test of src/nnlist.f90:124-130 with identical rounding.
__device__ __forceinline__ bool keep_pair(const View& v, double xi, double yi, double zi, double xj,
                                          double yj, double zj) {
    const double dx = minimg(__dsub_rn(xi, xj), v.lx, v.lxi);
    const double dy = minimg(__dsub_rn(yi, yj), v.ly, v.lyi);
    double dz = __dsub_rn(zi, zj);
    if (v.pbcz) dz = minimg(dz, v.lz, v.lzi);
    return dist2_exact(dx, dy, dz) < v.rskinsq;
}

__device__ __forceinline__ float fmin_img(float d, float l, float li, int periodic) {
    return periodic ? d - l * rintf(d * li) : d;
}

// Kept partners of one warp, staged in shared memory and written out in whole 128-byte lines
// (appending a few entries per ballot straight to global memory wrote partial lines).
constexpr int kStage = 128;

struct WarpOut {
    int* buf;  // kStage entries of shared memory
    int nbuf = 0, flushed = 0;
    __device__ __forceinline__ void flush(int* out, int cap, int lane) {
        for (int k = lane; k < nbuf; k += 32) {
            const int pos = flushed + k;
            if (pos < cap) out[pos] = buf[k];
        }
        flushed += nbuf;
        nbuf = 0;
        __syncwarp();
    }
    __device__ __forceinline__ void push(bool keep, int ja, unsigned m, int* out, int cap, int lane) {
        const int np = __popc(m);
        if (nbuf + np > kStage) flush(out, cap, lane);
        if (keep) buf[nbuf + __popc(m & ((1u << lane) - 1u))] = ja;
        nbuf += np;
        __syncwarp();
    }
    __device__ __forceinline__ int total() const { return flushed + nbuf; }
};

// One warp per head: the warp walks the neighbouring cells, lanes test 32 candidates at a time
// and the kept partners (j > i) are appended in order with a ballot.
__device__ __forceinline__ void build_hh(const View& v, const Grid& g, const int* cell_start, const float4* cpos,
                                         const double4* hpos, int* cell_count, int bid, int nblk) {
    if (!v.status[ST_REBUILD]) return;
    // the binning counts go back to zero for the next rebuild (zeroed at allocation)
    for (int i = bid * blockDim.x + threadIdx.x; i < g.ncell; i += nblk * blockDim.x) cell_count[i] = 0;
    const int lane = threadIdx.x & 31;
    const int h = (bid * blockDim.x + threadIdx.x) >> 5;
    if (h >= v.nheads) return;
    const int ia = v.head_atom[h];
    const double4 pw = hpos[h];
    const float px = (float)pw.x, py = (float)pw.y, pz = (float)pw.z;
    const double xi = v.x[ia], yi = v.y[ia], zi = v.z[ia];
    const float lxf = (float)v.lx, lyf = (float)v.ly, lzf = (float)v.lz;
    const float lxif = 1.0f / lxf, lyif = 1.0f / lyf, lzif = 1.0f / lzf;
    // FP32 distances of the binned positions are within ~1e-3 A^2 of the FP64 ones; only pairs
    // inside the shell [lim_lo, lim_hi] around rskinsq need the exact FP64 test (the FP64 pipe
    // is narrow on this part, so it is kept off the bulk of the candidates)
    const float lim_hi = (float)v.rskinsq * 1.0001f + 0.05f;
    const float lim_lo = (float)v.rskinsq * 0.9999f - 0.05f;
    const int cx = cell_coord(pw.x, 0, g), cy = cell_coord(pw.y, 1, g), cz = cell_coord(pw.z, 2, g);
    const bool surf_i = ia >= v.nliqa;
    __shared__ int stage[4][kStage];
    WarpOut wo;
    wo.buf = stage[(threadIdx.x >> 5) & 3];
    int* out = v.nb + (size_t)h * v.maxnb;
    const int rz = g.nc[2] >= 3 ? 1 : 0, ry = g.nc[1] >= 3 ? 1 : 0, rx = g.nc[0] >= 3 ? 1 : 0;
    for (int dz = -rz; dz <= rz; ++dz) {
        int zz = cz + dz;
        if (g.periodic[2]) zz = (zz + g.nc[2]) % g.nc[2];
        else if (zz < 0 || zz >= g.nc[2]) continue;
        for (int dy = -ry; dy <= ry; ++dy) {
            const int yy = (cy + dy + g.nc[1]) % g.nc[1];
            for (int dx = -rx; dx <= rx; ++dx) {
                const int xx = (cx + dx + g.nc[0]) % g.nc[0];
                const int c = (zz * g.nc[1] + yy) * g.nc[0] + xx;
                const int s1 = cell_start[c + 1];
                for (int base = cell_start[c]; base < s1; base += 32) {
                    const int s = base + lane;
                    bool keep = false;
                    int ja = 0;
                    if (s < s1) {
                        const float4 q = cpos[s];
                        ja = __float_as_int(q.w);
                        if (ja > ia) {
                            const float ddx = fmin_img(px - q.x, lxf, lxif, 1);
                            const float ddy = fmin_img(py - q.y, lyf, lyif, 1);
                            const float ddz = fmin_img(pz - q.z, lzf, lzif, g.periodic[2]);
                            const float d2 = ddx * ddx + ddy * ddy + ddz * ddz;
                            keep = d2 <= lim_hi;
                            if (keep && surf_i && ja >= v.nliqa && excluded(v, ia, ja)) keep = false;
                            if (keep && d2 >= lim_lo) keep = keep_pair(v, xi, yi, zi, v.x[ja], v.y[ja], v.z[ja]);
                        }
                    }
                    const unsigned m = __ballot_sync(0xffffffffu, keep);
                    wo.push(keep, ja, m, out, v.maxnb, lane);
                }
            }
        }
    }
    wo.flush(out, v.maxnb, lane);
    const int cnt = wo.total();
    if (lane == 0) {
        if (cnt > v.maxnb) atomicMax(&v.status[ST_LIST_OVF], cnt);
        v.nbcnt[h] = min(cnt, v.maxnb);
    }
}

__global__ void k_build_hh(View v, Grid g, const int* cell_start, const float4* cpos, const double4* hpos,
                           int* cell_count) {
    build_hh(v, g, cell_start, cpos, hpos, cell_count, blockIdx.x, gridDim.x);
}

// One warp per head: all wall atoms within rskin (src/nnlist.f90:143-161).
__device__ __forceinline__ void build_hw(const View& v, const Grid& g, const int* wcell_start, const float4* wpos,
                                         const double4* hpos, int bid) {
    if (!v.status[ST_REBUILD]) return;
    const int lane = threadIdx.x & 31;
    const int h = (bid * blockDim.x + threadIdx.x) >> 5;
    if (h >= v.nheads) return;
    const int ia = v.head_atom[h];
    const double xi = v.x[ia], yi = v.y[ia], zi = v.z[ia];
    const double4 pw = hpos[h];
    const float px = (float)pw.x, py = (float)pw.y, pz = (float)pw.z;
    const float lxf = (float)v.lx, lyf = (float)v.ly, lzf = (float)v.lz;
    const float lxif = 1.0f / lxf, lyif = 1.0f / lyf, lzif = 1.0f / lzf;
    const float lim_hi = (float)v.rskinsq * 1.0001f + 0.05f;
    const float lim_lo = (float)v.rskinsq * 0.9999f - 0.05f;
    const double wz = wrap(zi, v.lz, g.periodic[2]);
    const int cx = cell_coord(pw.x, 0, g), cy = cell_coord(pw.y, 1, g), cz = cell_coord(wz, 2, g);
    const bool surf_i = ia >= v.nliqa;
    __shared__ int stage[4][kStage];
    WarpOut wo;
    wo.buf = stage[(threadIdx.x >> 5) & 3];
    int* out = v.wnb + (size_t)h * v.maxwnb;
    const int rz = g.nc[2] >= 3 ? 1 : 0, ry = g.nc[1] >= 3 ? 1 : 0, rx = g.nc[0] >= 3 ? 1 : 0;
    for (int dz = -rz; dz <= rz; ++dz) {
        int zz = cz + dz;
        if (g.periodic[2]) zz = (zz + g.nc[2]) % g.nc[2];
        else if (zz < 0 || zz >= g.nc[2]) continue;
        for (int dy = -ry; dy <= ry; ++dy) {
            const int yy = (cy + dy + g.nc[1]) % g.nc[1];
            for (int dx = -rx; dx <= rx; ++dx) {
                const int xx = (cx + dx + g.nc[0]) % g.nc[0];
                const int c = (zz * g.nc[1] + yy) * g.nc[0] + xx;
                const int s1 = wcell_start[c + 1];
                for (int base = wcell_start[c]; base < s1; base += 32) {
                    const int s = base + lane;
                    bool keep = false;
                    int ja = 0;
                    if (s < s1) {
                        const float4 q = wpos[s];
                        ja = __float_as_int(q.w);
                        const float ddx = fmin_img(px - q.x, lxf, lxif, 1);
                        const float ddy = fmin_img(py - q.y, lyf, lyif, 1);
                        const float ddz = fmin_img(pz - q.z, lzf, lzif, g.periodic[2]);
                        const float d2 = ddx * ddx + ddy * ddy + ddz * ddz;
                        keep = d2 <= lim_hi;
                        if (keep && surf_i && excluded(v, ia, ja)) keep = false;
                        if (keep && d2 >= lim_lo) keep = keep_pair(v, xi, yi, zi, v.x[ja], v.y[ja], v.z[ja]);
                    }
                    const unsigned m = __ballot_sync(0xffffffffu, keep);
                    wo.push(keep, ja, m, out, v.maxwnb, lane);
                }
            }
        }
    }
    wo.flush(out, v.maxwnb, lane);
    const int cnt = wo.total();
    if (lane == 0) {
        if (cnt > v.maxwnb) atomicMax(&v.status[ST_WLIST_OVF], cnt);
        v.wnbcnt[h] = min(cnt, v.maxwnb);
    }
}

__global__ void k_build_hw(View v, Grid g, const int* wcell_start, const float4* wpos, const double4* hpos) {
    build_hw(v, g, wcell_start, wpos, hpos, blockIdx.x);
}

// ---- the list build of several systems, one launch per kernel ----------------------------------
// Per system: its view, grids and list scratch.  first[k] (k = bin, scan, scatter, head-head,
// head-wall) holds each system's first block in launch k (nrep + 1 entries); a block serves the
// system r with first[k][r] <= block < first[k][r + 1], as block (block - first[k][r]) of a grid
// of first[k][r + 1] - first[k][r] blocks.
struct alignas(16) LsRep {
    View v;
    Grid g, wg;
    int *head_cell, *cell_count, *cell_start, *wcell_start;
    double4* hpos;
    float4 *cpos, *wpos;
};

// the system of block b: the largest r with first[r] <= b (first[0] = 0 <= b < first[nrep])
__device__ __forceinline__ int rep_of_block(const int* __restrict__ first, int nrep, int b) {
    int lo = 0, hi = nrep - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(kNT) k_bin_heads_b(const LsRep* __restrict__ reps, const int* __restrict__ first,
                                                     int nrep) {
    const int r = rep_of_block(first, nrep, blockIdx.x);
    const LsRep& R = reps[r];
    bin_heads(R.v, R.g, R.head_cell, R.cell_count, R.hpos, blockIdx.x - first[r], first[r + 1] - first[r]);
}

__global__ void __launch_bounds__(kNT) k_scan_cells_b(const LsRep* __restrict__ reps) {
    const LsRep& R = reps[blockIdx.x];  // one block per system
    scan_cells(R.v, R.g.ncell, R.cell_count, R.cell_start);
}

__global__ void __launch_bounds__(kNT) k_scatter_heads_b(const LsRep* __restrict__ reps,
                                                         const int* __restrict__ first, int nrep) {
    const int r = rep_of_block(first, nrep, blockIdx.x);
    const LsRep& R = reps[r];
    scatter_heads(R.v, R.head_cell, R.cell_count, R.cell_start, R.hpos, R.cpos, blockIdx.x - first[r]);
}

__global__ void __launch_bounds__(128) k_build_hh_b(const LsRep* __restrict__ reps, const int* __restrict__ first,
                                                    int nrep) {
    const int r = rep_of_block(first, nrep, blockIdx.x);
    const LsRep& R = reps[r];
    build_hh(R.v, R.g, R.cell_start, R.cpos, R.hpos, R.cell_count, blockIdx.x - first[r], first[r + 1] - first[r]);
}

__global__ void __launch_bounds__(128) k_build_hw_b(const LsRep* __restrict__ reps, const int* __restrict__ first,
                                                    int nrep) {
    const int r = rep_of_block(first, nrep, blockIdx.x);
    const LsRep& R = reps[r];
    build_hw(R.v, R.wg, R.wcell_start, R.wpos, R.hpos, blockIdx.x - first[r]);
}

Grid make_grid(double lx, double ly, double lz, double rs, int pz, double zlo, double zhi) {
    Grid g{};
    const double L[3] = {lx, ly, lz};
    for (int d = 0; d < 3; ++d) {
        const bool per = d < 2 || pz;
        g.periodic[d] = per ? 1 : 0;
        double span = per ? L[d] : std::max(zhi - zlo, 1e-6);
        int n = (int)std::floor(span / (rs * (1.0 + 1e-9)));
        if (n < 3) n = 1;
        n = std::min(n, 256);
        g.nc[d] = n;
        g.cs[d] = span / n;
        g.org[d] = per ? 0.0 : zlo;
        if (n == 1) g.cs[d] = std::max(span, rs) * 2.0;  // everything in one cell
    }
    g.ncell = g.nc[0] * g.nc[1] * g.nc[2];
    return g;
}

}  // namespace

int nnlist_setup(Ctx& c, const double* x0, const double* y0, const double* z0) {
    View& v = c.v;
    const double rs = std::sqrt(v.rskinsq);
    // head grid: z spans the box (clamped for non-periodic boxes)
    c.grid = make_grid(v.lx, v.ly, v.lz, rs, v.pbcz, -0.5 * v.lz, 0.5 * v.lz);
    // wall grid: static wall atoms binned once
    double zlo = 0, zhi = 1;
    if (v.nwall > 0) {
        zlo = 1e300;
        zhi = -1e300;
        for (int i = v.nmove; i < v.ntota; ++i) {
            double w = v.pbcz ? z0[i] - v.lz * std::floor(z0[i] / v.lz) : z0[i];
            zlo = std::min(zlo, w);
            zhi = std::max(zhi, w);
        }
        zlo -= 1e-3;
        zhi += 1e-3;
    }
    c.wgrid = make_grid(v.lx, v.ly, v.lz, rs, v.pbcz, zlo, zhi);
    const Grid& g = c.grid;
    c.d_cell_start = (int*)dalloc(c, sizeof(int) * (g.ncell + 1));
    c.d_cell_count = (int*)dalloc(c, sizeof(int) * g.ncell);
    c.d_head_cell = (int*)dalloc(c, sizeof(int) * std::max(v.nheads, 1));
    c.d_hpos = (double4*)dalloc(c, sizeof(double4) * std::max(v.nheads, 1));
    // wall bins on the host (once)
    const Grid& wg = c.wgrid;
    std::vector<int> wcount(wg.ncell + 1, 0), wcell(std::max(v.nwall, 1));
    auto cc = [&](double w, int d) {
        int k = (int)std::floor((w - wg.org[d]) / wg.cs[d]);
        return std::min(std::max(k, 0), wg.nc[d] - 1);
    };
    std::vector<float4> wp(std::max(v.nwall, 1));
    for (int k = 0; k < v.nwall; ++k) {
        const int i = v.nmove + k;
        double wx = x0[i] - v.lx * std::floor(x0[i] / v.lx);
        double wy = y0[i] - v.ly * std::floor(y0[i] / v.ly);
        double wz = v.pbcz ? z0[i] - v.lz * std::floor(z0[i] / v.lz) : z0[i];
        wcell[k] = (cc(wz, 2) * wg.nc[1] + cc(wy, 1)) * wg.nc[0] + cc(wx, 0);
        wcount[wcell[k] + 1]++;
    }
    for (int k = 0; k < wg.ncell; ++k) wcount[k + 1] += wcount[k];
    std::vector<int> cur(wcount.begin(), wcount.end() - 1);
    std::vector<float4> wsorted(std::max(v.nwall, 1));
    for (int k = 0; k < v.nwall; ++k) {
        const int i = v.nmove + k;
        double wx = x0[i] - v.lx * std::floor(x0[i] / v.lx);
        double wy = y0[i] - v.ly * std::floor(y0[i] / v.ly);
        double wz = v.pbcz ? z0[i] - v.lz * std::floor(z0[i] / v.lz) : z0[i];
        float4 f;
        f.x = (float)wx;
        f.y = (float)wy;
        f.z = (float)wz;
        int ia = i;
        std::memcpy(&f.w, &ia, 4);
        wsorted[cur[wcell[k]]++] = f;
    }
    c.d_wcell_start = (int*)dalloc(c, sizeof(int) * (wg.ncell + 1));
    c.d_wpos = (float4*)dalloc(c, sizeof(float4) * std::max(v.nwall, 1));
    MDG_CUDA(cudaMemcpy(c.d_wcell_start, wcount.data(), sizeof(int) * (wg.ncell + 1), cudaMemcpyHostToDevice));
    MDG_CUDA(cudaMemcpy(c.d_wpos, wsorted.data(), sizeof(float4) * std::max(v.nwall, 1), cudaMemcpyHostToDevice));
    c.d_cpos = (float4*)dalloc(c, sizeof(float4) * std::max(v.nheads, 1));
    return MDG_OK;
}

void nnlist_trigger(Ctx& c, bool force) {
    View& v = c.v;
    const int n = v.nrig + (v.nmove - v.nriga);
    const int nb = std::max(1, std::min((n + kNT - 1) / kNT, 1024));
    k_trigger<<<nb, kNT, 0, c.stream>>>(v, force ? 1 : 0);
    k_trigger_decide<<<1, 1, 0, c.stream>>>(v, force ? 1 : 0);
}

// Blocks of the five list launches of one system: bin, scan, scatter, head-head, head-wall.
static void list_blocks(const View& v, int nb[5]) {
    const int nh = std::max(v.nheads, 1);
    nb[0] = std::max((std::max(nh, std::max(v.nrig, v.nmove - v.nriga)) + kNT - 1) / kNT, 1);
    nb[1] = 1;
    nb[2] = (nh + kNT - 1) / kNT;
    nb[3] = (nh + 3) / 4;
    nb[4] = v.nwall > 0 ? (nh + 3) / 4 : 0;
}

void nnlist_build(Ctx& c) {
    View& v = c.v;
    const Grid& g = c.grid;
    int nb[5];
    list_blocks(v, nb);
    k_bin_heads<<<nb[0], kNT, 0, c.stream>>>(v, g, c.d_head_cell, c.d_cell_count, c.d_hpos);
    k_scan_cells<<<nb[1], kNT, 0, c.stream>>>(v, g.ncell, c.d_cell_count, c.d_cell_start);
    k_scatter_heads<<<nb[2], kNT, 0, c.stream>>>(v, c.d_head_cell, c.d_cell_count, c.d_cell_start, c.d_hpos,
                                                  c.d_cpos);
    k_build_hh<<<nb[3], 128, 0, c.stream>>>(v, g, c.d_cell_start, c.d_cpos, c.d_hpos, c.d_cell_count);
    if (nb[4] > 0) k_build_hw<<<nb[4], 128, 0, c.stream>>>(v, c.wgrid, c.d_wcell_start, c.d_wpos, c.d_hpos);
}

int ls_batch_setup(LsBatch& lb, const std::vector<Ctx*>& cs, std::string& err) {
    const int nrep = (int)cs.size();
    lb.nrep = nrep;
    if (nrep == 0) return MDG_OK;
    std::vector<LsRep> reps(nrep);
    std::vector<int> first(5 * (nrep + 1), 0);
    for (int r = 0; r < nrep; ++r) {
        const Ctx& c = *cs[r];
        LsRep& R = reps[r];
        R.v = c.v;
        R.g = c.grid;
        R.wg = c.wgrid;
        R.head_cell = c.d_head_cell;
        R.cell_count = c.d_cell_count;
        R.cell_start = c.d_cell_start;
        R.wcell_start = c.d_wcell_start;
        R.hpos = c.d_hpos;
        R.cpos = c.d_cpos;
        R.wpos = c.d_wpos;
        int nb[5];
        list_blocks(c.v, nb);
        for (int k = 0; k < 5; ++k) first[k * (nrep + 1) + r + 1] = first[k * (nrep + 1) + r] + nb[k];
    }
    const size_t off_first = (sizeof(LsRep) * nrep + 255) & ~size_t(255);
    const size_t need = off_first + sizeof(int) * first.size();
    if (need > lb.cap) {
        if (lb.d_buf) cudaFree(lb.d_buf);
        lb.d_buf = nullptr;
        lb.cap = 0;
        if (cudaMalloc(&lb.d_buf, need) != cudaSuccess) {
            err = "replica batch: list descriptor allocation failed";
            return MDG_E_CUDA;
        }
        lb.cap = need;
    }
    unsigned char* base = static_cast<unsigned char*>(lb.d_buf);
    lb.reps = base;
    for (int k = 0; k < 5; ++k) {
        lb.first[k] = reinterpret_cast<int*>(base + off_first) + k * (nrep + 1);
        lb.nblk[k] = first[k * (nrep + 1) + nrep];
    }
    if (cudaMemcpy(base, reps.data(), sizeof(LsRep) * nrep, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(base + off_first, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        err = "replica batch: list descriptor upload failed";
        return MDG_E_CUDA;
    }
    return MDG_OK;
}

void ls_batch_launch(const LsBatch& lb, cudaStream_t st) {
    if (lb.nrep == 0) return;
    const LsRep* reps = static_cast<const LsRep*>(lb.reps);
    k_bin_heads_b<<<lb.nblk[0], kNT, 0, st>>>(reps, lb.first[0], lb.nrep);
    k_scan_cells_b<<<lb.nrep, kNT, 0, st>>>(reps);
    k_scatter_heads_b<<<lb.nblk[2], kNT, 0, st>>>(reps, lb.first[2], lb.nrep);
    k_build_hh_b<<<lb.nblk[3], 128, 0, st>>>(reps, lb.first[3], lb.nrep);
    if (lb.nblk[4] > 0) k_build_hw_b<<<lb.nblk[4], 128, 0, st>>>(reps, lb.first[4], lb.nrep);
}

void ls_batch_free(LsBatch& lb) {
    if (lb.d_buf) cudaFree(lb.d_buf);
    lb = LsBatch();
}

}  // namespace mdg
