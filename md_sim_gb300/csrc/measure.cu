// measure.cu - measurement histograms: the side outputs of the force loops and measure_do.
//
//   k_hist_pairs   moving pairs: slab variant, z force on Li/Cl-type ions (site types 3, 4) by
//                  the ion's z bin (efipos, src/forcem.f90:347-354,388-395); bulk variant, pair
//                  distances by site-type pair (ngc, src/forcem_back.f90:348-349,380-382)
//   k_hist_walls   site-wall distances (ngc, src/forcem.f90:493-495) and, slab variant, the ion
//                  wall terms of efipos (:486-489)
//   k_hist_ions    liquid ions: whole fz after force_fouri into efipos (:930-934), or the final
//                  ftz and the count into tefipos/nefipos (:1094-1098)
//   k_hist_angles  bend-angle cosines by molecule type (ngang, :617-625)
//   k_measure_do / k_measure_fin   measure_do (src/measure.f90:270-312): summed wall forces, site
//                  z-profile ngz, water dipole profile ndip*, near-wall 2-D maps ng2d1/ng2d2
//
// The histograms are side outputs, so these kernels recompute the quantities they bin from the
// positions and the neighbour lists instead of adding work to the force kernels; they run only
// while measuring.  This file is compiled without multiply-add contraction and every bin index
// is evaluated with the reference's operation order, so integer histograms of the same positions
// match the reference's exactly.  A bin outside its array (the reference does not check) is
// dropped and counted.
#include <algorithm>

#include "common.cuh"
#include "ctx.h"

namespace mdg {

namespace {

constexpr int kWarps = 8;
constexpr int kNT = kWarps * 32;
constexpr int kSmemMax = 160 * 1024;

// l = int((z + lwh)*rdeli + 0.5), l = int(r*rdeli + 0.5): truncation toward zero like int()
__device__ __forceinline__ long long zbin(const MeasView& m, double z) { return (long long)((z + m.lwh) * m.rdeli + 0.5); }
__device__ __forceinline__ long long rbin(const MeasView& m, double r) { return (long long)(r * m.rdeli + 0.5); }
__device__ __forceinline__ bool ion(int t) { return t == 2 || t == 3; }  // site types 3, 4 (1-based)

__device__ __forceinline__ void oor(const MeasView& m) { atomicAdd(&m.cnt[2], 1ull); }

__device__ __forceinline__ void add_gc(const MeasView& m, unsigned* s_ngc, int nijt, int ijt, long long l) {
    if (l < 0 || l > m.lmax) return oor(m);
    const int k = ijt + nijt * (int)l;
    if (s_ngc) atomicAdd(&s_ngc[k], 1u);
    else atomicAdd(&m.ngc[k], 1ull);
}

__device__ __forceinline__ void add_ef(const MeasView& m, double* s_ef, int t, long long l, double val) {
    if (t < 0 || t > 1 || l < 0 || l > m.lmax) return oor(m);
    const int k = t + 2 * (int)l;
    if (s_ef) atomicAdd(&s_ef[k], val);
    else atomicAdd(&m.efipos[k], val);
}

__device__ __forceinline__ double erfc_as(double alfar, double* ff, double spii) {
    const double t = 1.0 / (1.0 + kP * alfar);
    const double exp2a = exp(-alfar * alfar);
    const double erfx = ((((kA5 * t + kA4) * t + kA3) * t + kA2) * t + kA1) * t * exp2a;
    *ff = spii * alfar * exp2a + erfx;
    return erfx;
}

// vdW force factor of src/forcem.f90:311-328 (head pair)
__device__ __forceinline__ double vdw_fij(const View& v, int ijt, double rsq, double rsqi, double rij) {
    const int vk = v.vdw[ijt];
    if (vk == 1) {
        const double r6 = v.sig[ijt] * (rsqi * rsqi * rsqi);
        return 6.0 * rsqi * v.eps[ijt] * r6 * (2.0 * r6 - 1.0);
    }
    if (vk == 2) {
        const double r6 = v.cc[ijt] * (rsqi * rsqi * rsqi);
        const double aux = v.aa[ijt] * exp(-rij * v.rhoi[ijt]);
        return aux * v.rhoi[ijt] / rij - 6.0 * rsqi * r6;
    }
    return 0.0;
}

__device__ void hist_setup(const MeasView& m, int nijt, bool shared, unsigned char* sm, unsigned** s_ngc,
                           double** s_ef) {
    *s_ngc = nullptr;
    *s_ef = nullptr;
    if (!shared) return;
    const int nc = nijt * m.L;
    *s_ngc = reinterpret_cast<unsigned*>(sm);
    *s_ef = reinterpret_cast<double*>(sm + ((sizeof(unsigned) * nc + 15) & ~size_t(15)));
    for (int k = threadIdx.x; k < nc; k += blockDim.x) (*s_ngc)[k] = 0u;
    for (int k = threadIdx.x; k < 2 * m.L; k += blockDim.x) (*s_ef)[k] = 0.0;
    __syncthreads();
}

__device__ void hist_flush(const MeasView& m, int nijt, const unsigned* s_ngc, const double* s_ef) {
    if (!s_ngc) return;
    __syncthreads();
    for (int k = threadIdx.x; k < nijt * m.L; k += blockDim.x)
        if (s_ngc[k]) atomicAdd(&m.ngc[k], (unsigned long long)s_ngc[k]);
    for (int k = threadIdx.x; k < 2 * m.L; k += blockDim.x)
        if (s_ef[k] != 0.0) atomicAdd(&m.efipos[k], s_ef[k]);
}

__global__ void __launch_bounds__(kNT) k_hist_pairs(View v, MeasView m, int shared) {
    extern __shared__ __align__(16) unsigned char sm[];
    unsigned* s_ngc;
    double* s_ef;
    hist_setup(m, v.nijt, shared, sm, &s_ngc, &s_ef);
    const int lane = threadIdx.x & 31;
    const int warp = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int nwarps = gridDim.x * kWarps;
    for (int h = warp; h < v.nheads; h += nwarps) {
        const int i = v.head_atom[h];
        const int it = v.type[i];
        const int nsi_i = v.nsi[it];
        const double xi0 = v.x[i], yi0 = v.y[i], zi0 = v.z[i];
        const int n = v.nbcnt[h];
        const int* nb = v.nb + (size_t)h * v.maxnb;
        for (int k = lane; k < n; k += 32) {
            const int j = nb[k];
            const int jt = v.type[j];
            if (m.slab && !ion(it) && !ion(jt)) continue;
            const double xio = minimg(xi0 - v.x[j], v.lx, v.lxi);
            const double yio = minimg(yi0 - v.y[j], v.ly, v.lyi);
            double zio = zi0 - v.z[j];
            if (v.bulk) zio = minimg(zio, v.lz, v.lzi);
            const double rsq = xio * xio + yio * yio + zio * zio;
            if (rsq > v.rcutsq) continue;
            const int ijt = v.ijt[it * v.nit + jt];
            const int nsi_j = v.nsi[jt];
            const double rsqi = 1.0 / rsq;
            const double rij = sqrt(rsq);
            if (m.slab) {
                double ff;
                double fij = vdw_fij(v, ijt, rsq, rsqi, rij);
                const double aux = v.facq * v.q[i] * v.q[j] / rij;
                erfc_as(v.alfa * rij, &ff, v.spii);
                fij = fij + ff * aux * rsqi;
                const long long li = zbin(m, zi0), lj = zbin(m, v.z[j]);
                if (ion(it)) add_ef(m, s_ef, it - 2, li, zio * fij);
                if (ion(jt)) add_ef(m, s_ef, jt - 2, lj, -(zio * fij));
                for (int a = 0; a < nsi_i; ++a) {
                    const double xa = xio + v.rsx[i + a], ya = yio + v.rsy[i + a], za = zio + v.rsz[i + a];
                    const double qx = v.facq * v.q[i + a];
                    for (int b = (a == 0 ? 1 : 0); b < nsi_j; ++b) {
                        const double xd = xa - v.rsx[j + b], yd = ya - v.rsy[j + b], zd = za - v.rsz[j + b];
                        const double r2 = xd * xd + yd * yd + zd * zd;
                        const double r2i = 1.0 / r2;
                        const double rr = sqrt(r2);
                        const double au = qx * v.q[j + b] / rr;
                        double fq;
                        erfc_as(v.alfa * rr, &fq, v.spii);
                        const double fs = fq * au * r2i;
                        if (ion(it)) add_ef(m, s_ef, it - 2, li, zd * fs);
                        if (ion(jt)) add_ef(m, s_ef, jt - 2, lj, -(zd * fs));
                    }
                }
            } else {
                add_gc(m, s_ngc, v.nijt, ijt, rbin(m, rij));
                for (int a = 0; a < nsi_i; ++a) {
                    const double xa = xio + v.rsx[i + a], ya = yio + v.rsy[i + a], za = zio + v.rsz[i + a];
                    const int ta = v.type[i + a];
                    for (int b = (a == 0 ? 1 : 0); b < nsi_j; ++b) {
                        const double xd = xa - v.rsx[j + b], yd = ya - v.rsy[j + b], zd = za - v.rsz[j + b];
                        const double r2 = xd * xd + yd * yd + zd * zd;
                        add_gc(m, s_ngc, v.nijt, v.ijt[ta * v.nit + v.type[j + b]], rbin(m, sqrt(r2)));
                    }
                }
            }
        }
    }
    hist_flush(m, v.nijt, s_ngc, s_ef);
}

__global__ void __launch_bounds__(kNT) k_hist_walls(View v, MeasView m, int shared) {
    extern __shared__ __align__(16) unsigned char sm[];
    unsigned* s_ngc;
    double* s_ef;
    hist_setup(m, v.nijt, shared, sm, &s_ngc, &s_ef);
    const int lane = threadIdx.x & 31;
    const int warp = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int nwarps = gridDim.x * kWarps;
    for (int h = warp; h < v.nheads; h += nwarps) {
        const int i = v.head_atom[h];
        const int it = v.type[i];
        const int nsi_i = v.nsi[it];
        const bool efi = m.slab && ion(it);
        const double xi0 = v.x[i], yi0 = v.y[i], zi0 = v.z[i];
        const long long li = zbin(m, zi0);
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
            const int tj = v.type[j];
            double fij = 0.0;
            if (efi) {
                const int ijt = v.ijt[it * v.nit + tj];
                const double rsqi = 1.0 / rsq;
                fij = vdw_fij(v, ijt, rsq, rsqi, v.vdw[ijt] == 2 ? sqrt(rsq) : 0.0);
            }
            const double qx = v.facq * v.q[j];
            for (int a = 0; a < nsi_i; ++a) {
                const double xd = xi + v.rsx[i + a], yd = yi + v.rsy[i + a], zd = zi + v.rsz[i + a];
                const double r2 = xd * xd + yd * yd + zd * zd;
                const double rr = sqrt(r2);
                if (efi) {
                    const double r2i = 1.0 / r2;
                    const double au = qx * v.q[i + a] / rr;
                    double fq;
                    erfc_as(v.alfa * rr, &fq, v.spii);
                    fij = fij + fq * au * r2i;
                    add_ef(m, s_ef, it - 2, li, zd * fij);
                    fij = 0.0;
                }
                add_gc(m, s_ngc, v.nijt, v.ijt[v.type[i + a] * v.nit + tj], rbin(m, rr));
            }
        }
    }
    hist_flush(m, v.nijt, s_ngc, s_ef);
}

// mode 0: efipos += fz after force_fouri; mode 1: nefipos += 1, tefipos += final fz.  Block 0
// thread 0 of a mode-1 launch also counts the force evaluation.
__global__ void k_hist_ions(View v, MeasView m, int mode) {
    if (mode == 1 && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&m.cnt[0], 1ull);
    if (!m.slab) return;
    for (int i = v.nriga + blockIdx.x * blockDim.x + threadIdx.x; i < v.nliqa; i += gridDim.x * blockDim.x) {
        const int t = v.type[i] - 2;
        const long long l = zbin(m, v.z[i]);
        if (t < 0 || t > 1 || l < 0 || l > m.lmax) {
            oor(m);
            continue;
        }
        const int k = t + 2 * (int)l;
        if (mode == 0) {
            atomicAdd(&m.efipos[k], v.fz[i]);
        } else {
            atomicAdd(&m.nefipos[k], 1ull);
            atomicAdd(&m.tefipos[k], v.fz[i]);
        }
    }
}

__global__ void k_hist_angles(View v, MeasView m, int nterm, const int4* ang) {
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
    const double cang = -(ab * ai * bi);
    const long long l = (long long)((cang + 1.0) * 100.0) + 1;
    const int row = m.ang_mt[t];
    if (l < 0 || l > m.langmax || row >= m.ntz) return oor(m);
    atomicAdd(&m.ngang[row + m.ntz * (int)l], 1ull);
}

__global__ void k_measure_do(View v, MeasView m, const double* __restrict__ x, const double* __restrict__ y,
                             const double* __restrict__ z) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < v.nmove; i += gridDim.x * blockDim.x) {
        const int it = v.type[i];  // 0-based: the reference's it - 1
        const long long l = zbin(m, z[i]);
        if (l >= 0 && l <= m.lmax && it < m.ntz) {
            atomicAdd(&m.ngz[it + m.ntz * (int)l], 1ull);
            if (it == 0 && i + 2 < v.nmove) {  // a water O and its two H (the reference assumes it)
                atomicAdd(&m.mu[2 * m.L + l], z[i] - 0.5 * (z[i + 1] + z[i + 2]));
                atomicAdd(&m.mu[l], x[i] - 0.5 * (x[i + 1] + x[i + 2]));
                atomicAdd(&m.mu[m.L + l], y[i] - 0.5 * (y[i + 1] + y[i + 2]));
            }
        } else {
            oor(m);
        }
        const double rij = m.lwh - fabs(z[i]);
        if (m.l2d && rij < m.rscnd) {
            double px = fmod(x[i] + m.lxh + m.cx4, m.cx4);
            if (px != 0.0 && ((px < 0.0) != (m.cx4 < 0.0))) px += m.cx4;
            double py = fmod(y[i] + m.lyh + m.cy2, m.cy2);
            if (py != 0.0 && ((py < 0.0) != (m.cy2 < 0.0))) py += m.cy2;
            const long long lx = (long long)(0.5 * px * m.rdeli + 0.5);
            const long long ky = (long long)(0.5 * py * m.rdeli + 0.5);
            if (lx < 0 || ky < 0 || lx > m.lgx || ky > m.lgy || it >= m.ntz) {
                oor(m);
            } else {
                const long long kk = it + (long long)m.ntz * (lx + (long long)(m.lgx + 1) * ky);
                atomicAdd(rij < m.rfrst ? &m.ng2d1[kk] : &m.ng2d2[kk], 1ull);
            }
        }
    }
}

// ndip* += the call's dipole sums, ftot += fws of the last force evaluation; clears the scratch.
__global__ void k_measure_fin(View v, MeasView m) {
    for (int l = threadIdx.x; l < m.L; l += blockDim.x) {
        const double mx = m.mu[l], my = m.mu[m.L + l], mz = m.mu[2 * m.L + l];
        m.ndip[l] += mx;
        m.ndip[m.L + l] += my;
        m.ndip[2 * m.L + l] += mz;
        m.ndip[3 * m.L + l] += mx * mx + my * my + mz * mz;
        m.mu[l] = m.mu[m.L + l] = m.mu[2 * m.L + l] = 0.0;
    }
    if (threadIdx.x < 9) {
        const int comp = threadIdx.x / 3, s = threadIdx.x % 3;
        const double* sl = v.acc + 2 * v.nijt;
        m.ftot[threadIdx.x] += (s == 1) ? sl[ACC_FWS0 + comp] : sl[ACC_FWS + threadIdx.x];
    }
    if (threadIdx.x == 0) atomicAdd(&m.cnt[1], 1ull);
}

int grid_heads(const Ctx& c) { return std::max(1, std::min((c.v.nheads + kWarps - 1) / kWarps, 152 * 8)); }

}  // namespace

int measure_init(Ctx& c, const mdg_measure_params* p, mdg_measure_dims* d) {
    if (!p || !(p->rdel > 0.0)) return set_err(&c, MDG_E_ARG, "measure: rdel must be positive");
    const View& v = c.v;
    MeasView m;
    m.rdeli = 1.0 / p->rdel;
    m.lwh = v.lwh;
    m.lmax = (int)(long long)(c.sysc.lw * m.rdeli + 0.5) + 1;
    m.L = m.lmax + 1;
    m.ntz = std::max(v.nit - 2, 1);
    m.langmax = 201;
    m.l2d = p->l2d != 0;
    m.rfrst = p->rfrst;
    m.rscnd = p->rscnd;
    m.lxh = 0.5 * v.lx;
    m.lyh = 0.5 * v.ly;
    m.cx4 = 4.0 * c.sysc.cx;
    m.cy2 = 2.0 * c.sysc.cy;
    m.lgx = (int)(long long)(4.0 * c.sysc.cx * m.rdeli + 1.0);
    m.lgy = (int)(long long)(2.0 * c.sysc.cy * m.rdeli + 1.0);
    m.slab = c.variant == MDG_SLAB;
    if (m.L > (1 << 22) || (long long)v.nijt * m.L > (1ll << 28) || m.lgx > (1 << 14) || m.lgy > (1 << 14))
        return set_err(&c, MDG_E_ARG, "measure: too many bins");
    const size_t L = m.L, n2d = m.l2d ? (size_t)m.ntz * (m.lgx + 1) * (m.lgy + 1) : 1;
    const size_t nu = (size_t)v.nijt * L + 2 * L + (size_t)m.ntz * (m.langmax + 1) + (size_t)m.ntz * L + 2 * n2d + 3;
    // doubles: efipos 2L | tefipos 2L | ndip 4L | mu 3L | ftot 9 | pos 3 nmove
    const size_t o_tef = 2 * L, o_ndip = 4 * L, o_mu = 8 * L, o_ftot = 11 * L, o_pos = 11 * L + 9;
    const size_t nd = o_pos + 3 * (size_t)std::max(v.nmove, 1);
    auto* u = static_cast<unsigned long long*>(dalloc(c, sizeof(unsigned long long) * nu));
    auto* dd = static_cast<double*>(dalloc(c, sizeof(double) * nd));
    int* amt = c.h_ang_mt.empty() ? nullptr : static_cast<int*>(dalloc(c, sizeof(int) * c.h_ang_mt.size()));
    if (!u || !dd || (!c.h_ang_mt.empty() && !amt)) return set_err(&c, MDG_E_CUDA, "measure: out of device memory");
    if (amt) MDG_CUDA(cudaMemcpy(amt, c.h_ang_mt.data(), sizeof(int) * c.h_ang_mt.size(), cudaMemcpyHostToDevice));
    m.ngc = u;
    m.nefipos = m.ngc + (size_t)v.nijt * L;
    m.ngang = m.nefipos + 2 * L;
    m.ngz = m.ngang + (size_t)m.ntz * (m.langmax + 1);
    m.ng2d1 = m.ngz + (size_t)m.ntz * L;
    m.ng2d2 = m.ng2d1 + n2d;
    m.cnt = m.ng2d2 + n2d;
    m.efipos = dd;
    m.tefipos = dd + o_tef;
    m.ndip = dd + o_ndip;
    m.mu = dd + o_mu;
    m.ftot = dd + o_ftot;
    m.pos = dd + o_pos;
    m.ang_mt = amt;
    const size_t sm = (((size_t)sizeof(unsigned) * v.nijt * L + 15) & ~size_t(15)) + sizeof(double) * 2 * L;
    c.meas.smem = sm <= (size_t)kSmemMax ? (int)sm : 0;
    if (c.meas.smem) {
        MDG_CUDA(allow_max_smem(k_hist_pairs));
        MDG_CUDA(allow_max_smem(k_hist_walls));
    }
    c.meas.m = m;
    c.meas.force_hist = p->force_hist != 0;
    c.meas.profiles = p->profiles != 0;
    c.meas.init = true;
    if (d) {
        d->lmax = m.lmax;
        d->nijt = v.nijt;
        d->ntz = m.ntz;
        d->langmax = m.langmax;
        d->lgxmax = m.lgx;
        d->lgymax = m.lgy;
    }
    return MDG_OK;
}

void measure_zero(Ctx& c) {
    const MeasView& m = c.meas.m;
    const View& v = c.v;
    const size_t L = m.L, n2d = m.l2d ? (size_t)m.ntz * (m.lgx + 1) * (m.lgy + 1) : 1;
    const size_t nu = (size_t)v.nijt * L + 2 * L + (size_t)m.ntz * (m.langmax + 1) + (size_t)m.ntz * L + 2 * n2d + 3;
    cudaMemsetAsync(m.ngc, 0, sizeof(unsigned long long) * nu, c.stream);
    cudaMemsetAsync(m.efipos, 0, sizeof(double) * (11 * L + 9), c.stream);
}

void measure_force_real(Ctx& c) {
    const int g = grid_heads(c), sm = c.meas.smem;
    if (c.v.nheads == 0) return;
    k_hist_pairs<<<g, kNT, sm, c.stream>>>(c.v, c.meas.m, sm > 0);
    if (c.v.nwall > 0) k_hist_walls<<<g, kNT, sm, c.stream>>>(c.v, c.meas.m, sm > 0);
}

void measure_force_fouri(Ctx& c) {
    const int n = c.v.nliqa - c.v.nriga;
    if (c.variant != MDG_SLAB || n <= 0) return;
    k_hist_ions<<<std::min((n + 127) / 128, 152), 128, 0, c.stream>>>(c.v, c.meas.m, 0);
}

void measure_force_intra(Ctx& c) {
    if (c.nang_terms == 0) return;
    k_hist_angles<<<(c.nang_terms + 127) / 128, 128, 0, c.stream>>>(c.v, c.meas.m, c.nang_terms,
                                                                   reinterpret_cast<const int4*>(c.d_ang));
}

void measure_force_sum(Ctx& c) {
    const int n = std::max(c.v.nliqa - c.v.nriga, 1);
    k_hist_ions<<<std::min((n + 127) / 128, 152), 128, 0, c.stream>>>(c.v, c.meas.m, 1);
}

void measure_do_launch(Ctx& c, const double* x, const double* y, const double* z) {
    const int n = std::max(c.v.nmove, 1);
    k_measure_do<<<std::min((n + 255) / 256, 152 * 4), 256, 0, c.stream>>>(c.v, c.meas.m, x, y, z);
    k_measure_fin<<<1, 256, 0, c.stream>>>(c.v, c.meas.m);
}

int measure_get(Ctx& c, mdg_measure_out* o) {
    const MeasView& m = c.meas.m;
    const View& v = c.v;
    MDG_CUDA(cudaStreamSynchronize(c.stream));
    const size_t L = m.L, n2d = (size_t)m.ntz * (m.lgx + 1) * (m.lgy + 1);
    auto geti = [&](int64_t* dst, const unsigned long long* src, size_t n) -> cudaError_t {
        if (!dst || n == 0) return cudaSuccess;
        return cudaMemcpy(dst, src, sizeof(int64_t) * n, cudaMemcpyDeviceToHost);
    };
    auto getd = [&](double* dst, const double* src, size_t n) -> cudaError_t {
        if (!dst || n == 0) return cudaSuccess;
        return cudaMemcpy(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost);
    };
    MDG_CUDA(geti(o->ngc, m.ngc, (size_t)v.nijt * L));
    MDG_CUDA(geti(o->nefipos, m.nefipos, 2 * L));
    MDG_CUDA(geti(o->ngang, m.ngang, (size_t)m.ntz * (m.langmax + 1)));
    MDG_CUDA(geti(o->ngz, m.ngz, (size_t)m.ntz * L));
    if (m.l2d) {
        MDG_CUDA(geti(o->ng2d1, m.ng2d1, n2d));
        MDG_CUDA(geti(o->ng2d2, m.ng2d2, n2d));
    } else {
        if (o->ng2d1) std::fill(o->ng2d1, o->ng2d1 + n2d, 0);
        if (o->ng2d2) std::fill(o->ng2d2, o->ng2d2 + n2d, 0);
    }
    MDG_CUDA(getd(o->efipos, m.efipos, 2 * L));
    MDG_CUDA(getd(o->tefipos, m.tefipos, 2 * L));
    MDG_CUDA(getd(o->ndipx, m.ndip, L));
    MDG_CUDA(getd(o->ndipy, m.ndip + L, L));
    MDG_CUDA(getd(o->ndipz, m.ndip + 2 * L, L));
    MDG_CUDA(getd(o->ndipsq, m.ndip + 3 * L, L));
    double ft[9];
    MDG_CUDA(cudaMemcpy(ft, m.ftot, sizeof(ft), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 9; ++k) o->ftot[k / 3][k % 3] = ft[k];
    unsigned long long cnt[3];
    MDG_CUDA(cudaMemcpy(cnt, m.cnt, sizeof(cnt), cudaMemcpyDeviceToHost));
    o->calls_force = (int64_t)cnt[0];
    o->calls_do = (int64_t)cnt[1];
    o->out_of_range = (int64_t)cnt[2];
    return MDG_OK;
}

}  // namespace mdg
