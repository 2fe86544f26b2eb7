// widom.cu - Widom test-particle insertion of a rigid 3-site water (chempot, src/forcem.f90:1226-1507).
//
// The host draws the positions and orientations with the reference's congruential generator
// (src/rndmod.f90:26-35) in the reference's order, assuming every position is accepted, and
// records the generator state after each position and after its orientations.  One CTA per
// position then (k_widom):
//   - scans all sites for the O of the probe: overlap test (2.35 A to a water O, 2 A to others,
//     src/forcem.f90:1303-1313), vdW + Ewald erfc of the O (src/forcem.f90:1315-1334) and the
//     neighbour list within rcut (every site that is not of the H type), kept in shared memory;
//   - per orientation, the Ewald erfc terms of the probe's sites against the neighbours' sites
//     (src/forcem.f90:1378-1423), the reciprocal term 0.5 Ak Re(sum_s q_s e^{ik r_s} conj(Qsum))
//     with the phase tables built by repeated multiplication as the reference builds them
//     (src/forcem.f90:1428-1474), the optional slab term and the O's wall tail (:1481-1494);
//     exp(-beta u) summed over the orientations.
// The host keeps the positions up to the first overlap (the reference leaves the insertion loop
// there, src/forcem.f90:1342) unless MDG_WIDOM_SKIP_OVERLAP is set, and accumulates pave/inave.
// Contexts of the FP64 form run everything in FP64; those of the mixed form run the orientation
// loop in FP32 (block sums, the wall tail and the exponential stay FP64).
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "ctx.h"

namespace mdg {

namespace {

constexpr int kWT = 256;        // threads per insertion
constexpr int kWNb = 1024;      // neighbour capacity per insertion
constexpr int kMaxRot = 20;

struct WArgs {
    const double4* pos;   // O position per insertion (w: unused)
    const double* rot;    // [ins][kMaxRot][6]: H1 x y z, H2 x y z (the reference's rins(2,:), rins(3,:))
    const int* nrot;      // orientations per insertion
    double2* res;         // (sum exp(-beta u), status: 0 accepted, 1 overlap, 2 neighbour overflow)
    const int3* kvec;     // k set in the reference's order
    const double* ak;
    const double2* sk;    // moving-site S(k) of the last evaluation
    const double2* qw;    // wall S(k)
    const double* lr;     // [9][nit] wall tail tables
    int nk, KL, KM, KN;
    double pipix, pipiy, pipiz;
    double beta, rinsmin, rwinsmin, crf;
    double q0, q1;        // probe charges (O, H)
    // mixed form: FP32 operands of the orientation loop
    const float2* qsf;    // Qsum = S + S_wall in FP32
    const float* akf;     // Ak in FP32
    const float4* rsf;    // per site: rs offset (moving sites) and charge, FP32
};

__device__ __forceinline__ float ewald_ef(float rr, float alfa) {
    const float ar = alfa * rr;
    const float t = __fdividef(1.0f, 1.0f + (float)kP * ar);
    const float e2 = __expf(-ar * ar);
    return (((((float)kA5 * t + (float)kA4) * t + (float)kA3) * t + (float)kA2) * t + (float)kA1) * t * e2;
}

// FP32 operands of one call: Qsum per k, and per site its offset rs (as force_sum left it, like
// the reference's module array) and charge.
__global__ void k_widom_prep(View v, const double2* __restrict__ sk, const double2* __restrict__ qw, float2* qsf,
                             int nk, float4* rsf) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nk; k += gridDim.x * blockDim.x)
        qsf[k] = make_float2((float)(sk[k].x + qw[k].x), (float)(sk[k].y + qw[k].y));
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < v.ntota; a += gridDim.x * blockDim.x) {
        const bool mv = a < v.nmove;
        rsf[a] = make_float4(mv ? (float)v.rsx[a] : 0.f, mv ? (float)v.rsy[a] : 0.f, mv ? (float)v.rsz[a] : 0.f,
                             (float)v.q[a]);
    }
}

__device__ __forceinline__ double ewald_e(double rij, double alfa) {
    const double alfar = alfa * rij;
    const double t = 1.0 / (1.0 + kP * alfar);
    const double exp2a = exp(-alfar * alfar);
    return ((((kA5 * t + kA4) * t + kA3) * t + kA2) * t + kA1) * t * exp2a;
}

__device__ double block_sum_d(double x, double* red) {
    x = warp_sum(x);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = x;
    __syncthreads();
    double s = 0.0;
    for (int k = 0; k < kWT / 32; ++k) s += red[k];
    return s;
}

// MX: the orientation loop (real-space erfc terms and the reciprocal term) in FP32 with FP64 sums
// per block, for contexts of the mixed form; the O scan, the wall tail and exp stay FP64.
template <bool MX>
__global__ void __launch_bounds__(kWT) k_widom(View v, WArgs w) {
    extern __shared__ __align__(16) unsigned char sm[];
    int* nb_j = reinterpret_cast<int*>(sm);
    double* nb_d = reinterpret_cast<double*>(sm + sizeof(int) * kWNb);           // [kWNb][3]
    double2* tab = reinterpret_cast<double2*>(sm + sizeof(int) * kWNb + sizeof(double) * 3 * kWNb);
    const int nl = w.KL + 1, nm = 2 * w.KM + 1, nn = 2 * w.KN + 1;
    double2* el = tab;                 // [3][nl]
    double2* em = el + 3 * nl;         // [3][nm], index m + KM
    double2* en = em + 3 * nm;         // [3][nn], index n + KN
    __shared__ double red[kWT / 32];
    __shared__ int s_nnb, s_flag;
    const int ins = blockIdx.x, t = threadIdx.x;
    const double4 o = w.pos[ins];
    const double ox = o.x, oy = o.y, oz = o.z;
    if (t == 0) {
        s_nnb = 0;
        s_flag = 0;
    }
    __syncthreads();
    // ---- the probe's O against every site that is not of the H type
    double ux = 0.0;
    for (int j = t; j < v.ntota; j += kWT) {
        const int jt = v.type[j];
        if (jt == 1) continue;
        const double zio = oz - v.z[j];
        if (fabs(zio) > v.rcut) continue;
        const double xio = minimg(ox - v.x[j], v.lx, v.lxi);
        const double yio = minimg(oy - v.y[j], v.ly, v.lyi);
        const double rsq = xio * xio + yio * yio + zio * zio;
        if (rsq > v.rcutsq) continue;
        if (rsq < w.rwinsmin && (jt == 0 || rsq < w.rinsmin)) {
            atomicOr(&s_flag, 1);
            continue;
        }
        const int ijt = v.ijt[jt];  // it = 1 (the water O type)
        const double rsqi = 1.0 / rsq;
        const double rij = sqrt(rsq);
        const int vk = v.vdw[ijt];
        if (vk == 1) {
            const double r6 = v.sig[ijt] * (rsqi * rsqi * rsqi);
            ux += v.eps[ijt] * r6 * (r6 - 1.0);
        } else if (vk == 2) {
            const double r6 = v.cc[ijt] * (rsqi * rsqi * rsqi);
            ux += v.aa[ijt] * exp(-rij * v.rhoi[ijt]) - r6;
        }
        ux += ewald_e(rij, v.alfa) * (v.facq * w.q0 * v.q[j] / rij);
        const int k = atomicAdd(&s_nnb, 1);
        if (k < kWNb) {
            nb_j[k] = j;
            nb_d[3 * k + 0] = xio;
            nb_d[3 * k + 1] = yio;
            nb_d[3 * k + 2] = zio;
        } else {
            atomicOr(&s_flag, 2);
        }
    }
    ux = block_sum_d(ux, red);
    __syncthreads();
    const int flag = s_flag, nnb = min(s_nnb, kWNb);
    if (flag) {
        if (t == 0) w.res[ins] = make_double2(0.0, (flag & 1) ? 1.0 : 2.0);
        return;
    }
    const double qs3[3] = {w.q0, w.q1, w.q1};
    double acc = 0.0;
    const int nr = w.nrot[ins];
    for (int r = 0; r < nr; ++r) {
        const double* rr = w.rot + ((size_t)ins * kMaxRot + r) * 6;
        const double sx[3] = {ox, rr[0], rr[3]}, sy[3] = {oy, rr[1], rr[4]}, sz[3] = {oz, rr[2], rr[5]};
        double ur = 0.0, uk = 0.0;
        if constexpr (!MX) {
            // ---- real space: the probe's sites against the neighbours' sites
            for (int k = t; k < nnb; k += kWT) {
                const int j = nb_j[k];
                const double xio = nb_d[3 * k], yio = nb_d[3 * k + 1], zio = nb_d[3 * k + 2];
                const int jt = v.type[j];
                if (jt == 0) {
                    const int njx = v.nsi[jt];
                    for (int ix = 0; ix < 3; ++ix) {
                        const double xi = (xio + sx[ix]) - ox, yi = (yio + sy[ix]) - oy, zi = (zio + sz[ix]) - oz;
                        const double qx = v.facq * qs3[ix];
                        for (int jx = (ix == 0 ? j + 1 : j); jx < j + njx; ++jx) {
                            const double xd = xi - v.rsx[jx], yd = yi - v.rsy[jx], zd = zi - v.rsz[jx];
                            const double rsq = xd * xd + yd * yd + zd * zd;
                            const double rij = sqrt(rsq);
                            ur += ewald_e(rij, v.alfa) * (qx * v.q[jx] / rij);
                        }
                    }
                } else {
                    for (int ix = 1; ix < 3; ++ix) {
                        const double xi = (xio + sx[ix]) - ox, yi = (yio + sy[ix]) - oy, zi = (zio + sz[ix]) - oz;
                        const double rsq = xi * xi + yi * yi + zi * zi;
                        const double rij = sqrt(rsq);
                        ur += ewald_e(rij, v.alfa) * (v.facq * qs3[ix] * v.q[j] / rij);
                    }
                }
            }
            // ---- reciprocal space: per-site phase tables by repeated multiplication
            if (t < 9) {
                const int s = t / 3, ax = t % 3;
                const double ang = ax == 0 ? w.pipix * sx[s] : (ax == 1 ? w.pipiy * sy[s] : w.pipiz * sz[s]);
                double2 e1;
                sincos(ang, &e1.y, &e1.x);
                if (ax == 0) {
                    double2* T = el + s * nl;
                    T[0] = make_double2(1.0, 0.0);
                    if (w.KL >= 1) T[1] = e1;
                    for (int l = 2; l <= w.KL; ++l)
                        T[l] = make_double2(T[l - 1].x * e1.x - T[l - 1].y * e1.y, T[l - 1].x * e1.y + T[l - 1].y * e1.x);
                } else {
                    const int K = ax == 1 ? w.KM : w.KN;
                    double2* T = (ax == 1 ? em + s * nm : en + s * nn) + K;
                    T[0] = make_double2(1.0, 0.0);
                    if (K >= 1) T[1] = e1;
                    for (int l = 2; l <= K; ++l)
                        T[l] = make_double2(T[l - 1].x * e1.x - T[l - 1].y * e1.y, T[l - 1].x * e1.y + T[l - 1].y * e1.x);
                    for (int l = 1; l <= K; ++l) T[-l] = make_double2(T[l].x, -T[l].y);
                }
            }
            __syncthreads();
            for (int k = t; k < w.nk; k += kWT) {
                const int3 kv = w.kvec[k];
                double xr = 0.0, xi = 0.0;
#pragma unroll
                for (int s = 0; s < 3; ++s) {
                    const double2 a = el[s * nl + kv.x], b = em[s * nm + kv.y + w.KM], c = en[s * nn + kv.z + w.KN];
                    const double lr_ = qs3[s] * (a.x * b.x - a.y * b.y), li_ = qs3[s] * (a.x * b.y + a.y * b.x);
                    xr += lr_ * c.x - li_ * c.y;
                    xi += lr_ * c.y + li_ * c.x;
                }
                const double2 sk = w.sk[k], q = w.qw[k];
                const double qr = sk.x + q.x, qi = sk.y + q.y;
                uk += 0.5 * w.ak[k] * (xr * qr + xi * qi);
            }

        } else {
            // ---- the same terms in FP32: site offsets from the O, neighbour sites from the FP32
            // copy of rs and q
            const float qx3[3] = {(float)(v.facq * qs3[0]), (float)(v.facq * qs3[1]), (float)(v.facq * qs3[2])};
            float dsx[3], dsy[3], dsz[3];
#pragma unroll
            for (int ix = 0; ix < 3; ++ix) {
                dsx[ix] = (float)(sx[ix] - ox);
                dsy[ix] = (float)(sy[ix] - oy);
                dsz[ix] = (float)(sz[ix] - oz);
            }
            const float alfa = (float)v.alfa;
            float urf = 0.f;
            for (int k = t; k < nnb; k += kWT) {
                const int j = nb_j[k];
                const float xio = (float)nb_d[3 * k], yio = (float)nb_d[3 * k + 1], zio = (float)nb_d[3 * k + 2];
                const int jt = v.type[j];
                if (jt == 0) {
                    const int njx = v.nsi[jt];
                    for (int ix = 0; ix < 3; ++ix) {
                        const float xi = xio + dsx[ix], yi = yio + dsy[ix], zi = zio + dsz[ix];
                        for (int jx = (ix == 0 ? j + 1 : j); jx < j + njx; ++jx) {
                            const float4 qj = w.rsf[jx];
                            const float xd = xi - qj.x, yd = yi - qj.y, zd = zi - qj.z;
                            const float r2 = xd * xd + yd * yd + zd * zd;
                            const float ri = rsqrtf(r2);
                            urf += ewald_ef(r2 * ri, alfa) * (qx3[ix] * qj.w * ri);
                        }
                    }
                } else {
                    const float qj = w.rsf[j].w;
                    for (int ix = 1; ix < 3; ++ix) {
                        const float xi = xio + dsx[ix], yi = yio + dsy[ix], zi = zio + dsz[ix];
                        const float r2 = xi * xi + yi * yi + zi * zi;
                        const float ri = rsqrtf(r2);
                        urf += ewald_ef(r2 * ri, alfa) * (qx3[ix] * qj * ri);
                    }
                }
            }
            ur = (double)urf;
            float2* elf = reinterpret_cast<float2*>(tab);
            float2* emf = elf + 3 * nl;
            float2* enf = emf + 3 * nm;
            if (t < 9) {
                const int s = t / 3, ax = t % 3;
                const double ang = ax == 0 ? w.pipix * sx[s] : (ax == 1 ? w.pipiy * sy[s] : w.pipiz * sz[s]);
                double cd, sd;
                sincos(ang, &sd, &cd);
                const float2 e1 = make_float2((float)cd, (float)sd);
                if (ax == 0) {
                    float2* T = elf + s * nl;
                    T[0] = make_float2(1.f, 0.f);
                    if (w.KL >= 1) T[1] = e1;
                    for (int l = 2; l <= w.KL; ++l)
                        T[l] = make_float2(T[l - 1].x * e1.x - T[l - 1].y * e1.y, T[l - 1].x * e1.y + T[l - 1].y * e1.x);
                } else {
                    const int K = ax == 1 ? w.KM : w.KN;
                    float2* T = (ax == 1 ? emf + s * nm : enf + s * nn) + K;
                    T[0] = make_float2(1.f, 0.f);
                    if (K >= 1) T[1] = e1;
                    for (int l = 2; l <= K; ++l)
                        T[l] = make_float2(T[l - 1].x * e1.x - T[l - 1].y * e1.y, T[l - 1].x * e1.y + T[l - 1].y * e1.x);
                    for (int l = 1; l <= K; ++l) T[-l] = make_float2(T[l].x, -T[l].y);
                }
            }
            __syncthreads();
            const float q3f[3] = {(float)qs3[0], (float)qs3[1], (float)qs3[2]};
            float ukf = 0.f;
            for (int k = t; k < w.nk; k += kWT) {
                const int3 kv = w.kvec[k];
                float xr = 0.f, xi = 0.f;
#pragma unroll
                for (int s = 0; s < 3; ++s) {
                    const float2 a = elf[s * nl + kv.x], b = emf[s * nm + kv.y + w.KM], cc = enf[s * nn + kv.z + w.KN];
                    const float lr_ = q3f[s] * (a.x * b.x - a.y * b.y), li_ = q3f[s] * (a.x * b.y + a.y * b.x);
                    xr += lr_ * cc.x - li_ * cc.y;
                    xi += lr_ * cc.y + li_ * cc.x;
                }
                const float2 q = w.qsf[k];
                ukf += 0.5f * w.akf[k] * (xr * q.x + xi * q.y);
            }
            uk = (double)ukf;
        }
        const double u_real = block_sum_d(ur, red);
        const double u_rec = block_sum_d(uk, red);
        if (t == 0) {
            double u = u_real + ux + u_rec;
            u -= w.crf * (w.q0 * sz[0] + w.q1 * sz[1] + w.q1 * sz[2]);
            const int nit = v.nit;
            for (int j = -1; j <= 1; j += 2) {
                const double dw = v.lwh - (double)j * oz;
                if (dw < v.rcut) {
                    u += w.lr[8 * nit];
                } else {
                    u += w.lr[7 * nit];
                    const double dw3 = dw * dw * dw;
                    u += (w.lr[2 * nit] / (9.0 * (dw3 * dw3 * dw3)) - w.lr[3 * nit] / (3.0 * dw3));
                    const double tt = w.lr[6 * nit];
                    const double exp2a = w.lr[4 * nit] * exp(-dw / tt);
                    u += (tt * (2.0 * tt + dw) * exp2a - w.lr[5 * nit] / (3.0 * dw3));
                }
            }
            acc += exp(-w.beta * u);
        }
        __syncthreads();  // tables are rebuilt for the next orientation
    }
    if (t == 0) w.res[ins] = make_double2(acc, 0.0);
}

// The reference's generator: seed <- mod(8192 seed, 67099547), rnd = seed * 1.4903230270690e-8.
inline double rnd(double& seed) {
    seed = std::fmod(8192.0 * seed, 67099547.0);
    return seed * 1.4903230270690e-8;
}

}  // namespace

int widom(Ctx& c, const mdg_widom_params* p, double* seed, double* pave, int64_t* inave, int64_t* done) {
    View& v = c.v;
    KSet& ks = c.ks;
    if (c.variant != MDG_SLAB) return set_err(&c, MDG_E_UNSUPPORTED, "Widom insertion: slab variant only");
    if (!p || !seed || !pave || !inave || p->ichmax < 0 || p->lchmax < 1 || !(p->lwmax > p->lwmin))
        return set_err(&c, MDG_E_ARG, "Widom insertion: bad arguments");
    if (done) *done = 0;
    const int64_t nins = p->ichmax;
    if (nins == 0) return MDG_OK;
    // measure_init (src/measure.f90:151-155): distances from the wall -> distances from the centre
    const double lwh = v.lwh;
    const double zlo = lwh - p->lwmax, zhi = lwh - p->lwmin;
    const double facbin = 1.0 / (zhi - zlo) * (double)(float)p->lchmax;
    const double chtemper = p->temper > 0.0 ? p->temper : 300.0;
    const double beta = 1000.0 / ((double)8.31441f * chtemper);
    const double M_PI_R = (double)3.1415926535898f;
    const double aco = (double)-0.333333f, asi = (double)0.942809f;
    // draw the positions and orientations in the reference's order (src/forcem.f90:1256-1377)
    std::vector<double> hp(4 * nins), hr((size_t)nins * kMaxRot * 6, 0.0), seed_pos(nins), seed_rot(nins);
    std::vector<int> hn(nins), hil(nins);
    double sd = *seed;
    for (int64_t ic = 0; ic < nins; ++ic) {
        const double oxr = (rnd(sd) - 0.5) * v.lx;
        const double oyr = (rnd(sd) - 0.5) * v.ly;
        double ozr;
        for (int guard = 0;; ++guard) {
            ozr = ((rnd(sd) - 0.5) * zhi * 2.0);
            if (std::fabs(ozr) > zlo) break;
            if (guard > 100000000) return set_err(&c, MDG_E_ARG, "Widom insertion: empty band");
        }
        seed_pos[ic] = sd;
        const int il = (int)((std::fabs(ozr) - zlo) * facbin) + 1;
        if (il < 1 || il > p->lchmax) return set_err(&c, MDG_E_ARG, "Widom insertion: bin outside lchmax");
        hil[ic] = il;
        hn[ic] = il > p->ilmid ? 20 : 1;
        hp[4 * ic] = oxr;
        hp[4 * ic + 1] = oyr;
        hp[4 * ic + 2] = ozr;
        for (int ir = 0; ir < hn[ic]; ++ir) {
            double h1[3], ri;
            for (;;) {
                h1[0] = rnd(sd) - 0.5;
                h1[1] = rnd(sd) - 0.5;
                h1[2] = rnd(sd) - 0.5;
                ri = h1[0] * h1[0] + h1[1] * h1[1] + h1[2] * h1[2];
                if (ri < 0.25 && ri > (double)0.001f) break;
            }
            ri = 1.0 / std::sqrt(ri);
            for (double& hh : h1) hh = hh * ri;
            ri = 1.0 / std::sqrt(h1[0] * h1[0] + h1[1] * h1[1]);
            const double h2[3] = {-h1[1] * ri, h1[0] * ri, 0.0};
            const double mr[3] = {h2[1] * h1[2] - h2[2] * h1[1], h2[2] * h1[0] - h2[0] * h1[2],
                                  h2[0] * h1[1] - h2[1] * h1[0]};
            const double alph = 2.0 * M_PI_R * rnd(sd);
            const double cosa = std::cos(alph), sina = std::sin(alph);
            const double o[3] = {oxr, oyr, ozr};
            double* dst = &hr[((size_t)ic * kMaxRot + ir) * 6];
            for (int d = 0; d < 3; ++d) {
                dst[d] = o[d] + aco * h1[d] + asi * (cosa * h2[d] + sina * mr[d]);
                dst[3 + d] = o[d] + h1[d];
            }
        }
        seed_rot[ic] = sd;
    }
    // device scratch, grown on demand
    if (c.widom_cap < nins) {
        const int64_t cap = std::max<int64_t>(nins, 256);
        c.d_widom_pos = (double*)dalloc(c, sizeof(double) * 4 * cap);
        c.d_widom_rot = (double*)dalloc(c, sizeof(double) * cap * kMaxRot * 6);
        c.d_widom_n = (int*)dalloc(c, sizeof(int) * cap);
        c.d_widom_res = (double*)dalloc(c, sizeof(double) * 2 * cap);
        if (c.alloc_failed) return set_err(&c, MDG_E_CUDA, "Widom insertion: out of device memory");
        c.widom_cap = cap;
    }
    MDG_CUDA(cudaMemcpyAsync(c.d_widom_pos, hp.data(), sizeof(double) * 4 * nins, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(c.d_widom_rot, hr.data(), sizeof(double) * hr.size(), cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(c.d_widom_n, hn.data(), sizeof(int) * nins, cudaMemcpyHostToDevice, c.stream));
    double dipz = 0.0;
    if (p->flags & MDG_WIDOM_EW3DC)
        MDG_CUDA(cudaMemcpy(&dipz, v.acc + 2 * v.nijt + ACC_DIPZ, sizeof(double), cudaMemcpyDeviceToHost));
    WArgs w;
    w.pos = reinterpret_cast<const double4*>(c.d_widom_pos);
    w.rot = c.d_widom_rot;
    w.nrot = c.d_widom_n;
    w.res = reinterpret_cast<double2*>(c.d_widom_res);
    w.kvec = ks.kvec;
    w.ak = ks.ak;
    w.sk = ks.s;
    w.qw = ks.qw;
    w.lr = c.d_lr;
    w.nk = ks.nk;
    w.KL = ks.klmax;
    w.KM = ks.kmmax;
    w.KN = ks.knmax;
    w.pipix = ks.pipix;
    w.pipiy = ks.pipiy;
    w.pipiz = ks.pipiz;
    w.beta = beta;
    w.rinsmin = 4.0;                        // 2.0**2
    w.rwinsmin = (double)(2.35f * 2.35f);   // 2.35**2 in default real
    const double crf0 = -2.0 * M_PI_R * v.lzi * v.lxi * v.lyi;
    w.crf = (p->flags & MDG_WIDOM_EW3DC) ? 2.0 * crf0 * v.facq * dipz : 0.0;
    w.q0 = (double)-0.8476f;
    w.q1 = (double)0.4238f;
    const size_t smem = sizeof(int) * kWNb + sizeof(double) * 3 * kWNb +
                        sizeof(double2) * 3 * (size_t)((ks.klmax + 1) + (2 * ks.kmmax + 1) + (2 * ks.knmax + 1));
    const bool mx = c.precision == MDG_MIXED;
    if (!c.widom_attr) {
        MDG_CUDA(allow_max_smem(k_widom<false>));
        MDG_CUDA(allow_max_smem(k_widom<true>));
        c.widom_attr = true;
    }
    w.qsf = nullptr;
    w.akf = nullptr;
    w.rsf = nullptr;
    if (mx) {
        if (!c.d_widom_akf) {
            std::vector<float> akf(std::max(ks.nk, 1));
            std::vector<double> ak(ks.nk);
            if (ks.nk) MDG_CUDA(cudaMemcpy(ak.data(), ks.ak, sizeof(double) * ks.nk, cudaMemcpyDeviceToHost));
            for (int k = 0; k < ks.nk; ++k) akf[k] = (float)ak[k];
            c.d_widom_akf = (float*)dalloc(c, sizeof(float) * akf.size());
            c.d_widom_qsf = (float2*)dalloc(c, sizeof(float2) * akf.size());
            c.d_widom_rsf = (float4*)dalloc(c, sizeof(float4) * std::max(v.ntota, 1));
            if (c.alloc_failed) return set_err(&c, MDG_E_CUDA, "Widom insertion: out of device memory");
            MDG_CUDA(cudaMemcpy(c.d_widom_akf, akf.data(), sizeof(float) * akf.size(), cudaMemcpyHostToDevice));
        }
        const int np = std::max(std::max(ks.nk, v.ntota), 1);
        k_widom_prep<<<std::min((np + 255) / 256, 152 * 4), 256, 0, c.stream>>>(v, ks.s, ks.qw, c.d_widom_qsf, ks.nk,
                                                                             c.d_widom_rsf);
        w.qsf = c.d_widom_qsf;
        w.akf = c.d_widom_akf;
        w.rsf = c.d_widom_rsf;
        k_widom<true><<<(unsigned)nins, kWT, smem, c.stream>>>(v, w);
    } else {
        k_widom<false><<<(unsigned)nins, kWT, smem, c.stream>>>(v, w);
    }
    MDG_CUDA(cudaGetLastError());
    std::vector<double> res(2 * nins);
    MDG_CUDA(cudaMemcpyAsync(res.data(), c.d_widom_res, sizeof(double) * 2 * nins, cudaMemcpyDeviceToHost, c.stream));
    MDG_CUDA(cudaStreamSynchronize(c.stream));
    // the reference's accumulation: inave counts the tries of every position drawn, including the
    // one that overlaps; the first overlap ends the call unless overlaps are skipped
    int64_t n = 0;
    for (int64_t ic = 0; ic < nins; ++ic) {
        const int st = (int)res[2 * ic + 1];
        if (st == 2) return set_err(&c, MDG_E_LIST_OVERFLOW, "Widom insertion: more than 1024 sites around the probe");
        inave[hil[ic] - 1] += hn[ic];
        ++n;
        if (st == 1) {
            if (!(p->flags & MDG_WIDOM_SKIP_OVERLAP)) {
                *seed = seed_pos[ic];
                if (done) *done = n;
                return MDG_OK;
            }
            continue;
        }
        pave[hil[ic] - 1] += res[2 * ic];
    }
    *seed = seed_rot[nins - 1];
    if (done) *done = n;
    return MDG_OK;
}

}  // namespace mdg
