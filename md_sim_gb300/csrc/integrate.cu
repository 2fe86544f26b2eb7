// integrate.cu - the MD step around the force phases, on the device (resident mode).
//
//   k_pred   move_predict, src/move.f90:48-217: 5-value Gear predictor for ions, centres of mass,
//            angular velocities and quaternions; quaternion normalisation, rotation matrix, site
//            rebuild and the H offsets rsx (:148-162); the block that finishes last computes the
//            kinetic energies, the Nose-like thermostat predictor, htot and sft/sfr.
//   k_corr   move_correct, src/move.f90:220-383, for ions and rigid molecules; its last block adds
//            uconf and press of force_sum (src/forcem.f90:1055,1079,1081) and the thermostat
//            corrector.
//
// One thread per ion or molecule in small blocks (the FP64 work of one molecule is a long
// dependent chain, so the molecules are spread over as many SMs as possible); kinetic sums go
// through block reductions into a small accumulator array that the last block reads and clears.
// Gear coefficients are the reference's single-precision literals.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "ctx.h"
#include "merge.cuh"
#include "pack.cuh"

namespace mdg {

namespace {

// A warp serves `lanes` molecules. An FP64 instruction costs the SM's FP64 pipe about the same
// whatever the number of active lanes, so large systems pack 32 molecules per warp (blocks of four
// warps); small ones spread one warp per SM with just enough molecules to cover the system, since
// there the per-molecule chain of dependent FP64 operations sets the time, and with at most 16
// molecules per warp each molecule takes a pair of lanes (centre and angular velocity on one,
// orientation on the other) to shorten that chain.
constexpr int kSM = 152;

// unit served by this thread in sweep `r` of the grid-stride loop over the first `nb` blocks, or -1
template <int NT>
__device__ __forceinline__ int unit_of(int lanes, int r, int nb) {
    const int lane = threadIdx.x & 31;
    if (lane >= lanes) return -1;
    const int gw = blockIdx.x * (NT / 32) + (threadIdx.x >> 5);
    return (r * nb * (NT / 32) + gw) * lanes + lane;
}

// the same for lane pairs (two lanes per unit, `lanes` units per warp, lanes <= 16): role = lane & 1
template <int NT>
__device__ __forceinline__ int unit_of_pair(int lanes, int r, int nb, int& role) {
    const int lane = threadIdx.x & 31, slot = lane >> 1;
    role = lane & 1;
    if (slot >= lanes) return -1;
    const int gw = blockIdx.x * (NT / 32) + (threadIdx.x >> 5);
    return (r * nb * (NT / 32) + gw) * lanes + slot;
}

constexpr double Gf01 = F32D(0.348611111), Gf11 = 1.0, Gf21 = F32D(0.916666667), Gf31 = F32D(0.333333333),
                 Gf41 = F32D(0.041666667);
constexpr double Gf02 = F32D(0.158300000), Gf12 = F32D(0.757000000), Gf22 = 1.0, Gf32 = 0.5,
                 Gf42 = F32D(0.083333333);

__device__ __forceinline__ void gpred(double& a0, double& a1, double& a2, double& a3, double a4) {
    a0 = a0 + a1 + a2 + a3 + a4;
    a1 = a1 + 2 * a2 + 3 * a3 + 4 * a4;
    a2 = a2 + 3 * a3 + 6 * a4;
    a3 = a3 + 4 * a4;
}

struct Dyn {
    unsigned* done;  // [2] blocks finished (k_pred, k_corr), reset by the last block
    double* xd;     // [4][3][nion]
    double* c;      // [5][3][nrig]
    double* q;      // [4][5][nrig]
    double* w;      // [5][3][nrig]
    double* a;      // [9][nrig]
    double* th;     // thermostat + scalars
    double* isum;   // kinetic partial sums
    const double* ft;  // 3 x nflex
    const double* fc;  // 3 x nrig
    const double* tq;  // 3 x nrig
    mdg_rigid body;
    int nion;
};

__device__ __forceinline__ double pred_ion(const View& v, const Dyn& D, int k, double* xn) {
    const int n = D.nion;
    const int i = v.nriga + k;
    double* X[3] = {v.x, v.y, v.z};
    double s2 = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double* x1 = D.xd + (0 * 3 + d) * n;
        double* x2 = D.xd + (1 * 3 + d) * n;
        double* x3 = D.xd + (2 * 3 + d) * n;
        double* x4 = D.xd + (3 * 3 + d) * n;
        double a0 = X[d][i], a1 = x1[k], a2 = x2[k], a3 = x3[k];
        gpred(a0, a1, a2, a3, x4[k]);
        X[d][i] = a0;
        xn[d] = a0;
        x1[k] = a1;
        x2[k] = a2;
        x3[k] = a3;
        s2 += a1 * a1;
    }
    return v.mi[i] * s2;
}

// True in every thread of the block that finished last; each block's atomics are visible before
// it counts itself done.
__device__ __forceinline__ bool last_block(unsigned* done) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    return last;
}

// Register arithmetic of the rigid-body predictor and corrector, shared by the one-lane forms and
// the lane-pair forms below (the same operations in the same order, so both give the same bits).

// rotation matrix of the normalised predicted quaternion (src/move.f90:128-146)
__device__ __forceinline__ void quat_rot(const double* qq, double* qn, double* a) {
    const double cr = 1.0 / sqrt(qq[0] * qq[0] + qq[1] * qq[1] + qq[2] * qq[2] + qq[3] * qq[3]);
    const double q1 = qq[0] * cr, q2 = qq[1] * cr, q3 = qq[2] * cr, q4 = qq[3] * cr;
    qn[0] = q1;
    qn[1] = q2;
    qn[2] = q3;
    qn[3] = q4;
    a[0] = -q1 * q1 + q2 * q2 - q3 * q3 + q4 * q4;
    a[1] = 2.0 * (q3 * q4 - q1 * q2);
    a[2] = 2.0 * (q2 * q3 + q1 * q4);
    a[3] = -2.0 * (q1 * q2 + q3 * q4);
    a[4] = q1 * q1 - q2 * q2 - q3 * q3 + q4 * q4;
    a[5] = 2.0 * (q2 * q4 - q1 * q3);
    a[6] = 2.0 * (q2 * q3 - q1 * q4);
    a[7] = -2.0 * (q1 * q3 + q4 * q2);
    a[8] = -q1 * q1 - q2 * q2 + q3 * q3 + q4 * q4;
}

// lab-frame position of site j (src/move.f90:148-162)
__device__ __forceinline__ void site_pos(const double* cx, const double* a, const mdg_rigid& b, int j, double& x,
                                         double& y, double& z) {
    x = cx[0] + a[0] * b.xbody[j] + a[3] * b.ybody[j] + a[6] * b.zbody[j];
    y = cx[1] + a[1] * b.xbody[j] + a[4] * b.ybody[j] + a[7] * b.zbody[j];
    z = cx[2] + a[2] * b.xbody[j] + a[5] * b.ybody[j] + a[8] * b.zbody[j];
}

__device__ __forceinline__ void load_cw(const Dyn& D, int nr, int i, double (&C)[5][3], double (&W)[5][3]) {
#pragma unroll
    for (int k = 0; k < 5; ++k)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            C[k][d] = D.c[(k * 3 + d) * nr + i];
            W[k][d] = D.w[(k * 3 + d) * nr + i];
        }
}

__device__ __forceinline__ void load_q(const Dyn& D, int nr, int i, double (&Q)[5][4]) {
#pragma unroll
    for (int k = 0; k < 5; ++k)
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) Q[k][cc] = D.q[(cc * 5 + k) * nr + i];
}

// predictor of the centre and angular velocity; stores their first four derivatives
__device__ __forceinline__ void pred_cw(const Dyn& D, int nr, int i, double (&C)[5][3], double (&W)[5][3], double* sc,
                                        double* sw, double* cx) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        gpred(C[0][d], C[1][d], C[2][d], C[3][d], C[4][d]);
        sc[d] += C[1][d] * C[1][d];
        cx[d] = C[0][d];
        gpred(W[0][d], W[1][d], W[2][d], W[3][d], W[4][d]);
        sw[d] += W[0][d] * W[0][d];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
        for (int k = 0; k < 4; ++k) D.c[(k * 3 + d) * nr + i] = C[k][d];
#pragma unroll
        for (int k = 0; k < 4; ++k) D.w[(k * 3 + d) * nr + i] = W[k][d];
    }
}

// predictor of the orientation; stores the quaternion derivatives and the rotation matrix
__device__ __forceinline__ void pred_q(const Dyn& D, int nr, int i, double (&Q)[5][4], double* a) {
    double qq[4], qn[4];
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
        gpred(Q[0][cc], Q[1][cc], Q[2][cc], Q[3][cc], Q[4][cc]);
        qq[cc] = Q[0][cc];
    }
    quat_rot(qq, qn, a);
#pragma unroll
    for (int cc = 0; cc < 4; ++cc)
#pragma unroll
        for (int k = 1; k < 4; ++k) D.q[(cc * 5 + k) * nr + i] = Q[k][cc];
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) D.q[(cc * 5) * nr + i] = qn[cc];
#pragma unroll
    for (int k = 0; k < 9; ++k) D.a[k * nr + i] = a[k];
}

// All of a molecule's state is loaded before anything is stored: the arrays may alias as far as
// the compiler knows, and loads issued back to back overlap their latency instead of queueing
// behind the stores (the per-molecule work is short; memory latency, not FP64, bounds it).
__device__ __forceinline__ void pred_rigid(const View& v, const Dyn& D, int i, double* sc, double* sw, double* cn,
                                           double* sx, double* sy, double* sz) {
    const int nr = v.nrig;
    double C[5][3], W[5][3], Q[5][4], a[9];
    load_cw(D, nr, i, C, W);
    load_q(D, nr, i, Q);
    pred_cw(D, nr, i, C, W, sc, sw, cn);
    pred_q(D, nr, i, Q, a);
    const int ix = 3 * i;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        site_pos(cn, a, D.body, j, sx[j], sy[j], sz[j]);
        v.x[ix + j] = sx[j];
        v.y[ix + j] = sy[j];
        v.z[ix + j] = sz[j];
    }
#pragma unroll
    for (int j = 1; j < 3; ++j) {
        v.rsx[ix + j] = sx[j] - sx[0];
        v.rsy[ix + j] = sy[j] - sy[0];
        v.rsz[ix + j] = sz[j] - sz[0];
    }
}

// The same on a pair of lanes (mask: the lanes of the pairs on rigid molecules this sweep): role 0
// predicts the centre and angular velocity, role 1 the orientation; after the exchange of the
// centre and the rotation matrix, role 0 places sites 0 and 1, role 1 sites 0 and 2 (returned in
// slots 0 and 1; each writes its own besides site 0, which role 0 writes).
__device__ __forceinline__ void pred_rigid_pair(const View& v, const Dyn& D, int i, int role, unsigned mask,
                                                double* sc, double* sw, double* cn, double* sx, double* sy,
                                                double* sz) {
    const int nr = v.nrig;
    double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    cn[0] = cn[1] = cn[2] = 0.0;
    if (role == 0) {
        double C[5][3], W[5][3];
        load_cw(D, nr, i, C, W);
        pred_cw(D, nr, i, C, W, sc, sw, cn);
    } else {
        double Q[5][4];
        load_q(D, nr, i, Q);
        pred_q(D, nr, i, Q, a);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double t = __shfl_xor_sync(mask, role ? a[k] : cn[k], 1);
        if (role) cn[k] = t;
        else a[k] = t;
    }
#pragma unroll
    for (int k = 3; k < 9; ++k) {
        const double t = __shfl_xor_sync(mask, a[k], 1);
        if (!role) a[k] = t;
    }
    const int ix = 3 * i, j1 = role ? 2 : 1;
    site_pos(cn, a, D.body, 0, sx[0], sy[0], sz[0]);
    site_pos(cn, a, D.body, j1, sx[1], sy[1], sz[1]);
    if (role == 0) {
        v.x[ix] = sx[0];
        v.y[ix] = sy[0];
        v.z[ix] = sz[0];
    }
    v.x[ix + j1] = sx[1];
    v.y[ix + j1] = sy[1];
    v.z[ix + j1] = sz[1];
    v.rsx[ix + j1] = sx[1] - sx[0];
    v.rsy[ix + j1] = sy[1] - sy[0];
    v.rsz[ix + j1] = sz[1] - sz[0];
}

// thermostat predictor and kinetic energies from the summed isum[0..6] (one thread).  Runs in the
// tail of a kernel, where every dependent round trip to L2 is about a microsecond: all loads are
// issued first, into registers, then the arithmetic, then the stores.
struct ThermoIn {
    double is[7], s[5], rs[5], uc;
};

__device__ __forceinline__ ThermoIn thermo_pred_load(const Dyn& D) {
    ThermoIn t;
#pragma unroll
    for (int k = 0; k < 7; ++k) t.is[k] = __ldcg(&D.isum[k]);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        t.s[k] = __ldcg(&D.th[TH_S + k]);
        t.rs[k] = __ldcg(&D.th[TH_RS + k]);
    }
    t.uc = __ldcg(&D.th[TH_UCONF]);
    return t;
}

__device__ void thermo_pred(const View& v, const Dyn& D, ThermoIn t) {
    double* th = D.th;
    const mdg_rigid& b = D.body;
    double* is = t.is;
    double* s = t.s;
    double* rs = t.rs;
    const double uc = t.uc;
    const double kp = is[0] + b.mw * (is[1] + is[2] + is[3]);
    const double kw = b.inxx * is[4] + b.inyy * is[5] + b.inzz * is[6];
    if (b.temper == -1.0) {
        s[0] = s[1] = rs[0] = rs[1] = 0.0;
    } else {
        gpred(s[0], s[1], s[2], s[3], s[4]);
        gpred(rs[0], rs[1], rs[2], rs[3], rs[4]);
    }
    const long nfree = v.nliqa - v.nriga;
    const double tstar = F32D(8.31441) * b.temper / 1000.0;
    double qmass = (double)(float)(3 * (nfree + v.nrig)) * tstar * F32D(2e3);
    double rmass = (double)(float)(3 * v.nrig) * tstar * F32D(1e3);
    qmass = qmass / 10.0;
    rmass = rmass / 10.0;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        th[TH_S + k] = s[k];
        th[TH_RS + k] = rs[k];
    }
    th[TH_KP] = kp;
    th[TH_KW] = kw;
    th[TH_KE] = kp + kw;
    th[TH_HTOT] = 0.5 * (kp + kw + qmass * s[0] * s[0] + rmass * rs[0] * rs[0]) + uc;
    th[TH_SFT] = (kp - (double)(float)(3 * (nfree + v.nrig) - 2) * tstar) / qmass;
    th[TH_SFR] = (kw - (double)(float)(3 * v.nrig + 1) * tstar) / rmass;
#pragma unroll
    for (int k = 0; k < 7; ++k) D.isum[k] = 0.0;  // ready for the next step
}

// Sums that the rest of the step accumulates into, zeroed by the predictor (block 0) so that the
// step graph needs no memset nodes.
struct Clear {
    double* p[2];
    int n[2];
};

// The records of the force evaluation that follows (pack.cuh), written by the predictor of a
// resident mixed-precision step from the positions it has just computed: blocks below npred
// predict and pack their molecules and flexible atoms, the blocks after them pack the wall atoms.
struct PackArgs {
    Pk pk;
    int dip;    // slab dipole term
    int npred;  // blocks of the predictor proper
};

// A packing predictor has no tail: block 0 clears the energy sums first (all but the displacement
// maximum, which the blocks raise as they go), and the close of the packing and the thermostat
// predictor run in k_step_close on the list's stream, off the path of the reciprocal sum.
template <int NT, bool PACK, bool PAIR>
__global__ void __launch_bounds__(NT) k_pred(View v, Dyn D, int lanes, Clear z, PackArgs P) {
    __shared__ double red[8];
    double kp = 0.0, sc[3] = {0, 0, 0}, sw[3] = {0, 0, 0};
    double mz = 0.0, md = 0.0;
    const int nu = D.nion + v.nrig;
    const int npred = PACK ? P.npred : gridDim.x;
    if (blockIdx.x == 0) {
        for (int j = 0; j < 2; ++j)
            for (int k = threadIdx.x; k < z.n[j]; k += NT) z.p[j][k] = 0.0;
        if constexpr (PACK) {
            const int na = 2 * v.nijt + ACC_NSLOT, kmax = 2 * v.nijt + ACC_MAXD;
            for (int k = threadIdx.x; k < na; k += NT)
                if (k != kmax) v.acc[k] = 0.0;
            if (P.pk.cmax && threadIdx.x == 0) *P.pk.cmax = 0.f;
        }
    }
    if (blockIdx.x < npred) {
        for (int r = 0;; ++r) {
            int u, role = 0;
            if constexpr (PAIR) u = unit_of_pair<NT>(lanes, r, npred, role);
            else u = unit_of<NT>(lanes, r, npred);
            const bool act = u >= 0 && u < nu;
            unsigned mask = 0u;
            if constexpr (PAIR) {
                if (!__any_sync(0xffffffffu, act)) break;
                mask = __ballot_sync(0xffffffffu, act && u >= D.nion);
                if (!act) continue;
            } else {
                if (!act) break;
            }
            if (u < D.nion) {
                if (role != 0) continue;
                double xn[3];
                kp += pred_ion(v, D, u, xn);
                if constexpr (PACK) {
                    const int at = v.nriga + u;
                    const double a = v.ox[u] - xn[0], b = v.oy[u] - xn[1], c = v.oz[u] - xn[2];
                    md = fmax(md, a * a + b * b + c * c);
                    mz += pack_atom(v, P.pk, at, xn[0], xn[1], xn[2], v.rsx[at], v.rsy[at], v.rsz[at], true);
                }
                continue;
            }
            const int i = u - D.nion, ix = 3 * i;
            double cn[3], px[3], py[3], pz[3];
            if constexpr (PAIR) {
                pred_rigid_pair(v, D, i, role, mask, sc, sw, cn, px, py, pz);
                if constexpr (PACK) {
                    // site 0's offset is the stored one (force_sum leaves rsx(1:3) stale), the others
                    // the offsets just computed, as the packing kernel would read them back
                    if (role == 0) {
                        const double a = v.ocx[i] - cn[0], b = v.ocy[i] - cn[1], c = v.ocz[i] - cn[2];
                        md = fmax(md, a * a + b * b + c * c);
                        mz += pack_atom(v, P.pk, ix, px[0], py[0], pz[0], v.rsx[ix], v.rsy[ix], v.rsz[ix], true);
                        mz += pack_atom(v, P.pk, ix + 1, px[1], py[1], pz[1], px[1] - px[0], py[1] - py[0],
                                        pz[1] - pz[0], true);
                    } else {
                        mz += pack_atom(v, P.pk, ix + 2, px[1], py[1], pz[1], px[1] - px[0], py[1] - py[0],
                                        pz[1] - pz[0], true);
                    }
                }
            } else {
                pred_rigid(v, D, i, sc, sw, cn, px, py, pz);
                if constexpr (PACK) {
                    const double a = v.ocx[i] - cn[0], b = v.ocy[i] - cn[1], c = v.ocz[i] - cn[2];
                    md = fmax(md, a * a + b * b + c * c);
                    mz += pack_atom(v, P.pk, ix, px[0], py[0], pz[0], v.rsx[ix], v.rsy[ix], v.rsz[ix], true);
#pragma unroll
                    for (int j = 1; j < 3; ++j)
                        mz += pack_atom(v, P.pk, ix + j, px[j], py[j], pz[j], px[j] - px[0], py[j] - py[0],
                                        pz[j] - pz[0], true);
                }
            }
        }
    } else if constexpr (PACK) {
        const int nw = gridDim.x - npred;
        for (int a = v.nmove + (blockIdx.x - npred) * NT + threadIdx.x; a < v.ntota; a += nw * NT)
            pack_atom(v, P.pk, a, v.x[a], v.y[a], v.z[a], 0.0, 0.0, 0.0, false);
    }
    if (blockIdx.x < npred) {
        block_atomic_sum<NT>(kp, &D.isum[0]);
        for (int d = 0; d < 3; ++d) block_atomic_sum<NT>(sc[d], &D.isum[1 + d]);
        for (int d = 0; d < 3; ++d) block_atomic_sum<NT>(sw[d], &D.isum[4 + d]);
    }
    if constexpr (PACK) {
        pack_block(v, P.pk, mz, md, red);
    } else if (last_block(&D.done[0]) && threadIdx.x == 0) {
        thermo_pred(v, D, thermo_pred_load(D));
        D.done[0] = 0u;
    }
}

// After a packing predictor (one block of two warps): the close of its packing (slab dipole from
// the nparts block shares, list rebuild decision) on one warp and the thermostat predictor on the
// other.
__global__ void __launch_bounds__(64) k_step_close(View v, Dyn D, Pk pk, int dip, int nparts) {
    if (threadIdx.x < 32) {
        pack_close_warp(v, pk, dip, 0, 0, nparts, false);
    } else if (threadIdx.x == 32) {
        thermo_pred(v, D, thermo_pred_load(D));
    }
}

__device__ __forceinline__ void corr_ion(const View& v, const Dyn& D, int k) {
    const int n = D.nion;
    const double s0i = D.th[TH_S];
    const int nflex = v.nmove - v.nriga;
    {
        const int i = v.nriga + k;
        double* X[3] = {v.x, v.y, v.z};
        for (int d = 0; d < 3; ++d) {
            double* x1 = D.xd + (0 * 3 + d) * n;
            double* x2 = D.xd + (1 * 3 + d) * n;
            double* x3 = D.xd + (2 * 3 + d) * n;
            double* x4 = D.xd + (3 * 3 + d) * n;
            const double cort = 0.5 * D.ft[d * nflex + k] * v.mii[i] - x1[k] * s0i - x2[k];
            X[d][i] = X[d][i] + Gf02 * cort;
            x1[k] = x1[k] + Gf12 * cort;
            x2[k] = x2[k] + Gf22 * cort;
            x3[k] = x3[k] + Gf32 * cort;
            x4[k] = x4[k] + Gf42 * cort;
        }
    }
}

// corrector of the orientation (Q and the predicted angular velocity w0); stores its derivatives
__device__ __forceinline__ void corr_q(const Dyn& D, int nr, int i, double (&Q)[5][4], const double* w0) {
    const double q1 = Q[0][0], q2 = Q[0][1], q3 = Q[0][2], q4 = Q[0][3];
    const double wx = w0[0], wy = w0[1], wz = w0[2];
    double cq[4];
    cq[0] = 0.5 * (-q3 * wx - q4 * wy + q2 * wz);
    cq[1] = 0.5 * (q4 * wx - q3 * wy - q1 * wz);
    cq[2] = 0.5 * (q1 * wx + q2 * wy + q4 * wz);
    cq[3] = 0.5 * (-q2 * wx + q1 * wy - q3 * wz);
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
        const double co = cq[cc] - Q[1][cc];
        Q[0][cc] = Q[0][cc] + Gf01 * co;
        Q[1][cc] = Q[1][cc] + Gf11 * co;
        Q[2][cc] = Q[2][cc] + Gf21 * co;
        Q[3][cc] = Q[3][cc] + Gf31 * co;
        Q[4][cc] = Q[4][cc] + Gf41 * co;
    }
#pragma unroll
    for (int k = 0; k < 5; ++k)
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) D.q[(cc * 5 + k) * nr + i] = Q[k][cc];
}

// corrector of the centre (force fc) and the angular velocity (torque tq through the rotation
// matrix a); stores their derivatives
__device__ __forceinline__ void corr_cw(const Dyn& D, int nr, int i, double (&C)[5][3], double (&W)[5][3],
                                        const double* a, const double* fc, const double* tq, double s0i,
                                        double rs0i) {
    const mdg_rigid& b = D.body;
    const double rcorr = 0.5 / b.mw;
    const double inxxi = 1.0 / b.inxx, inyyi = 1.0 / b.inyy, inzzi = 1.0 / b.inzz;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double co = rcorr * fc[d] - C[1][d] * s0i - C[2][d];
        C[0][d] = C[0][d] + Gf02 * co;
        C[1][d] = C[1][d] + Gf12 * co;
        C[2][d] = C[2][d] + Gf22 * co;
        C[3][d] = C[3][d] + Gf32 * co;
        C[4][d] = C[4][d] + Gf42 * co;
    }
    const double wx = W[0][0], wy = W[0][1], wz = W[0][2];
    const double tx = tq[0], ty = tq[1], tz = tq[2];
    double c1 = a[0] * tx + a[1] * ty + a[2] * tz;
    c1 = ((c1 * 1.0 + wy * wz * (b.inyy - b.inzz)) * inxxi) - W[1][0] - rs0i * wx;
    double c2 = a[3] * tx + a[4] * ty + a[5] * tz;
    c2 = ((c2 * 1.0 + wz * wx * (b.inzz - b.inxx)) * inyyi) - W[1][1] - rs0i * wy;
    double c3 = a[6] * tx + a[7] * ty + a[8] * tz;
    c3 = ((c3 * 1.0 + wx * wy * (b.inxx - b.inyy)) * inzzi) - W[1][2] - rs0i * wz;
    const double cw[3] = {c1, c2, c3};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        W[0][d] += Gf01 * cw[d];
        W[1][d] += Gf11 * cw[d];
        W[2][d] += Gf21 * cw[d];
        W[3][d] += Gf31 * cw[d];
        W[4][d] += Gf41 * cw[d];
    }
#pragma unroll
    for (int k = 0; k < 5; ++k)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            D.c[(k * 3 + d) * nr + i] = C[k][d];
            D.w[(k * 3 + d) * nr + i] = W[k][d];
        }
}

__device__ __forceinline__ void corr_rigid(const View& v, const Dyn& D, int i) {
    const int nr = v.nrig;
    const double s0i = D.th[TH_S], rs0i = D.th[TH_RS];
    // loads first (see pred_rigid)
    double C[5][3], W[5][3], Q[5][4], a[9], fc[3], tq[3];
    load_cw(D, nr, i, C, W);
    load_q(D, nr, i, Q);
#pragma unroll
    for (int k = 0; k < 9; ++k) a[k] = D.a[k * nr + i];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        fc[d] = D.fc[d * nr + i];
        tq[d] = D.tq[d * nr + i];
    }
    const double w0[3] = {W[0][0], W[0][1], W[0][2]};
    corr_q(D, nr, i, Q, w0);
    corr_cw(D, nr, i, C, W, a, fc, tq, s0i, rs0i);
}

// The same on a pair of lanes: role 0 corrects the centre and angular velocity (with fc, tq),
// role 1 the orientation, with the predicted angular velocity passed over from role 0.
__device__ __forceinline__ void corr_rigid_pair(const View& v, const Dyn& D, int i, int role, unsigned mask,
                                                const double* fc, const double* tq) {
    const int nr = v.nrig;
    const double s0i = D.th[TH_S], rs0i = D.th[TH_RS];
    double C[5][3], W[5][3], Q[5][4], a[9];
    double w0[3] = {0.0, 0.0, 0.0};
    if (role == 0) {
        load_cw(D, nr, i, C, W);
#pragma unroll
        for (int k = 0; k < 9; ++k) a[k] = D.a[k * nr + i];
        w0[0] = W[0][0];
        w0[1] = W[0][1];
        w0[2] = W[0][2];
    } else {
        load_q(D, nr, i, Q);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double t = __shfl_xor_sync(mask, w0[d], 1);
        if (role) w0[d] = t;
    }
    if (role == 0) corr_cw(D, nr, i, C, W, a, fc, tq, s0i, rs0i);
    else corr_q(D, nr, i, Q, w0);
}

constexpr int kTailAcc = 512;  // energy sums staged in shared memory by the corrector's tail

// The corrector's tail, in the block that finished last, as two independent parts on two warps:
// uconf = sum(elj) + sum(eqq) + uewa + urf (src/forcem.f90:1055,1079) and the wall pressure (the
// energy sums loaded by one warp at once into shared memory, then summed by its lane 0 in the
// reference's order), and the thermostat corrector with the step counters.
__device__ void corr_energy(const View& v, const Dyn& D, int slab, double* sh) {
    const int l = threadIdx.x & 31;
    const int na = 2 * v.nijt + ACC_NSLOT;
    const bool staged = na <= kTailAcc;
    if (staged)
        for (int k = l; k < na; k += 32) sh[k] = __ldcg(&v.acc[k]);
    __syncwarp();
    if (l != 0) return;
    double* th = D.th;
    const double* a = staged ? sh : v.acc;
    const double* sl = a + 2 * v.nijt;
    double slj = 0.0, sqq = 0.0;
    for (int k = 0; k < v.nijt; ++k) {
        slj += a[k];
        sqq += a[v.nijt + k];
    }
    double urf = 0.0;
    if (slab) {
        const double crf = -2.0 * F32D(3.1415926535898) * v.lzi * v.lxi * v.lyi;
        urf = -crf * v.facq * sl[ACC_DIPZ] * sl[ACC_DIPZ];
    }
    th[TH_UCONF] = slj + sqq + 0.5 * sl[ACC_UEWA] + urf;
    th[TH_PRESS] = (sl[ACC_FWS + 8] - sl[ACC_FWS + 6]) / (2.0 * v.lx * v.ly) * 1000.0 /
                   (F32D(6.022045e23) * F32D(1e-30)) * F32D(1e-5);
}

// the thermostat corrector and the step counters (one thread; all loads first)
__device__ void corr_thermo(const View& v, const Dyn& D) {
    double* th = D.th;
    double s[5], rs[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        s[k] = __ldcg(&th[TH_S + k]);
        rs[k] = __ldcg(&th[TH_RS + k]);
    }
    const double sft = __ldcg(&th[TH_SFT]), sfr = __ldcg(&th[TH_SFR]), ke = __ldcg(&th[TH_KE]);
    const double steps = __ldcg(&th[TH_STEPS]), nreb = __ldcg(&th[TH_REBUILDS]);
    const int reb = __ldcg(&v.status[ST_REBUILD]);
    if (D.body.temper != -1.0) {
        double rc = sft - s[1];
        s[0] = s[0] + Gf01 * rc;
        s[1] = sft;
        s[2] = s[2] + Gf21 * rc;
        s[3] = s[3] + Gf31 * rc;
        s[4] = s[4] + Gf41 * rc;
        rc = sfr - rs[1];
        rs[0] = rs[0] + Gf01 * rc;
        rs[1] = sfr;
        rs[2] = rs[2] + Gf21 * rc;
        rs[3] = rs[3] + Gf31 * rc;
        rs[4] = rs[4] + Gf41 * rc;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            th[TH_S + k] = s[k];
            th[TH_RS + k] = rs[k];
        }
    }
    const long nfree = v.nliqa - v.nriga;
    th[TH_TEMPNOW] = ke * 1000.0 / (3.0 * F32D(8.31441) * (double)(float)(nfree + 2 * v.nrig));
    th[TH_STEPS] = steps + 1.0;
    if (reb) th[TH_REBUILDS] = nreb + 1.0;
}

// Blocks of one-warp correctors carry a second warp for the tail (as the predictor's).
template <int NT>
struct CorrBlock {
    static constexpr int kThreads = NT == 32 ? 64 : NT;
};

// The correctors read the thermostat values of the predictor; the block that finishes last then
// adds uconf/press and corrects the thermostat.  MERGE: the mixed force form's final merge and
// force_sum (merge.cuh) run here, each unit's just before its corrector, instead of in a kernel
// of their own; units past the molecules and ions are the surface atoms, whose forces SHAKE's
// Verlet step reads next.
template <int NT, bool MERGE, bool PAIR>
__global__ void __launch_bounds__(CorrBlock<NT>::kThreads) k_corr(View v, Dyn D, int slab, int lanes, MergeArgs A) {
    constexpr bool kTailWarp = CorrBlock<NT>::kThreads > NT;
    const int nsurf = MERGE ? v.nmove - v.nliqa : 0;
    const int nu = D.nion + v.nrig + nsurf;
    MergeArgs M;
    if constexpr (MERGE) M = merge_begin(v, A);
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int r = 0; !kTailWarp || threadIdx.x < NT; ++r) {
        int u, role = 0;
        if constexpr (PAIR) u = unit_of_pair<NT>(lanes, r, gridDim.x, role);
        else u = unit_of<NT>(lanes, r, gridDim.x);
        const bool act = u >= 0 && u < nu;
        const bool rigid = act && u >= D.nion && u < D.nion + v.nrig;
        unsigned mask = 0u;
        if constexpr (PAIR) {
            if (!__any_sync(0xffffffffu, act)) break;
            mask = __ballot_sync(0xffffffffu, rigid);
            if (!act) continue;
        } else {
            if (!act) break;
        }
        if (rigid) {
            const int i = u - D.nion;
            if constexpr (PAIR) {
                double fc[3] = {0, 0, 0}, tq[3] = {0, 0, 0};
                if constexpr (MERGE) {
                    merge_rigid_pair(v, M, i, role, mask, sx, sy, sz, fc, tq);
                } else if (role == 0) {
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        fc[d] = D.fc[d * v.nrig + i];
                        tq[d] = D.tq[d * v.nrig + i];
                    }
                }
                corr_rigid_pair(v, D, i, role, mask, fc, tq);
            } else {
                if constexpr (MERGE) merge_rigid(v, M, i, sx, sy, sz);
                corr_rigid(v, D, i);
            }
        } else if (role == 0) {
            if (u < D.nion) {
                if constexpr (MERGE) merge_flex(v, M, u, sx, sy, sz);
                corr_ion(v, D, u);
            } else if constexpr (MERGE) {
                merge_flex(v, M, u - v.nrig, sx, sy, sz);  // surface atom: flexible index nion + s
            }
        }
    }
    if constexpr (MERGE) {
        if (!kTailWarp || threadIdx.x < NT) {
            block_atomic_sum<NT>(sx, &v.acc[2 * v.nijt + ACC_FWS0 + 0]);
            block_atomic_sum<NT>(sy, &v.acc[2 * v.nijt + ACC_FWS0 + 1]);
            block_atomic_sum<NT>(sz, &v.acc[2 * v.nijt + ACC_FWS0 + 2]);
        }
    }
    __shared__ double sh_acc[kTailAcc];
    if (last_block(&D.done[1])) {
        if (threadIdx.x < 32) {
            if (threadIdx.x == 0) D.done[1] = 0u;
            corr_energy(v, D, slab, sh_acc);
        } else if (threadIdx.x == 32) {
            corr_thermo(v, D);
        }
    }
}

Dyn dyn_of(Ctx& c) {
    Dyn D;
    D.done = c.d_done;
    D.xd = c.d_xd;
    D.c = c.d_c;
    D.q = c.d_q;
    D.w = c.d_w;
    D.a = c.d_a;
    D.th = c.d_thermo;
    D.isum = c.d_isum;
    D.ft = c.d_ft;
    D.fc = c.d_fc;
    D.tq = c.d_tq;
    D.body = c.body;
    D.nion = c.v.nliqa - c.v.nriga;
    return D;
}

// molecules per warp, and the block size: one warp per block while a warp per SM covers the
// system, else full warps in blocks of four
int lanes_of(int n) { return std::max(1, std::min(32, (n + kSM - 1) / kSM)); }
int nblk(int n, int nt) {
    const int lanes = lanes_of(n), warps = (n + lanes - 1) / lanes;
    return std::max(1, std::min((warps + nt / 32 - 1) / (nt / 32), kSM * 8));
}

}  // namespace

void predict_launch(Ctx& c, bool clear_acc, bool clear_kps, bool pack) {
    const View& v = c.v;
    Dyn D = dyn_of(c);
    const int nu = D.nion + v.nrig, lanes = lanes_of(nu);
    Clear z{{v.acc, c.d_kps}, {clear_acc ? 2 * v.nijt + ACC_NSLOT : 0, clear_kps && c.d_kps ? v.nit : 0}};
    PackArgs P{};
    if (pack) {
        P.pk = c.pk;
        P.dip = c.variant == MDG_SLAB ? 1 : 0;
    }
    const int nwall = v.ntota - v.nmove;
    if (lanes < 32) {
        const int nb = nblk(nu, 32);
        P.npred = nb;
        const int nwb = pack ? std::min((nwall + 31) / 32, kSM * 8) : 0;
        c.pred_parts = nb + nwb;
        if (lanes <= 16) {  // two lanes per molecule
            if (pack) k_pred<32, true, true><<<nb + nwb, 32, 0, c.stream>>>(v, D, lanes, z, P);
            else k_pred<32, false, true><<<nb, 32, 0, c.stream>>>(v, D, lanes, z, P);
        } else {
            if (pack) k_pred<32, true, false><<<nb + nwb, 32, 0, c.stream>>>(v, D, lanes, z, P);
            else k_pred<32, false, false><<<nb, 32, 0, c.stream>>>(v, D, lanes, z, P);
        }
    } else {
        const int nb = nblk(nu, 128);
        P.npred = nb;
        const int nwb = pack ? std::min((nwall + 127) / 128, kSM * 8) : 0;
        c.pred_parts = nb + nwb;
        if (pack) k_pred<128, true, false><<<nb + nwb, 128, 0, c.stream>>>(v, D, lanes, z, P);
        else k_pred<128, false, false><<<nb, 128, 0, c.stream>>>(v, D, lanes, z, P);
    }
}

void step_close_launch(Ctx& c) {
    k_step_close<<<1, 64, 0, c.stream>>>(c.v, dyn_of(c), c.pk, c.variant == MDG_SLAB ? 1 : 0, c.pred_parts);
}

void correct_launch(Ctx& c, bool merge) {
    const View& v = c.v;
    Dyn D = dyn_of(c);
    const int nu = D.nion + v.nrig + (merge ? v.nmove - v.nliqa : 0), lanes = lanes_of(nu);
    const int slab = c.variant == MDG_SLAB ? 1 : 0;
    const MergeArgs A = merge ? merge_args(c, c.d_frc) : MergeArgs{};
    constexpr int kCT = CorrBlock<32>::kThreads;
    if (lanes <= 16) {
        if (merge) k_corr<32, true, true><<<nblk(nu, 32), kCT, 0, c.stream>>>(v, D, slab, lanes, A);
        else k_corr<32, false, true><<<nblk(nu, 32), kCT, 0, c.stream>>>(v, D, slab, lanes, A);
    } else if (lanes < 32) {
        if (merge) k_corr<32, true, false><<<nblk(nu, 32), kCT, 0, c.stream>>>(v, D, slab, lanes, A);
        else k_corr<32, false, false><<<nblk(nu, 32), kCT, 0, c.stream>>>(v, D, slab, lanes, A);
    } else {
        if (merge) k_corr<128, true, false><<<nblk(nu, 128), 128, 0, c.stream>>>(v, D, slab, lanes, A);
        else k_corr<128, false, false><<<nblk(nu, 128), 128, 0, c.stream>>>(v, D, slab, lanes, A);
    }
}

}  // namespace mdg
