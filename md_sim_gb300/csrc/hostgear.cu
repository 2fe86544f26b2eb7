// hostgear.cu - the reference's Gear predictor-corrector on host arrays, for drop-in callers.
//
// In the reference, move_predict (src/move.f90:48-217) and move_correct (src/move.f90:220-383)
// stay in Fortran around the force call: a drop-in caller of mdg_force_get keeps them on the host
// and the library only replaces force_get / nnlist_make / move_shake.  This file is that host
// integrator for callers written in C or C++ (and the stand-in for the Fortran one when the
// end-to-end cost of a drop-in MD step is measured): rigid waters (centre, quaternion and body
// angular velocity, 5-value Gear with the reference's coefficients, Q11) and flexible atoms
// nriga+1..nliqa, with the Nose-type thermostat of src/move.f90:168-217,356-375.  Surface atoms
// (nliqa+1..nmove) move in mdg_shake, as in the reference (src/move.f90:376).
//
// The reference's loops over the molecules, split into contiguous ranges of molecules over the host
// threads (OpenMP; MDG_HOST_THREADS if set, else all cores the process may run on, one thread
// below 2,048 molecules): each thread runs every loop on its own range, so a molecule's arrays stay in
// one core's cache from one loop to the next.  The kinetic sums are seven independent chains, each
// summed in molecule order by one thread (several chains at once), so the result does not depend
// on the thread count.  No device memory.
// The arithmetic is the reference's operation by operation (this file is compiled without
// multiply-add contraction), so a drop-in loop reproduces the library's resident steps to rounding.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <new>
#include <vector>

#include <omp.h>

#include "../../include/mdgpu.h"

struct mdg_host_gear {
    int64_t nrig = 0, nriga = 0, nliqa = 0;
    std::vector<double> mi, mii;  // masses and inverse masses of the flexible atoms nriga..nliqa-1
    mdg_rigid body{};
    double kp = 0, kw = 0, ke = 0, htot = 0, sft = 0, sfr = 0, uconf = 0;
    int nthreads = 1;
};

namespace {

// single-precision literals of the reference (Q1, src/move.f90:224-225)
inline double F(float x) { return (double)x; }
const double kG01 = F(0.348611111f), kG21 = F(0.916666667f), kG31 = F(0.333333333f), kG41 = F(0.041666667f);
const double kG02 = F(0.158300000f), kG12 = F(0.757000000f), kG42 = F(0.083333333f);
const double kR = F(8.31441f);  // PH_R, src/global.f90:21

// 5-value Gear predictor of one coordinate (src/move.f90:56-66)
inline void predict4(double& a0, double& a1, double& a2, double& a3, double a4) {
    a0 = a0 + a1 + a2 + a3 + a4;
    a1 = a1 + 2 * a2 + 3 * a3 + 4 * a4;
    a2 = a2 + 3 * a3 + 6 * a4;
    a3 = a3 + 4 * a4;
}

inline void correct5(double& a0, double& a1, double& a2, double& a3, double& a4, double c, double g0, double g1,
                     double g2, double g3, double g4) {
    a0 = a0 + g0 * c;
    a1 = a1 + g1 * c;
    a2 = a2 + g2 * c;
    a3 = a3 + g3 * c;
    a4 = a4 + g4 * c;
}

// normalised quaternion and its rotation matrix (src/move.f90:120-136)
inline void quat_rot(const double* qq, double* qn, double* a) {
    const double cr = 1.0 / std::sqrt(qq[0] * qq[0] + qq[1] * qq[1] + qq[2] * qq[2] + qq[3] * qq[3]);
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

// rotation matrix of an already normalised quaternion: the same products as quat_rot's
inline void rot_of(double q1, double q2, double q3, double q4, double* a) {
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

// [lo, hi) of thread k of nt over n items
inline void split_range(int64_t n, int k, int nt, int64_t& lo, int64_t& hi) {
    lo = n * k / nt;
    hi = n * (k + 1) / nt;
}

int host_threads(int64_t nmol) {
    int nt = nmol < 2048 ? 1 : omp_get_num_procs();
    if (const char* e = std::getenv("MDG_HOST_THREADS")) nt = std::atoi(e);
    return std::max(1, std::min(nt, 64));
}

}  // namespace

extern "C" {

int mdg_host_gear_create(const mdg_sysdesc* s, const mdg_rigid* body, mdg_host_gear** out) {
    if (!s || !body || !out) return MDG_E_ARG;
    if (s->nrig < 0 || s->nriga != 3 * s->nrig || s->nliqa < s->nriga || s->nmove < s->nliqa || !s->mi || !s->mii)
        return MDG_E_ARG;
    mdg_host_gear* g = new (std::nothrow) mdg_host_gear();
    if (!g) return MDG_E_ARG;
    g->nrig = s->nrig;
    g->nriga = s->nriga;
    g->nliqa = s->nliqa;
    g->mi.assign(s->mi + s->nriga, s->mi + s->nliqa);
    g->mii.assign(s->mii + s->nriga, s->mii + s->nliqa);
    g->body = *body;
    g->nthreads = host_threads(std::max(s->nrig, s->nliqa - s->nriga));
    *out = g;
    return MDG_OK;
}

void mdg_host_gear_destroy(mdg_host_gear* g) { delete g; }

// move_predict (src/move.f90:48-217) on the caller's state: predicted flexible atoms, centres,
// angular velocities and quaternions (normalised), rotation matrices, site positions and the
// offsets rsx(ix+2:ix+3) of the water H sites (src/move.f90:148-162; rsx(ix+1) is left alone, Q3),
// the thermostat predictor, kp / kw / ke / htot and the thermostat forces sft / sfr.  htot uses
// the uconf of the previous mdg_host_correct (0 before the first).
int mdg_host_predict(mdg_host_gear* g, mdg_state* st) {
    if (!g || !st) return MDG_E_ARG;
    const int64_t nrig = g->nrig, n0 = g->nriga, n1 = g->nliqa;
    const mdg_rigid& b = g->body;
    // kinetic sums: seven independent chains (flexible atoms; centre velocity x, y, z; angular
    // velocity x, y, z), each summed in molecule order by one thread as the reference does, so the
    // result does not depend on the thread count; several threads run different chains at once
    double chain[7] = {0, 0, 0, 0, 0, 0, 0};
    auto run_chain = [&](int ch) {
        double s = 0.0;
        if (ch == 0) {
            for (int64_t i = n0; i < n1; ++i)
                s += g->mi[i - n0] * (st->xd[0][i] * st->xd[0][i] + st->yd[0][i] * st->yd[0][i] + st->zd[0][i] * st->zd[0][i]);
        } else {
            const double* a = ch == 1 ? st->cx[1] : ch == 2 ? st->cy[1] : ch == 3 ? st->cz[1]
                            : ch == 4 ? st->wx[0] : ch == 5 ? st->wy[0] : st->wz[0];
            for (int64_t i = 0; i < nrig; ++i) s += a[i] * a[i];
        }
        chain[ch] = s;
    };
#pragma omp parallel num_threads(g->nthreads) if (g->nthreads > 1)
    {
        const int nt = omp_get_num_threads(), k = omp_get_thread_num();
        int64_t lo, hi;
        split_range(n1 - n0, k, nt, lo, hi);
        for (int64_t i = n0 + lo; i < n0 + hi; ++i) {
            predict4(st->x0[i], st->xd[0][i], st->xd[1][i], st->xd[2][i], st->xd[3][i]);
            predict4(st->y0[i], st->yd[0][i], st->yd[1][i], st->yd[2][i], st->yd[3][i]);
            predict4(st->z0[i], st->zd[0][i], st->zd[1][i], st->zd[2][i], st->zd[3][i]);
        }
        // one loop per quantity, in the reference's order (src/move.f90:72-136), each over this
        // thread's molecules
        split_range(nrig, k, nt, lo, hi);
        double* const* c3[3] = {st->cx, st->cy, st->cz};
        for (int d = 0; d < 3; ++d) {
            double* const* a = c3[d];
            for (int64_t i = lo; i < hi; ++i) predict4(a[0][i], a[1][i], a[2][i], a[3][i], a[4][i]);
        }
        double* const* w3[3] = {st->wx, st->wy, st->wz};
        for (int d = 0; d < 3; ++d) {
            double* const* a = w3[d];
            for (int64_t i = lo; i < hi; ++i) predict4(a[0][i], a[1][i], a[2][i], a[3][i], a[4][i]);
        }
        for (int c = 0; c < 4; ++c) {
            double* const* a = st->q[c];
            for (int64_t i = lo; i < hi; ++i) predict4(a[0][i], a[1][i], a[2][i], a[3][i], a[4][i]);
        }
        // normalised quaternion, rotation matrix (in registers; the corrector rebuilds it from the
        // same quaternion), sites from the centre and the body frame, H offsets from the O
        // (src/move.f90:120-162)
        double *Q1 = st->q[0][0], *Q2 = st->q[1][0], *Q3 = st->q[2][0], *Q4 = st->q[3][0];
        const double *CX = st->cx[0], *CY = st->cy[0], *CZ = st->cz[0];
        for (int64_t i = lo; i < hi; ++i) {
            double qn[4], r[9];
            const double qq[4] = {Q1[i], Q2[i], Q3[i], Q4[i]};
            quat_rot(qq, qn, r);
            Q1[i] = qn[0];
            Q2[i] = qn[1];
            Q3[i] = qn[2];
            Q4[i] = qn[3];
            const int64_t ix = 3 * i;
            double sx[3], sy[3], sz[3];
            for (int j = 0; j < 3; ++j) {
                sx[j] = CX[i] + r[0] * b.xbody[j] + r[3] * b.ybody[j] + r[6] * b.zbody[j];
                sy[j] = CY[i] + r[1] * b.xbody[j] + r[4] * b.ybody[j] + r[7] * b.zbody[j];
                sz[j] = CZ[i] + r[2] * b.xbody[j] + r[5] * b.ybody[j] + r[8] * b.zbody[j];
                st->x0[ix + j] = sx[j];
                st->y0[ix + j] = sy[j];
                st->z0[ix + j] = sz[j];
            }
            for (int j = 1; j < 3; ++j) {
                st->rsx[ix + j] = sx[j] - sx[0];
                st->rsy[ix + j] = sy[j] - sy[0];
                st->rsz[ix + j] = sz[j] - sz[0];
            }
        }
#pragma omp barrier
        for (int ch = k; ch < 7; ch += nt) run_chain(ch);
    }
    double kp = chain[0];
    const double sc[3] = {chain[1], chain[2], chain[3]}, sw[3] = {chain[4], chain[5], chain[6]};
    kp = kp + b.mw * (sc[0] + sc[1] + sc[2]);
    const double kw = b.inxx * sw[0] + b.inyy * sw[1] + b.inzz * sw[2];
    if (b.temper == -1.0) {
        st->s[0] = st->s[1] = st->rs[0] = st->rs[1] = 0.0;
    } else {
        predict4(st->s[0], st->s[1], st->s[2], st->s[3], st->s[4]);
        predict4(st->rs[0], st->rs[1], st->rs[2], st->rs[3], st->rs[4]);
    }
    g->kp = kp;
    g->kw = kw;
    g->ke = kp + kw;
    // thermostat masses and forces (src/move.f90:173-217)
    const int64_t nfree = g->nliqa - g->nriga;
    const double ts = kR * b.temper / 1000.0;
    const double qmass = (double)(float)(3 * (nfree + nrig)) * ts * F(2e3f) / 10.0;
    const double rmass = (double)(float)(3 * nrig) * ts * F(1e3f) / 10.0;
    g->htot = 0.5 * (g->ke + qmass * st->s[0] * st->s[0] + rmass * st->rs[0] * st->rs[0]) + g->uconf;
    g->sft = (kp - (double)(float)(3 * (nfree + nrig) - 2) * ts) / qmass;
    g->sfr = (kw - (double)(float)(3 * nrig + 1) * ts) / rmass;
    return MDG_OK;
}

// move_correct (src/move.f90:220-383) with the outputs of mdg_force_get for the positions of the
// preceding mdg_host_predict: ftx.. (nmove - nriga, flexible atoms first), fcx.. and tx.. (nrig).
// uconf is the configurational energy of that force call (kept for the next htot).
int mdg_host_correct(mdg_host_gear* g, mdg_state* st, const double* ftx, const double* fty, const double* ftz,
                     const double* fcx, const double* fcy, const double* fcz, const double* tx, const double* ty,
                     const double* tz, double uconf) {
    if (!g || !st) return MDG_E_ARG;
    const int64_t nrig = g->nrig, n0 = g->nriga, n1 = g->nliqa;
    const mdg_rigid& b = g->body;
    const double s0i = st->s[0], rs0i = st->rs[0];
    if (n1 > n0 && (!ftx || !fty || !ftz)) return MDG_E_ARG;
    if (nrig > 0 && (!fcx || !fcy || !fcz || !tx || !ty || !tz)) return MDG_E_ARG;
    const double rc = 0.5 / b.mw;
    const double inxxi = 1.0 / b.inxx, inyyi = 1.0 / b.inyy, inzzi = 1.0 / b.inzz;
#pragma omp parallel num_threads(g->nthreads) if (g->nthreads > 1)
    {
        const int nt = omp_get_num_threads(), k = omp_get_thread_num();
        int64_t lo, hi;
        split_range(n1 - n0, k, nt, lo, hi);
        for (int64_t i = n0 + lo; i < n0 + hi; ++i) {
            const double mii = g->mii[i - n0];
            const double* f[3] = {ftx, fty, ftz};
            double* x[3] = {st->x0, st->y0, st->z0};
            double* const* xd[3] = {st->xd, st->yd, st->zd};
            for (int d = 0; d < 3; ++d) {
                const double c = 0.5 * f[d][i - n0] * mii - xd[d][0][i] * s0i - xd[d][1][i];
                x[d][i] = x[d][i] + kG02 * c;
                xd[d][0][i] = xd[d][0][i] + kG12 * c;
                xd[d][1][i] = xd[d][1][i] + c;
                xd[d][2][i] = xd[d][2][i] + 0.5 * c;
                xd[d][3][i] = xd[d][3][i] + kG42 * c;
            }
        }
        split_range(nrig, k, nt, lo, hi);
        // centre (src/move.f90:262-281)
        {
            const double* f3[3] = {fcx, fcy, fcz};
            double* const* cm[3] = {st->cx, st->cy, st->cz};
            for (int d = 0; d < 3; ++d) {
                double* const* a = cm[d];
                const double* f = f3[d];
                for (int64_t i = lo; i < hi; ++i) {
                    const double c = rc * f[i] - a[1][i] * s0i - a[2][i];
                    correct5(a[0][i], a[1][i], a[2][i], a[3][i], a[4][i], c, kG02, kG12, 1.0, 0.5, kG42);
                }
            }
        }
        // per molecule: the quaternion corrector from the angular velocity before its correction
        // (src/move.f90:283-317), then the body angular velocity by Euler's equations with the lab
        // torque rotated into the body frame by the matrix of the predicted quaternion
        // (src/move.f90:319-354); both read their inputs before either writes
        for (int64_t i = lo; i < hi; ++i) {
            const double q1 = st->q[0][0][i], q2 = st->q[1][0][i], q3 = st->q[2][0][i], q4 = st->q[3][0][i];
            const double wx = st->wx[0][i], wy = st->wy[0][i], wz = st->wz[0][i];
            double a[9];
            rot_of(q1, q2, q3, q4, a);
            const double cq[4] = {0.5 * (-q3 * wx - q4 * wy + q2 * wz), 0.5 * (q4 * wx - q3 * wy - q1 * wz),
                                  0.5 * (q1 * wx + q2 * wy + q4 * wz), 0.5 * (-q2 * wx + q1 * wy - q3 * wz)};
            for (int c = 0; c < 4; ++c) {
                double* const* qa = st->q[c];
                const double co = cq[c] - qa[1][i];
                correct5(qa[0][i], qa[1][i], qa[2][i], qa[3][i], qa[4][i], co, kG01, 1.0, kG21, kG31, kG41);
            }
            const double t0 = tx[i], t1 = ty[i], t2 = tz[i];
            double c1 = a[0] * t0 + a[1] * t1 + a[2] * t2;
            c1 = ((c1 + wy * wz * (b.inyy - b.inzz)) * inxxi) - st->wx[1][i] - rs0i * wx;
            double c2 = a[3] * t0 + a[4] * t1 + a[5] * t2;
            c2 = ((c2 + wz * wx * (b.inzz - b.inxx)) * inyyi) - st->wy[1][i] - rs0i * wy;
            double c3 = a[6] * t0 + a[7] * t1 + a[8] * t2;
            c3 = ((c3 + wx * wy * (b.inxx - b.inyy)) * inzzi) - st->wz[1][i] - rs0i * wz;
            correct5(st->wx[0][i], st->wx[1][i], st->wx[2][i], st->wx[3][i], st->wx[4][i], c1, kG01, 1.0, kG21, kG31,
                     kG41);
            correct5(st->wy[0][i], st->wy[1][i], st->wy[2][i], st->wy[3][i], st->wy[4][i], c2, kG01, 1.0, kG21, kG31,
                     kG41);
            correct5(st->wz[0][i], st->wz[1][i], st->wz[2][i], st->wz[3][i], st->wz[4][i], c3, kG01, 1.0, kG21, kG31,
                     kG41);
        }
    }
    if (b.temper != -1.0) {  // thermostat corrector (src/move.f90:356-375)
        double c = g->sft - st->s[1];
        st->s[0] = st->s[0] + kG01 * c;
        st->s[1] = g->sft;
        st->s[2] = st->s[2] + kG21 * c;
        st->s[3] = st->s[3] + kG31 * c;
        st->s[4] = st->s[4] + kG41 * c;
        c = g->sfr - st->rs[1];
        st->rs[0] = st->rs[0] + kG01 * c;
        st->rs[1] = g->sfr;
        st->rs[2] = st->rs[2] + kG21 * c;
        st->rs[3] = st->rs[3] + kG31 * c;
        st->rs[4] = st->rs[4] + kG41 * c;
    }
    g->uconf = uconf;
    return MDG_OK;
}

// The scalars the reference prints after a step (src/main.f90:320-335): kp, kw, ke and htot of
// the last mdg_host_predict, tempnow, and the uconf of the last mdg_host_correct.
int mdg_host_report(const mdg_host_gear* g, mdg_report* rep) {
    if (!g || !rep) return MDG_E_ARG;
    rep->kp = g->kp;
    rep->kw = g->kw;
    rep->ke = g->ke;
    rep->htot = g->htot;
    const int64_t nfree = g->nliqa - g->nriga;
    rep->tempnow = g->ke * 1000.0 / (3.0 * kR * (double)(float)(nfree + 2 * g->nrig));
    rep->uconf = g->uconf;
    return MDG_OK;
}

}  // extern "C"
