// mdref.cpp - CPU restatement of md_sim's force / neighbour-list / SHAKE / Gear path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA library is checked against and
// the CPU baseline that bench.py times.  It is never linked into, loaded by or called from the
// product library (md_sim_gb300/csrc).
//
// Parity status: the reference (Fortran 90 + MPI) cannot be compiled in this environment (no
// Fortran compiler) and ships no tests, golden vectors or known answers for this path, so this
// restatement is "parity unpinned" against the reference's own outputs.  It is validated by
// independent checks instead (the NaCl Madelung constant from its Ewald sum, finite-difference
// forces, independence of the total from the Ewald split, Newton's third law, translation
// invariance; tests/test_oracle_physics.py).
//
// Each routine follows the reference loop by loop, in the same order, so that sums match to
// rounding.  References are to files under src/ of the reference tree:
//   global.f90:18-24           constants (single-precision literals promoted to real*8)
//   forcem.f90:11-13           Abramowitz-Stegun 7.1.26 erfc coefficients
//   forcem.f90:54-81           force_init
//   forcem.f90:157-231         force_real_init (wall long-range tail tables)
//   forcem.f90:233-552         force_real
//   forcem.f90:565-652         force_intra
//   forcem.f90:657-825         force_fouri_init
//   forcem.f90:827-937         force_fouri
//   forcem_3d.f90:1031-1058    serial force_sum
//   forcem_back.f90:297,410,489-522,561,568,903-907   bulk variant
//   nnlist.f90:14-208          nnlist_init / nnlist_make / nnlist_constr
//   move.f90:48-529            move_predict / move_correct / move_shake(_init)
//
// Built with -ffp-contract=off so that no multiply-add is fused (the reference targets x86-64
// without FMA); with -fopenmp the pair, k-vector and atom loops are split over threads the way
// the reference splits them over MPI ranks, each thread summing into private buffers that are
// reduced at the end (the mpi_allreduce of force_sum).

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/mdgpu.h"

namespace {

typedef std::complex<double> cplx;

inline double F(float x) { return (double)x; }  // single-precision literal in real*8 context

const double M_PI_R = F(3.1415926535898f);
const double PH_e = F(1.6021892e-19f);
const double PH_Na = F(6.022045e23f);
const double PH_R = F(8.31441f);
const double PH_eps0 = F(8.85418782e-12f);
const double PH_4epi = F(8.987551784952e+9f);
const double PH_A2m = F(1.0e-10f);
const double A1 = F(0.254829592f), A2 = F(-0.284496736f), A3 = F(1.421413741f);
const double A4 = F(-1.453152027f), A5 = F(1.061405429f), PP = F(0.3275911f);

inline double anint(double x) { return std::round(x); }  // Fortran ANINT: half away from zero
inline double fsign(double z) { return std::signbit(z) ? -1.0 : 1.0; }
inline double pw3(double x) { return x * x * x; }
// Fortran MODULO(a, p) for reals as gfortran evaluates it: the exact remainder fmod(a, p), moved
// into p's sign range when it is non-zero and of the other sign.
inline double fmodulo(double a, double p) {
    double m = std::fmod(a, p);
    if (m != 0.0 && ((m < 0.0) != (p < 0.0))) m += p;
    return m;
}

// Measurement arrays of src/measure.f90:12-22 (column-major, bins from 0).
struct Meas {
    bool init = false, force_hist = false, profiles = false, l2d = false;
    double rdeli = 0, rfrst = 0, rscnd = 0;
    int64_t lmax = 0, ntz = 0, langmax = 201, lgxmax = 0, lgymax = 0;
    std::vector<int64_t> ngc, nefipos, ngang, ngz, ng2d1, ng2d2;
    std::vector<double> efipos, tefipos, ndipx, ndipy, ndipz, ndipsq;
    double ftot[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double fws[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // wall forces of the last evaluation
    int64_t calls_force = 0, calls_do = 0, oor = 0;
};

struct Ref {
    // sizes
    int64_t ntype, nrig, nriga, nliqa, nsurf, nmove, nwall, ntota, ngogo, nit, nijt, nltype;
    int64_t ncons, nang;
    std::vector<int64_t> moltypen, nt, ns, nst, nconst, nangt, nsi, ijtype, vdwnum, itype;
    std::vector<int64_t> ictype, constra, constrb, iatype, ang1, ang2, ang3;
    std::vector<int64_t> nss_wall;
    std::vector<double> eps, sig, aa, rhoi, cc, qs, mi, mii, length, kt, theta;
    double lx, ly, lz, lxi, lyi, lzi, cx, cy, cz, lw, lwh, dt;
    // params
    double rcut, rcutsq, skin, alfa, spii, facq, dshsq;
    int variant, pbcz;
    uint32_t quirks;
    int maxit;
    double tol2, rptol;
    // wall positions (frozen), full position copies for create-time work
    std::vector<double> wx, wy, wz;
    // neighbour lists
    double rskinsq;
    std::vector<int64_t> list1, list2, listw1, listw2;  // 0-based
    std::vector<double> ocx0, ocy0, ocz0, ox0, oy0, oz0;
    std::vector<std::vector<int64_t>> excl;  // constrained partners of surface atoms
    // reciprocal
    Meas ms;
    // state of the last force evaluation that chempot reads (module arrays x0, rsx, Qsum)
    std::vector<double> wx0, wy0, wz0, wrsx, wrsy, wrsz;
    std::vector<cplx> wqsum;
    double wdipz = 0.0;
    int64_t kmax, klmax, kmmax, knmax;
    double pipix, pipiy, pipiz;
    std::vector<int> kl_, km_, kn_;  // valid k in reference order
    std::vector<double> Ak;
    std::vector<cplx> Qsumw;  // Qsumw1 + Qsumw2
    std::vector<cplx> Qsumw1, Qsumw2;
    double ewqWW, uself;
    // long-range tail
    std::vector<double> flr_l, flr_w, flr_lja, flr_ljc, flr_bua, flr_buc, flr_bur, ulr_l, ulr_w;
    // SHAKE
    int64_t nfreed;
    std::string err;
    // resident-mode integrator state (src/config.f90:20-51)
    bool have_state = false;
    std::vector<double> X[3], XD[4][3], C[5][3], Q[4][5], W[5][3], OLD[3], RS[3], A[9];
    double s[5], rs[5];
    mdg_rigid body;
    double kp = 0, kw = 0, ke = 0, htot = 0, sft = 0, sfr = 0, tempnow = 0, uconf = 0, tkps = 0, press = 0;
    int32_t last_sweeps = 0;

    // l = int((z + lwh)*rdeli + 0.5) and l = int(r*rdeli + 0.5) (src/forcem.f90:348,493)
    int64_t zbin(double z) const { return (int64_t)((z + lwh) * ms.rdeli + 0.5); }
    int64_t rbin(double d) const { return (int64_t)(d * ms.rdeli + 0.5); }
    int ij(int64_t it, int64_t jt) const { return (int)ijtype[(it - 1) + nit * (jt - 1)] - 1; }
    double mx(double d) const { return d - lx * anint(d * lxi); }
    double my(double d) const { return d - ly * anint(d * lyi); }
    double mz_real(double d) const { return variant == MDG_BULK ? d - lz * anint(d * lzi) : d; }
    double mz_list(double d) const { return pbcz ? d - lz * anint(d * lzi) : d; }
    bool constrained(int64_t i, int64_t j) const {  // nnlist_constr (0-based atoms)
        if (i < 0 || i >= (int64_t)excl.size()) return false;
        for (int64_t p : excl[i])
            if (p == j) return true;
        return false;
    }
};

// Thread-private efipos / ngc contributions of one force loop, added to the context's arrays
// under the loop's merge lock.
struct Hist {
    Ref* r;
    bool on;
    std::vector<double> efi;
    std::vector<int64_t> ngc;
    int64_t oor = 0;
    Hist(Ref* r_, bool on_) : r(r_), on(on_) {
        if (on) {
            efi.assign(2 * (r->ms.lmax + 1), 0.0);
            ngc.assign(r->nijt * (r->ms.lmax + 1), 0);
        }
    }
    void ef(int64_t t, int64_t l, double v) {
        if (t >= 0 && t < 2 && l >= 0 && l <= r->ms.lmax) efi[t + 2 * l] += v;
        else ++oor;
    }
    void gc(int64_t ijt0, int64_t l) {
        if (l >= 0 && l <= r->ms.lmax) ++ngc[ijt0 + r->nijt * l];
        else ++oor;
    }
    void merge() {
        if (!on) return;
        for (size_t k = 0; k < efi.size(); ++k) r->ms.efipos[k] += efi[k];
        for (size_t k = 0; k < ngc.size(); ++k) r->ms.ngc[k] += ngc[k];
        r->ms.oor += oor;
    }
};

std::string g_err;

int fail(Ref* r, int code, const std::string& msg) {
    if (r) r->err = msg;
    g_err = msg;
    return code;
}

// ------------------------------------------------------------------------------------------
// nnlist_init (src/nnlist.f90:14-90) and nnlist_make (:92-165).  The candidate arrays
// list3/list4 and listw3/listw4 are enumerated on the fly in the same i-major, j-ascending
// order instead of being stored (they would need O(heads^2) memory).
// ------------------------------------------------------------------------------------------
void nnlist_make(Ref* r, const double* x0, const double* y0, const double* z0, const double* cx0,
                 const double* cy0, const double* cz0) {
    for (int64_t i = 0; i < r->nrig; ++i) {
        r->ocx0[i] = cx0[i];
        r->ocy0[i] = cy0[i];
        r->ocz0[i] = cz0[i];
    }
    for (int64_t i = r->nriga; i < r->nmove; ++i) {
        r->ox0[i - r->nriga] = x0[i];
        r->oy0[i - r->nriga] = y0[i];
        r->oz0[i - r->nriga] = z0[i];
    }
    r->list1.clear();
    r->list2.clear();
    const int64_t nmove = r->nmove, nliqa = r->nliqa;
    for (int64_t i = 0; i < nmove - 1; ++i) {
        if (r->nsi[r->itype[i] - 1] == 0) continue;
        for (int64_t j = i + 1; j < nmove; ++j) {
            if (r->nsi[r->itype[j] - 1] == 0) continue;
            if (i >= nliqa && j >= nliqa && r->constrained(i, j)) continue;
            double xijs = r->mx(x0[i] - x0[j]);
            double yijs = r->my(y0[i] - y0[j]);
            double zijs = r->mz_list(z0[i] - z0[j]);
            if (xijs * xijs + yijs * yijs + zijs * zijs < r->rskinsq) {
                r->list1.push_back(i);
                r->list2.push_back(j);
            }
        }
    }
    r->listw1.clear();
    r->listw2.clear();
    for (int64_t i = 0; i < nmove; ++i) {
        if (r->nsi[r->itype[i] - 1] == 0) continue;
        for (int64_t j = nmove; j < r->ntota; ++j) {
            if (i >= nliqa && r->constrained(i, j)) continue;
            const int64_t w = j - nmove;
            double xijs = r->mx(x0[i] - r->wx[w]);
            double yijs = r->my(y0[i] - r->wy[w]);
            double zijs = r->mz_list(z0[i] - r->wz[w]);
            if (xijs * xijs + yijs * yijs + zijs * zijs < r->rskinsq) {
                r->listw1.push_back(i);
                r->listw2.push_back(j);
            }
        }
    }
}

// ------------------------------------------------------------------------------------------
// force_real_init long-range tables (src/forcem.f90:167-228)
// ------------------------------------------------------------------------------------------
void lr_init(Ref* r) {
    const int64_t nit = r->nit;
    const int64_t nstw = r->nst[r->ntype - 1];
    r->flr_l.assign(nit, 0.0);
    r->flr_w.assign(nit, 0.0);
    r->flr_lja.assign(nit, 0.0);
    r->flr_ljc.assign(nit, 0.0);
    r->flr_bua.assign(nit, 0.0);
    r->flr_buc.assign(nit, 0.0);
    r->flr_bur.assign(nit, 1.0);
    r->ulr_l.assign(nit, 0.0);
    r->ulr_w.assign(nit, 0.0);
    if (r->variant != MDG_SLAB) return;
    const double rholiq = (double)r->nmove / (r->lx * r->ly * r->lw);
    int64_t nsswsum = 0;
    for (int64_t s = 0; s < nstw; ++s) nsswsum += r->nss_wall[s];
    const double rhowall = (double)nsswsum / (2.0 * r->cx * r->cy * r->cz);
    std::vector<double> xdens(nit, 0.0);
    for (int64_t i = 0; i < r->nmove; ++i) xdens[r->itype[i] - 1] += 1.0;
    for (int64_t t = 0; t < nit - nstw; ++t) xdens[t] = xdens[t] / (double)(float)r->nmove * rholiq;
    // real(nss)/real(sum(nss)) is a default-real (single precision) quotient
    const float nss12 = (float)(r->nss_wall[0] + r->nss_wall[1]);
    if (nit >= 2) {
        xdens[nit - 2] = (double)((float)r->nss_wall[0] / nss12) * rhowall;
        xdens[nit - 1] = (double)((float)r->nss_wall[1] / nss12) * rhowall;
    }
    const double rc = r->rcut;
    for (int64_t it = 1; it <= nit - nstw; ++it) {
        for (int64_t jt = 1; jt <= nit; ++jt) {
            const int k = r->ij(it, jt);
            double sgn = (jt <= nit - nstw) ? -1.0 : 1.0;
            double flr = 0.0, ul = 0.0;
            const double e = r->eps[k], s = r->sig[k];
            switch (r->vdwnum[k]) {
                case 0: break;
                case 1: {
                    double rc10 = std::pow(rc, 10), rc4 = std::pow(rc, 4), rc9 = std::pow(rc, 9),
                           rc3 = rc * rc * rc;
                    flr = e * s * (s / (10.0 * rc10) - 1.0 / (4.0 * rc4));
                    ul = e * s * (s / (90.0 * rc9) - 1.0 / (12.0 * rc3));
                    r->flr_lja[it - 1] += sgn * xdens[jt - 1] * e * (s * s) / 10.0;
                    r->flr_ljc[it - 1] += sgn * xdens[jt - 1] * e * s / 4.0;
                } break;
                case 2: {
                    double ro = 1.0 / r->rhoi[k];
                    double rc4 = std::pow(rc, 4), rc3 = rc * rc * rc;
                    flr = ro * (ro + rc) * r->aa[k] * std::exp(-rc / ro) - r->cc[k] / (4.0 * rc4);
                    ul = ro * ro * (2.0 * ro + rc) * r->aa[k] * std::exp(-rc / ro) -
                         r->cc[k] / (12.0 * rc3);
                    r->flr_bua[it - 1] += sgn * xdens[jt - 1] * r->aa[k] * ro;
                    r->flr_buc[it - 1] += sgn * xdens[jt - 1] * r->cc[k] / 4.0;
                    r->flr_bur[it - 1] = ro;
                } break;
                default: break;
            }
            if (sgn < 0.0) {
                r->flr_l[it - 1] += flr * xdens[jt - 1];
                r->ulr_l[it - 1] += ul * xdens[jt - 1];
            } else {
                r->flr_w[it - 1] += flr * xdens[jt - 1];
                r->ulr_w[it - 1] += ul * xdens[jt - 1];
            }
        }
    }
    const double tp = 2.0 * M_PI_R;
    for (int64_t t = 0; t < nit; ++t) {
        r->flr_lja[t] *= tp;
        r->flr_ljc[t] *= tp;
        r->flr_bua[t] *= tp;
        r->flr_buc[t] *= tp;
        r->flr_l[t] *= tp;
        r->flr_w[t] *= tp;
        r->ulr_l[t] *= tp;
        r->ulr_w[t] *= tp;
    }
}

// ------------------------------------------------------------------------------------------
// force_fouri_init (src/forcem.f90:657-825)
// ------------------------------------------------------------------------------------------
void fouri_init(Ref* r, const double* x0, const double* y0, const double* z0) {
    r->pipix = 2.0 * M_PI_R / r->lx;
    r->pipiy = 2.0 * M_PI_R / r->ly;
    r->pipiz = 2.0 * M_PI_R / r->lz;
    const double alf4i = -1.0 / (4.0 * r->alfa * r->alfa);
    const double fac = 2.0 * PH_e * PH_e * PH_Na / (PH_eps0 * PH_A2m * 1000.0 * r->lx * r->ly * r->lz);
    const double lmin = std::min(r->lx, std::min(r->ly, r->lz));
    const double rk = (double)(float)r->kmax;
    r->klmax = (int64_t)std::lround(rk * r->lx / lmin);
    r->kmmax = (int64_t)std::lround(rk * r->ly / lmin);
    r->knmax = (int64_t)std::lround(rk * r->lz / lmin);
    const int64_t nw = r->nwall, KL = r->klmax, KM = r->kmmax, KN = r->knmax;
    // wall phase factors by recurrence
    std::vector<cplx> el((size_t)nw * (KL + 1)), em((size_t)nw * (2 * KM + 1)), en((size_t)nw * (2 * KN + 1));
    auto EL = [&](int64_t i, int64_t l) -> cplx& { return el[i * (KL + 1) + l]; };
    auto EM = [&](int64_t i, int64_t m) -> cplx& { return em[i * (2 * KM + 1) + m + KM]; };
    auto EN = [&](int64_t i, int64_t n) -> cplx& { return en[i * (2 * KN + 1) + n + KN]; };
    for (int64_t i = 0; i < nw; ++i) {
        EL(i, 0) = EM(i, 0) = EN(i, 0) = cplx(1.0, 0.0);
        double tx = r->pipix * r->wx[i], ty = r->pipiy * r->wy[i], tz = r->pipiz * r->wz[i];
        EL(i, 1) = cplx(std::cos(tx), std::sin(tx));
        EM(i, 1) = cplx(std::cos(ty), std::sin(ty));
        EN(i, 1) = cplx(std::cos(tz), std::sin(tz));
        for (int64_t l = 2; l <= KL; ++l) EL(i, l) = EL(i, l - 1) * EL(i, 1);
        for (int64_t m = 2; m <= KM; ++m) EM(i, m) = EM(i, m - 1) * EM(i, 1);
        for (int64_t m = 1; m <= KM; ++m) EM(i, -m) = std::conj(EM(i, m));
        for (int64_t n = 2; n <= KN; ++n) EN(i, n) = EN(i, n - 1) * EN(i, 1);
        for (int64_t n = 1; n <= KN; ++n) EN(i, -n) = std::conj(EN(i, n));
    }
    // ranges of the two static walls (src/forcem.f90:690-701, ngogo = nmove)
    const int64_t h1a = 0, h1b = nw / 2, h2a = nw / 2, h2b = nw;
    r->kl_.clear();
    r->km_.clear();
    r->kn_.clear();
    r->Ak.clear();
    r->Qsumw.clear();
    r->Qsumw1.clear();
    r->Qsumw2.clear();
    r->ewqWW = 0.0;
    std::vector<cplx> elm(nw);
    int64_t kmmin = 0, knmin = 1;
    const float kmaxsq_lim = (float)(r->kmax * r->kmax) + 2.01f;
    for (int64_t kl = 0; kl <= KL; ++kl) {
        double rl = r->pipix * (double)(float)kl;
        for (int64_t km = kmmin; km <= KM; ++km) {
            double rm = r->pipiy * (double)(float)km;
            for (int64_t i = 0; i < nw; ++i) elm[i] = r->qs[r->nmove + i] * EL(i, kl) * EM(i, km);
            for (int64_t kn = knmin; kn <= KN; ++kn) {
                double rn = r->pipiz * (double)(float)kn;
                volatile float a = (float)(kl * kl + km * km);
                volatile float b = (float)(kn * kn * r->kmax * r->kmax) / (float)(KN * KN);
                volatile float ksq = a + b;
                if (ksq < kmaxsq_lim) {
                    double rksq = rl * rl + rm * rm + rn * rn;
                    r->kl_.push_back((int)kl);
                    r->km_.push_back((int)km);
                    r->kn_.push_back((int)kn);
                    r->Ak.push_back(fac * std::exp(rksq * alf4i) / rksq);
                    cplx q1(0.0, 0.0), q2(0.0, 0.0);
                    for (int64_t i = h1a; i < h1b; ++i) q1 += elm[i] * EN(i, kn);
                    for (int64_t i = h2a; i < h2b; ++i) q2 += elm[i] * EN(i, kn);
                    r->Qsumw1.push_back(q1);
                    r->Qsumw2.push_back(q2);
                    cplx qws = q1 + q2;
                    r->Qsumw.push_back(qws);
                    r->ewqWW += (r->Ak.back() * qws * std::conj(qws)).real();
                }
            }
            knmin = -KN;
        }
        kmmin = -KM;
    }
    r->ewqWW *= 0.5;

    // self energy (src/forcem.f90:793-822)
    double sq = 0.0;
    for (int64_t i = 0; i < r->ntota; ++i) sq += r->qs[i] * r->qs[i];
    r->uself = -0.5 * r->spii * r->facq * r->alfa * sq;
    int64_t ix = 0;
    int64_t ntprev = 0;
    for (int64_t it = 0; it < r->ntype; ++it) {
        if (r->moltypen[it] == 0) {
            const int64_t i0 = ntprev;  // nt(it-1) used as an atom offset, as the reference does
            for (int64_t is = i0; is < i0 + r->ns[it]; ++is)
                for (int64_t js = is + 1; js < i0 + r->ns[it]; ++js) {
                    double dx = x0[is] - x0[js], dy = y0[is] - y0[js], dz = z0[is] - z0[js];
                    double rij = std::sqrt(dx * dx + dy * dy + dz * dz);
                    double t = 1.0 / (1.0 + PP * r->alfa * rij);
                    double ar = r->alfa * rij;
                    double erfv = 1.0 - ((((A5 * t + A4) * t + A3) * t + A2) * t + A1) * t * std::exp(-(ar * ar));
                    r->uself -= (double)r->nt[it] * r->facq * r->qs[is] * r->qs[js] * erfv / rij;
                }
        } else if (r->moltypen[it] == 2) {
            for (int64_t iq = 0; iq < r->nt[it]; ++iq) {
                ++ix;
                for (int64_t is = 1; is <= r->nconst[it]; ++is) {
                    // constra(ix, is): the reference indexes the (SMX, ncons) table transposed
                    int64_t flat = (ix - 1) + MDG_SMX * (is - 1);
                    int64_t i = flat < (int64_t)r->constra.size() ? r->constra[flat] : 0;
                    int64_t j = flat < (int64_t)r->constrb.size() ? r->constrb[flat] : 0;
                    if (i <= 0 || j <= 0) continue;  // unset table entry: the reference reads qs(0)
                    double rij = r->length[it + r->ntype * (is - 1)];
                    double t = 1.0 / (1.0 + PP * r->alfa * rij);
                    double ar = r->alfa * rij;
                    double erfv = 1.0 - ((((A5 * t + A4) * t + A3) * t + A2) * t + A1) * t * std::exp(-(ar * ar));
                    r->uself -= r->facq * r->qs[i - 1] * r->qs[j - 1] * erfv / rij;
                }
            }
        }
        ntprev = r->nt[it];
    }
}

}  // namespace

struct RefCtx : Ref {};

extern "C" {

const char* ref_last_error(const RefCtx* c) { return c ? c->err.c_str() : g_err.c_str(); }

void ref_destroy(RefCtx* c) { delete c; }

int ref_create(const mdg_sysdesc* s, const mdg_params* p, const double* x0, const double* y0,
               const double* z0, const double* cx0, const double* cy0, const double* cz0,
               RefCtx** out) {
    if (!s || !p || !out) return fail(nullptr, MDG_E_ARG, "null argument");
    if (s->ngogo != s->nmove) return fail(nullptr, MDG_E_UNSUPPORTED, "ngogo /= nmove (pulled walls)");
    RefCtx* r = new RefCtx();
    r->ntype = s->ntype; r->nrig = s->nrig; r->nriga = s->nriga; r->nliqa = s->nliqa;
    r->nsurf = s->nsurf; r->nmove = s->nmove; r->nwall = s->nwall; r->ntota = s->ntota;
    r->ngogo = s->ngogo; r->nit = s->nit; r->nijt = s->nijt; r->nltype = s->nltype;
    r->ncons = s->ncons; r->nang = s->nang;
    auto cp = [](const int64_t* a, int64_t n) { return std::vector<int64_t>(a, a + n); };
    auto cpd = [](const double* a, int64_t n) { return std::vector<double>(a, a + n); };
    r->moltypen = cp(s->moltypen, s->ntype); r->nt = cp(s->nt, s->ntype); r->ns = cp(s->ns, s->ntype);
    r->nst = cp(s->nst, s->ntype); r->nconst = cp(s->nconst, s->ntype); r->nangt = cp(s->nangt, s->ntype);
    r->nss_wall = cp(s->nss_wall, std::max<int64_t>(2, s->nst[s->ntype - 1]));
    r->nsi = cp(s->nsi, s->nit); r->ijtype = cp(s->ijtype, s->nit * s->nit);
    r->vdwnum = cp(s->vdwnum, s->nijt);
    r->eps = cpd(s->eps, s->nijt); r->sig = cpd(s->sig, s->nijt); r->aa = cpd(s->aa, s->nijt);
    r->rhoi = cpd(s->rhoi, s->nijt); r->cc = cpd(s->cc, s->nijt);
    r->itype = cp(s->itype, s->ntota); r->qs = cpd(s->qs, s->ntota); r->mi = cpd(s->mi, s->ntota);
    r->mii = cpd(s->mii, s->ntota);
    if (s->ncons > 0) {
        r->ictype = cp(s->ictype, s->ncons);
        r->constra = cp(s->constra, MDG_SMX * s->ncons);
        r->constrb = cp(s->constrb, MDG_SMX * s->ncons);
    }
    if (s->nang > 0) {
        r->iatype = cp(s->iatype, s->nang);
        r->ang1 = cp(s->ang1, MDG_SMX * s->nang);
        r->ang2 = cp(s->ang2, MDG_SMX * s->nang);
        r->ang3 = cp(s->ang3, MDG_SMX * s->nang);
    }
    r->length = cpd(s->length, s->ntype * MDG_SMX);
    r->kt = cpd(s->kt, s->ntype * MDG_SMX);
    r->theta = cpd(s->theta, s->ntype * MDG_SMX);
    r->lx = s->lx; r->ly = s->ly; r->lz = s->lz;
    r->lxi = 1.0 / s->lx; r->lyi = 1.0 / s->ly; r->lzi = 1.0 / s->lz;
    r->cx = s->cx; r->cy = s->cy; r->cz = s->cz; r->lw = s->lw; r->lwh = 0.5 * s->lw; r->dt = s->dt;
    for (int64_t k = 0; k < r->nijt; ++k)
        if (r->vdwnum[k] < 0 || r->vdwnum[k] > 2) {
            delete r;
            return fail(nullptr, MDG_E_ARG, "force_real(): unknown interaction type");
        }

    // force_init (src/forcem.f90:58-60)
    r->rcut = p->rcut;
    r->rcutsq = p->rcut * p->rcut;
    r->skin = p->skin;
    r->spii = 2.0 / std::sqrt(M_PI_R);
    r->alfa = p->alpha > 0.0 ? p->alpha : F(3.09f) / p->rcut;
    r->facq = PH_4epi * PH_e * PH_e * PH_Na / (1000.0 * PH_A2m);
    r->dshsq = p->dshsq;
    r->variant = p->variant;
    r->pbcz = p->pbc_z_list;
    r->quirks = p->quirks;
    r->kmax = p->kmax;
    r->maxit = p->shake_maxit > 0 ? p->shake_maxit : 10;
    r->tol2 = p->shake_tol2 > 0.0 ? p->shake_tol2 : F(1.e-8f);
    r->rptol = p->shake_rptol > 0.0 ? p->shake_rptol : F(0.85f);

    r->wx.assign(x0 + r->nmove, x0 + r->ntota);
    r->wy.assign(y0 + r->nmove, y0 + r->ntota);
    r->wz.assign(z0 + r->nmove, z0 + r->ntota);

    // exclusion table for nnlist_constr (O(1) per test instead of a scan of all constraints)
    r->excl.assign(r->ntota, {});
    for (int64_t ic = 0; ic < r->ncons; ++ic) {
        const int64_t it = r->ictype[ic] - 1;
        for (int64_t is = 0; is < r->nconst[it]; ++is) {
            int64_t a = r->constra[is + MDG_SMX * ic] - 1, b = r->constrb[is + MDG_SMX * ic] - 1;
            if (a < 0 || b < 0 || a >= r->ntota || b >= r->ntota) {
                std::string m = "constraint atom out of range";
                delete r;
                return fail(nullptr, MDG_E_ARG, m);
            }
            r->excl[a].push_back(b);
            r->excl[b].push_back(a);
        }
    }

    fouri_init(r, x0, y0, z0);
    // nnlist_init (src/nnlist.f90:18-28)
    r->ocx0.assign(r->nrig, 0.0); r->ocy0.assign(r->nrig, 0.0); r->ocz0.assign(r->nrig, 0.0);
    r->ox0.assign(r->nmove - r->nriga, 0.0); r->oy0.assign(r->nmove - r->nriga, 0.0);
    r->oz0.assign(r->nmove - r->nriga, 0.0);
    double rs = r->rcut + r->skin;
    if (r->nrig > 0) {
        double dx = x0[0] - cx0[0], dy = y0[0] - cy0[0], dz = z0[0] - cz0[0];
        rs = rs + 2.0 * std::sqrt(dx * dx + dy * dy + dz * dz);
    }
    r->rskinsq = rs * rs;
    lr_init(r);
    nnlist_make(r, x0, y0, z0, cx0, cy0, cz0);
    // move_shake_init (src/move.f90:402)
    r->nfreed = 3 * (r->nmove - r->nliqa);
    for (int64_t it = r->nltype; it < r->ntype; ++it)
        if (r->moltypen[it] == 2) r->nfreed -= r->nt[it] * r->nconst[it];
    *out = r;
    return MDG_OK;
}

int ref_nnlist_make(RefCtx* r, const double* x0, const double* y0, const double* z0, const double* cx0,
                    const double* cy0, const double* cz0, int64_t* ipack, int64_t* wpack) {
    nnlist_make(r, x0, y0, z0, cx0, cy0, cz0);
    if (ipack) *ipack = (int64_t)r->list1.size();
    if (wpack) *wpack = (int64_t)r->listw1.size();
    return MDG_OK;
}

int ref_get_lists(RefCtx* r, int64_t* li, int64_t* lj, int64_t cap, int64_t* wi, int64_t* wj,
                  int64_t wcap, int64_t* ipack, int64_t* wpack) {
    int64_t n = (int64_t)r->list1.size(), nw = (int64_t)r->listw1.size();
    for (int64_t k = 0; k < n && k < cap && li; ++k) {
        li[k] = r->list1[k] + 1;
        lj[k] = r->list2[k] + 1;
    }
    for (int64_t k = 0; k < nw && k < wcap && wi; ++k) {
        wi[k] = r->listw1[k] + 1;
        wj[k] = r->listw2[k] + 1;
    }
    if (ipack) *ipack = n;
    if (wpack) *wpack = nw;
    return MDG_OK;
}

// k-vector table, for tests: kl/km/kn per valid k in reference order and Ak.
int64_t ref_kvectors(RefCtx* r, int32_t* kl, int32_t* km, int32_t* kn, double* ak, int64_t cap) {
    int64_t n = (int64_t)r->Ak.size();
    for (int64_t k = 0; k < n && k < cap; ++k) {
        if (kl) kl[k] = r->kl_[k];
        if (km) km[k] = r->km_[k];
        if (kn) kn[k] = r->kn_[k];
        if (ak) ak[k] = r->Ak[k];
    }
    return n;
}

double ref_uself(RefCtx* r) { return r->uself; }

int ref_force_get(RefCtx* r, const double* x0, const double* y0, const double* z0, const double* cx0,
                  const double* cy0, const double* cz0, double* rsx, double* rsy, double* rsz,
                  double* ftx, double* fty, double* ftz, double* fcx, double* fcy, double* fcz,
                  double* tx, double* ty, double* tz, double* fxo, double* fyo, double* fzo,
                  mdg_energies* e) {
    const int64_t nmove = r->nmove, nrig = r->nrig, nriga = r->nriga, nijt = r->nijt;
    std::vector<double> fx(nmove, 0.0), fy(nmove, 0.0), fz(nmove, 0.0);
    std::vector<double> elj(nijt, 0.0), eqq(nijt, 0.0);
    double fwsx[3] = {0, 0, 0}, fwsy[3] = {0, 0, 0}, fwsz[3] = {0, 0, 0};  // index sgn+1
    double uewa = 0.0, urf = 0.0, ulr = 0.0, uavex = 0.0;
    const bool hist = r->ms.init && r->ms.force_hist;

    // ---- force_real: rebuild trigger (src/forcem.f90:245-250)
    {
        double aux = r->dshsq;
        double m1 = -HUGE_VAL, m2 = -HUGE_VAL;
        for (int64_t i = 0; i < nrig; ++i) {
            double a = r->ocx0[i] - cx0[i], b = r->ocy0[i] - cy0[i], c = r->ocz0[i] - cz0[i];
            m1 = std::max(m1, a * a + b * b + c * c);
        }
        for (int64_t i = nriga; i < nmove; ++i) {
            double a = r->ox0[i - nriga] - x0[i], b = r->oy0[i - nriga] - y0[i], c = r->oz0[i - nriga] - z0[i];
            m2 = std::max(m2, a * a + b * b + c * c);
        }
        aux = std::max(std::max(m1, m2), aux);
        if (4.0 * aux > r->skin * r->skin) nnlist_make(r, x0, y0, z0, cx0, cy0, cz0);
    }
    const double alfa = r->alfa, facq = r->facq, spii = r->spii, rcutsq = r->rcutsq;
    const int64_t npair = (int64_t)r->list1.size();
    const int64_t nwpair = (int64_t)r->listw1.size();

#ifdef _OPENMP
#pragma omp parallel
#endif
    {
        std::vector<double> tfx(nmove, 0.0), tfy(nmove, 0.0), tfz(nmove, 0.0), telj(nijt, 0.0),
            teqq(nijt, 0.0);
        double tuav = 0.0;
        Hist th(r, hist);
        // ---- moving-moving pairs (src/forcem.f90:288-403)
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int64_t k = 0; k < npair; ++k) {
            const int64_t i = r->list1[k], j = r->list2[k];
            double xio = r->mx(x0[i] - x0[j]);
            double yio = r->my(y0[i] - y0[j]);
            double zio = r->mz_real(z0[i] - z0[j]);
            double rsq = xio * xio + yio * yio + zio * zio;
            if (rsq > rcutsq) continue;
            const int64_t it = r->itype[i], jt = r->itype[j];
            const int ijt = r->ij(it, jt);
            double rsqi = 1.0 / rsq;
            double rij = std::sqrt(rsq);
            double fij = 0.0, r6, aux;
            switch (r->vdwnum[ijt]) {
                case 1:
                    r6 = r->sig[ijt] * pw3(rsqi);
                    telj[ijt] += r->eps[ijt] * r6 * (r6 - 1.0);
                    tuav += r->eps[ijt] * r6 * (r6 - 1.0);
                    fij = 6.0 * rsqi * r->eps[ijt] * r6 * (2.0 * r6 - 1.0);
                    break;
                case 2:
                    r6 = r->cc[ijt] * pw3(rsqi);
                    aux = r->aa[ijt] * std::exp(-rij * r->rhoi[ijt]);
                    telj[ijt] += aux - r6;
                    tuav += aux - r6;
                    fij = aux * r->rhoi[ijt] / rij - 6.0 * rsqi * r6;
                    break;
                default: fij = 0.0;
            }
            aux = facq * r->qs[i] * r->qs[j] / rij;
            double alfar = alfa * rij;
            double t = 1.0 / (1.0 + PP * alfar);
            double exp2a = std::exp(-alfar * alfar);
            double erfx = ((((A5 * t + A4) * t + A3) * t + A2) * t + A1) * t * exp2a;
            teqq[ijt] += erfx * aux;
            tuav += erfx * aux;
            fij = fij + (spii * alfar * exp2a + erfx) * aux * rsqi;
            tfx[i] += xio * fij; tfy[i] += yio * fij; tfz[i] += zio * fij;
            tfx[j] -= xio * fij; tfy[j] -= yio * fij; tfz[j] -= zio * fij;
            if (hist) {
                if (r->variant == MDG_SLAB) {  // src/forcem.f90:347-354
                    if (it == 3 || it == 4) th.ef(it - 3, r->zbin(z0[i]), zio * fij);
                    if (jt == 3 || jt == 4) th.ef(jt - 3, r->zbin(z0[j]), -zio * fij);
                } else {                       // src/forcem_back.f90:348-349
                    th.gc(ijt, r->rbin(rij));
                }
            }
            int64_t jmin = j + 1;
            const int64_t nsi_i = r->nsi[it - 1], nsi_j = r->nsi[jt - 1];
            for (int64_t ix = i; ix < i + nsi_i; ++ix) {
                double xi = xio + rsx[ix], yi = yio + rsy[ix], zi = zio + rsz[ix];
                double qx = facq * r->qs[ix];
                for (int64_t jx = jmin; jx < j + nsi_j; ++jx) {
                    double xd = xi - rsx[jx], yd = yi - rsy[jx], zd = zi - rsz[jx];
                    double rs2 = xd * xd + yd * yd + zd * zd;
                    double rs2i = 1.0 / rs2;
                    double rr = std::sqrt(rs2);
                    double au = qx * r->qs[jx] / rr;
                    double ar = alfa * rr;
                    double tt = 1.0 / (1.0 + PP * ar);
                    double e2 = std::exp(-ar * ar);
                    double ef = ((((A5 * tt + A4) * tt + A3) * tt + A2) * tt + A1) * tt * e2;
                    teqq[ijt] += ef * au;
                    tuav += ef * au;
                    double fj = (spii * ar * e2 + ef) * au * rs2i;
                    tfx[ix] += xd * fj; tfy[ix] += yd * fj; tfz[ix] += zd * fj;
                    tfx[jx] -= xd * fj; tfy[jx] -= yd * fj; tfz[jx] -= zd * fj;
                    if (hist) {
                        if (r->variant == MDG_SLAB) {  // src/forcem.f90:388-395
                            if (it == 3 || it == 4) th.ef(it - 3, r->zbin(z0[i]), zd * fj);
                            if (jt == 3 || jt == 4) th.ef(jt - 3, r->zbin(z0[j]), -zd * fj);
                        } else {                       // src/forcem_back.f90:380-382
                            th.gc(r->ij(r->itype[ix], r->itype[jx]), r->rbin(rr));
                        }
                    }
                }
                jmin = j;
            }
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            for (int64_t i = 0; i < nmove; ++i) {
                fx[i] += tfx[i]; fy[i] += tfy[i]; fz[i] += tfz[i];
            }
            for (int64_t k = 0; k < nijt; ++k) {
                elj[k] += telj[k]; eqq[k] += teqq[k];
            }
            uavex += tuav;
            th.merge();
        }
    }

    // wall partition of the surface-atom z forces (src/forcem.f90:408-413)
    for (int64_t i = r->nliqa; i < nmove; ++i) fwsz[(int)fsign(z0[i]) + 1] += fz[i];

    // ---- moving-wall pairs (src/forcem.f90:418-498)
#ifdef _OPENMP
#pragma omp parallel
#endif
    {
        std::vector<double> tfx(nmove, 0.0), tfy(nmove, 0.0), tfz(nmove, 0.0), telj(nijt, 0.0),
            teqq(nijt, 0.0);
        double tuav = 0.0, tws[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        Hist th(r, hist);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int64_t k = 0; k < nwpair; ++k) {
            const int64_t i = r->listw1[k], j = r->listw2[k];
            const int64_t w = j - nmove;
            double xi = r->mx(x0[i] - r->wx[w]);
            double yi = r->my(y0[i] - r->wy[w]);
            double zi = r->mz_real(z0[i] - r->wz[w]);
            double rsq = xi * xi + yi * yi + zi * zi;
            if (rsq > rcutsq) continue;
            const int sg = (int)fsign(r->wz[w]) + 1;
            const int64_t it = r->itype[i];
            const int ijt = r->ij(it, r->itype[j]);
            double fij = 0.0, rsqi, rij, r6, aux;
            switch (r->vdwnum[ijt]) {
                case 1:
                    rsqi = 1.0 / rsq;
                    r6 = r->sig[ijt] * pw3(rsqi);
                    telj[ijt] += r->eps[ijt] * r6 * (r6 - 1.0);
                    tuav += r->eps[ijt] * r6 * (r6 - 1.0);
                    fij = 6.0 * rsqi * r->eps[ijt] * r6 * (2.0 * r6 - 1.0);
                    break;
                case 2:
                    rsqi = 1.0 / rsq;
                    rij = std::sqrt(rsq);
                    r6 = r->cc[ijt] * pw3(rsqi);
                    aux = r->aa[ijt] * std::exp(-rij * r->rhoi[ijt]);
                    telj[ijt] += aux - r6;
                    tuav += aux - r6;
                    fij = aux * r->rhoi[ijt] / rij - 6.0 * rsqi * r6;
                    break;
                default: fij = 0.0;
            }
            const double qx = facq * r->qs[j];
            for (int64_t ix = i; ix < i + r->nsi[it - 1]; ++ix) {
                double xd = xi + rsx[ix], yd = yi + rsy[ix], zd = zi + rsz[ix];
                double rs2 = xd * xd + yd * yd + zd * zd;
                double rr = std::sqrt(rs2);
                double rs2i = 1.0 / rs2;
                double au = qx * r->qs[ix] / rr;
                double ar = alfa * rr;
                double tt = 1.0 / (1.0 + PP * ar);
                double e2 = std::exp(-ar * ar);
                double ef = ((((A5 * tt + A4) * tt + A3) * tt + A2) * tt + A1) * tt * e2;
                teqq[ijt] += ef * au;
                tuav += ef * au;
                fij = fij + (spii * ar * e2 + ef) * au * rs2i;
                tfx[ix] += xd * fij; tfy[ix] += yd * fij; tfz[ix] += zd * fij;
                if (it <= r->nltype) {
                    tws[0][sg] -= xd * fij; tws[1][sg] -= yd * fij; tws[2][sg] -= zd * fij;
                }
                if (hist && r->variant == MDG_SLAB && (it == 3 || it == 4))  // src/forcem.f90:486-489
                    th.ef(it - 3, r->zbin(z0[i]), zd * fij);
                fij = 0.0;
                if (hist) th.gc(r->ij(r->itype[ix], r->itype[j]), r->rbin(rr));  // :493-495
            }
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            for (int64_t i = 0; i < nmove; ++i) {
                fx[i] += tfx[i]; fy[i] += tfy[i]; fz[i] += tfz[i];
            }
            for (int64_t k = 0; k < nijt; ++k) {
                elj[k] += telj[k]; eqq[k] += teqq[k];
            }
            uavex += tuav;
            for (int c = 0; c < 3; ++c) {
                fwsx[c] += tws[0][c]; fwsy[c] += tws[1][c]; fwsz[c] += tws[2][c];
            }
            th.merge();
        }
    }

    // ---- wall long-range tail (src/forcem.f90:509-543; absent in the bulk variant)
    if (r->variant == MDG_SLAB) {
        for (int64_t i = 0; i < nmove; ++i) {
            const int64_t it = r->itype[i];
            if (std::fabs(r->qs[i]) < F(0.7f)) continue;
            for (int j = -1; j <= 1; j += 2) {
                double aux = 0.0, sgn = (double)j;
                double dw = r->lwh - sgn * z0[i];
                const int64_t t0 = it - 1;
                if (dw < r->rcut) {
                    aux = aux + sgn * r->flr_w[t0];
                    ulr += r->ulr_w[t0];
                } else {
                    aux = aux + sgn * r->flr_l[t0];
                    ulr += r->ulr_l[t0];
                    double dwa = 1.0 / (dw * dw);
                    double dwa2 = dwa * dwa;
                    double dwa5 = dwa2 * dwa2 * dwa;
                    aux = aux + sgn * (r->flr_lja[t0] * dwa5 - r->flr_ljc[t0] * dwa2);
                    double dw3 = dw * dw * dw;
                    double dw9 = dw3 * dw3 * dw3;
                    ulr += (r->flr_lja[t0] / (9.0 * dw9) - r->flr_ljc[t0] / (3.0 * dw3));
                    double t = r->flr_bur[t0];
                    double exp2a = r->flr_bua[t0] * std::exp(-dw / t);
                    aux = aux + sgn * ((t + dw) * exp2a - r->flr_buc[t0] * dwa2);
                    ulr += (t * (2.0 * t + dw) * exp2a - r->flr_buc[t0] / (3.0 * dw3));
                }
                fz[i] -= aux;
                if (it <= r->nltype) fwsz[j + 1] += aux;
            }
        }
        uavex += ulr;
    }

    // ---- force_fouri (src/forcem.f90:827-937)
    {
        const int64_t ng = r->ngogo, KL = r->klmax, KM = r->kmmax, KN = r->knmax;
        std::vector<cplx> el((size_t)ng * (KL + 1)), em((size_t)ng * (2 * KM + 1)), en((size_t)ng * (2 * KN + 1));
        auto EL = [&](int64_t i, int64_t l) -> cplx& { return el[i * (KL + 1) + l]; };
        auto EM = [&](int64_t i, int64_t m) -> cplx& { return em[i * (2 * KM + 1) + m + KM]; };
        auto EN = [&](int64_t i, int64_t n) -> cplx& { return en[i * (2 * KN + 1) + n + KN]; };
        for (int64_t i = 0; i < ng; ++i) {
            EL(i, 0) = EM(i, 0) = EN(i, 0) = cplx(1.0, 0.0);
            double ax = r->pipix * x0[i], ay = r->pipiy * y0[i], az = r->pipiz * z0[i];
            EL(i, 1) = cplx(std::cos(ax), std::sin(ax));
            EM(i, 1) = cplx(std::cos(ay), std::sin(ay));
            EN(i, 1) = cplx(std::cos(az), std::sin(az));
            for (int64_t l = 2; l <= KL; ++l) EL(i, l) = EL(i, l - 1) * EL(i, 1);
            for (int64_t m = 2; m <= KM; ++m) EM(i, m) = EM(i, m - 1) * EM(i, 1);
            for (int64_t m = 1; m <= KM; ++m) EM(i, -m) = std::conj(EM(i, m));
            for (int64_t n = 2; n <= KN; ++n) EN(i, n) = EN(i, n - 1) * EN(i, 1);
            for (int64_t n = 1; n <= KN; ++n) EN(i, -n) = std::conj(EN(i, n));
        }
        const int64_t nk = (int64_t)r->Ak.size();
        r->wqsum.assign(nk, cplx(0.0, 0.0));
        double ewqLL = 0.0;
#ifdef _OPENMP
#pragma omp parallel
#endif
        {
            std::vector<double> tfx(nmove, 0.0), tfy(nmove, 0.0), tfz(nmove, 0.0);
            std::vector<cplx> elmn(ng);
            double tLL = 0.0, tew = 0.0;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
            for (int64_t k = 0; k < nk; ++k) {
                const int kl = r->kl_[k], km = r->km_[k], kn = r->kn_[k];
                const double rl = r->pipix * (double)(float)kl, rm = r->pipiy * (double)(float)km,
                             rn = r->pipiz * (double)(float)kn;
                cplx qll(0.0, 0.0);
                for (int64_t i = 0; i < ng; ++i) {
                    elmn[i] = r->qs[i] * EL(i, kl) * EM(i, km) * EN(i, kn);
                    qll += elmn[i];
                }
                cplx qsum = qll + r->Qsumw1[k] + r->Qsumw2[k];
                r->wqsum[k] = qsum;
                const double akx = r->Ak[k];
                tLL += (akx * qll * std::conj(qll)).real();
                tew += akx * (qsum * std::conj(qsum)).real();
                for (int64_t i = 0; i < nmove; ++i) {
                    double ft = akx * (std::conj(qsum) * elmn[i]).imag();
                    tfx[i] += ft * rl; tfy[i] += ft * rm; tfz[i] += ft * rn;
                }
            }
#ifdef _OPENMP
#pragma omp critical
#endif
            {
                for (int64_t i = 0; i < nmove; ++i) {
                    fx[i] += tfx[i]; fy[i] += tfy[i]; fz[i] += tfz[i];
                }
                ewqLL += tLL;
                uewa += tew;
            }
        }
        ewqLL *= 0.5;
        uewa *= 0.5;
        uavex += uewa;
        if (e) {
            e->ewqLL = ewqLL;
            e->ewqWW = r->ewqWW;
            e->ewqWL = uewa - r->ewqWW - ewqLL;
        }
        if (r->variant == MDG_SLAB) {  // EW3DC (src/forcem.f90:924-928)
            double dipz = 0.0;
            for (int64_t i = 0; i < nmove; ++i) dipz += r->qs[i] * z0[i];
            r->wdipz = dipz;
            double crf = -2.0 * M_PI_R * r->lzi * r->lxi * r->lyi;
            urf = -crf * facq * dipz * dipz;
            crf = 2.0 * crf * facq * dipz;
            for (int64_t i = 0; i < nmove; ++i) fz[i] += crf * r->qs[i];
            if (hist) {  // src/forcem.f90:930-934: whole fz of the liquid ions so far
                Hist th(r, hist);
                for (int64_t i = nriga; i < r->nliqa; ++i) th.ef(r->itype[i] - 3, r->zbin(z0[i]), fz[i]);
                th.merge();
            }
        }
    }

    // ---- force_intra (src/forcem.f90:565-652)
    for (int64_t ia = 0; ia < r->nang; ++ia) {
        const int64_t it = r->iatype[ia] - 1;
        for (int64_t is = 0; is < r->nangt[it]; ++is) {
            const int64_t i = r->ang1[is + MDG_SMX * ia] - 1, j = r->ang2[is + MDG_SMX * ia] - 1,
                          k = r->ang3[is + MDG_SMX * ia] - 1;
            auto X = [&](int64_t a) { return a < nmove ? x0[a] : r->wx[a - nmove]; };
            auto Y = [&](int64_t a) { return a < nmove ? y0[a] : r->wy[a - nmove]; };
            auto Z = [&](int64_t a) { return a < nmove ? z0[a] : r->wz[a - nmove]; };
            double ax = r->mx(X(k) - X(j)), ay = r->my(Y(k) - Y(j)), az = r->mz_real(Z(k) - Z(j));
            double bx = r->mx(X(j) - X(i)), by = r->my(Y(j) - Y(i)), bz = r->mz_real(Z(j) - Z(i));
            double ai = 1.0 / std::sqrt(ax * ax + ay * ay + az * az);
            double bi = 1.0 / std::sqrt(bx * bx + by * by + bz * bz);
            double ab = ax * bx + ay * by + az * bz;
            double cang = -ab * ai * bi;
            double fij = r->kt[it + r->ntype * is] * (std::acos(cang) - r->theta[it + r->ntype * is]) /
                         std::sqrt(1.0 - cang * cang);
            fij = fij * ai * bi;
            double bb = ab * bi * bi, aa = ab * ai * ai;
            double tmp = aa * ax - bx;
            if (k < nmove) fx[k] += fij * tmp;
            if (j < nmove) fx[j] += fij * (bb * bx - ax - tmp);
            tmp = aa * ay - by;
            if (k < nmove) fy[k] += fij * tmp;
            if (j < nmove) fy[j] += fij * (bb * by - ay - tmp);
            tmp = aa * az - bz;
            if (k < nmove) fz[k] += fij * tmp;
            if (j < nmove) fz[j] += fij * (bb * bz - az - tmp);
            if (hist) {  // src/forcem.f90:617-625
                const int64_t l = (int64_t)((cang + 1.0) * 100.0) + 1;
                Meas& m = r->ms;
                if (l >= 0 && l <= m.langmax && it < m.ntz) ++m.ngang[it + m.ntz * l];
                else ++m.oor;
            }
        }
    }

    // ---- serial force_sum (src/forcem_3d.f90:1031-1070)
    uavex += urf;
    {
        double sx = 0, sy = 0, sz = 0;
        for (int64_t i = 0; i < nmove; ++i) {
            sx += fx[i]; sy += fy[i]; sz += fz[i];
        }
        fwsx[1] = sx; fwsy[1] = sy; fwsz[1] = sz;
    }
    for (int c = 0; c < 3; ++c) {
        r->ms.fws[0][c] = fwsx[c]; r->ms.fws[1][c] = fwsy[c]; r->ms.fws[2][c] = fwsz[c];
    }
    if (hist) {
        Meas& m = r->ms;
        if (r->variant == MDG_SLAB)  // src/forcem.f90:1094-1098 (ftz = fz of the flexible atoms)
            for (int64_t i = nriga; i < r->nliqa; ++i) {
                const int64_t t = r->itype[i] - 3, l = r->zbin(z0[i]);
                if (t >= 0 && t < 2 && l >= 0 && l <= m.lmax) {
                    ++m.nefipos[t + 2 * l];
                    m.tefipos[t + 2 * l] += fz[i];
                } else {
                    ++m.oor;
                }
            }
        ++m.calls_force;
    }
    if (fxo)
        for (int64_t i = 0; i < nmove; ++i) {
            fxo[i] = fx[i]; fyo[i] = fy[i]; fzo[i] = fz[i];
        }
    for (int64_t i = nriga; i < nmove; ++i) {
        if (ftx) {
            ftx[i - nriga] = fx[i]; fty[i - nriga] = fy[i]; ftz[i - nriga] = fz[i];
        }
    }
    for (int64_t i = 0; i < nrig; ++i) {
        const int64_t j = 3 * i;
        if (fcx) {
            fcx[i] = fx[j] + fx[j + 1] + fx[j + 2];
            fcy[i] = fy[j] + fy[j + 1] + fy[j + 2];
            fcz[i] = fz[j] + fz[j + 1] + fz[j + 2];
        }
    }
    for (int64_t i = 0; i < nrig; ++i) {
        const int64_t j = 3 * i;
        for (int s = 0; s < 3; ++s) {
            rsx[s] = x0[j + s] - cx0[i];
            rsy[s] = y0[j + s] - cy0[i];
            rsz[s] = z0[j + s] - cz0[i];
        }
        if (tx) {
            tx[i] = (rsy[0] * fz[j] - rsz[0] * fy[j]) + (rsy[1] * fz[j + 1] - rsz[1] * fy[j + 1]) +
                    (rsy[2] * fz[j + 2] - rsz[2] * fy[j + 2]);
            ty[i] = (rsz[0] * fx[j] - rsx[0] * fz[j]) + (rsz[1] * fx[j + 1] - rsx[1] * fz[j + 1]) +
                    (rsz[2] * fx[j + 2] - rsx[2] * fz[j + 2]);
            tz[i] = (rsx[0] * fy[j] - rsy[0] * fx[j]) + (rsx[1] * fy[j + 1] - rsy[1] * fx[j + 1]) +
                    (rsx[2] * fy[j + 2] - rsy[2] * fx[j + 2]);
        }
    }
    r->wx0.assign(x0, x0 + nmove);
    r->wy0.assign(y0, y0 + nmove);
    r->wz0.assign(z0, z0 + nmove);
    r->wx0.insert(r->wx0.end(), r->wx.begin(), r->wx.end());
    r->wy0.insert(r->wy0.end(), r->wy.begin(), r->wy.end());
    r->wz0.insert(r->wz0.end(), r->wz.begin(), r->wz.end());
    r->wrsx.assign(rsx, rsx + nmove);
    r->wrsy.assign(rsy, rsy + nmove);
    r->wrsz.assign(rsz, rsz + nmove);
    if (e) {
        double sumlj = 0.0, sumqq = 0.0;
        for (int64_t k = 0; k < nijt; ++k) {
            sumlj += elj[k];
            sumqq += eqq[k];
            if (e->elj) e->elj[k] = elj[k];
            if (e->eqq) e->eqq[k] = eqq[k];
        }
        e->uewa = uewa;
        e->urf = urf;
        e->ulr = ulr;
        e->uself = r->uself;
        double uconf = sumlj + sumqq + uewa + r->uself + urf;
        e->uconf = uconf - r->uself;
        e->uavex = uavex;
        e->vir = 0.0;
        e->press = (fwsz[2] - fwsz[0]) / (2.0 * r->lx * r->ly) * 1000.0 / (PH_Na * F(1e-30f)) * F(1e-5f);
        for (int c = 0; c < 3; ++c) {
            e->fwsx[c] = fwsx[c]; e->fwsy[c] = fwsy[c]; e->fwsz[c] = fwsz[c];
        }
    }
    return MDG_OK;
}

// move_shake (src/move.f90:408-529).  x0..: ntota; xold..: ntota-nliqa; ftx..: nmove-nriga.
int ref_shake(RefCtx* r, double* x0, double* y0, double* z0, double* xold, double* yold, double* zold,
              const double* ftx, const double* fty, const double* ftz, double* kps_out, double* tkps,
              int32_t* sweeps) {
    const int64_t ismin = r->nliqa, ismax = r->nmove;  // 0-based [ismin, ismax)
    const int64_t nl = r->nliqa, nr = r->nriga;
    std::vector<double> kps(r->nit, 0.0);
    for (int64_t i = ismin; i < ismax; ++i) {
        const int64_t it = r->itype[i] - 1;
        double aux = xold[i - nl];
        xold[i - nl] = x0[i];
        aux = x0[i] - aux;
        aux = r->mx(aux);
        x0[i] = x0[i] + aux + ftx[i - nr] * r->mii[i];
        double kaux = aux * aux;
        aux = yold[i - nl];
        yold[i - nl] = y0[i];
        aux = y0[i] - aux;
        aux = r->my(aux);
        y0[i] = y0[i] + aux + fty[i - nr] * r->mii[i];
        kaux = kaux + aux * aux;
        aux = zold[i - nl];
        zold[i - nl] = z0[i];
        aux = z0[i] - aux;
        z0[i] = z0[i] + aux + ftz[i - nr] * r->mii[i];
        kaux = kaux + aux * aux;
        kps[it] += r->mi[i] * kaux;
    }
    double ks = 0.0;
    for (double v : kps) ks += v;
    if (tkps) *tkps = r->nfreed > 0 ? ks * 1000.0 / (PH_R * (double)(float)r->nfreed) : 0.0;
    if (kps_out)
        for (int64_t t = 0; t < r->nit; ++t) kps_out[t] = kps[t];

    // moving/moved flags over ismin..ntota (walls stay "not moved" = 1)
    std::vector<int> moving(r->ntota - ismin, 1), moved(r->ntota - ismin, 1);
    for (int64_t i = ismin; i < ismax; ++i) moved[i - ismin] = 0;
    auto X = [&](int64_t a) -> double& { return x0[a]; };
    const bool clean = (r->quirks & MDG_QUIRK_CLEAN_SHAKE_DONE) != 0;
    bool done = false;
    int ite = 0;
    const double lx = r->lx, ly = r->ly, lz = r->lz, lxi = r->lxi, lyi = r->lyi, lzi = r->lzi;
    for (;;) {
        if (done || ite > r->maxit) break;
        bool any = false;
        for (int64_t ic = 0; ic < r->ncons; ++ic) {
            done = true;
            const int64_t it = r->ictype[ic] - 1;
            for (int64_t is = 0; is < r->nconst[it]; ++is) {
                const int64_t ia = r->constra[is + MDG_SMX * ic] - 1, ib = r->constrb[is + MDG_SMX * ic] - 1;
                if (ia < ismin || ib < ismin) return fail(r, MDG_E_ARG, "constraint atom below the surface range");
                if (moved[ia - ismin] * moved[ib - ismin] != 0) continue;
                double px = x0[ia] - x0[ib]; px = px - lx * anint(px * lxi);
                double py = y0[ia] - y0[ib]; py = py - ly * anint(py * lyi);
                double pz = z0[ia] - z0[ib]; pz = pz - lz * anint(pz * lzi);
                const double L = r->length[it + r->ntype * is];
                double rabsq = L * L;
                double diffsq = rabsq - (px * px + py * py + pz * pz);
                if (std::fabs(diffsq) > rabsq * r->tol2) {
                    auto OX = [&](int64_t a, int c) -> double {
                        if (a >= nl) return c == 0 ? xold[a - nl] : c == 1 ? yold[a - nl] : zold[a - nl];
                        return 0.0;
                    };
                    double rx = OX(ia, 0) - OX(ib, 0); rx = rx - lx * anint(rx * lxi);
                    double ry = OX(ia, 1) - OX(ib, 1); ry = ry - ly * anint(ry * lyi);
                    double rz = OX(ia, 2) - OX(ib, 2); rz = rz - lz * anint(rz * lzi);
                    double rpab = rx * px + ry * py + rz * pz;
                    if (rpab < rabsq * r->rptol) {
                        char b[160];
                        snprintf(b, sizeof b, "Constraint failure: atoms %lld %lld", (long long)ia + 1, (long long)ib + 1);
                        if (sweeps) *sweeps = ite + 1;
                        return fail(r, MDG_E_SHAKE_RPTOL, b);
                    }
                    double rma = r->mii[ia], rmb = r->mii[ib];
                    double aux = diffsq / (2.0 * (rma + rmb) * rpab);
                    rma = rma * aux;
                    rmb = rmb * aux;
                    X(ia) += rx * rma; y0[ia] += ry * rma; z0[ia] += rz * rma;
                    x0[ib] -= rx * rmb; y0[ib] -= ry * rmb; z0[ib] -= rz * rmb;
                    moving[ia - ismin] = 0;
                    moving[ib - ismin] = 0;
                    done = false;
                    any = true;
                }
            }
        }
        if (clean) done = !any;
        ++ite;
        for (int64_t i = ismin; i < ismax; ++i) {
            moved[i - ismin] = moving[i - ismin];
            moving[i - ismin] = 1;
        }
    }
    if (sweeps) *sweeps = ite;
    if (!done && r->ncons > 0) return fail(r, MDG_E_SHAKE_MAXIT, "shake(): Too many constraint iterations!");
    return MDG_OK;
}

// ------------------------------------------------------------------------------------------
// Resident mode: move_predict (src/move.f90:48-217), force_get, move_correct (:220-383) and
// move_shake, in the order of the production loop (src/main.f90:58-68).
// ------------------------------------------------------------------------------------------
static const double Gf01 = F(0.348611111f), Gf11 = 1.0, Gf21 = F(0.916666667f), Gf31 = F(0.333333333f),
                    Gf41 = F(0.041666667f);
static const double Gf02 = F(0.158300000f), Gf12 = F(0.757000000f), Gf22 = 1.0, Gf32 = 0.5,
                    Gf42 = F(0.083333333f);

static void gear_predict(double& a0, double& a1, double& a2, double& a3, double a4) {
    a0 = a0 + a1 + a2 + a3 + a4;
    a1 = a1 + 2 * a2 + 3 * a3 + 4 * a4;
    a2 = a2 + 3 * a3 + 6 * a4;
    a3 = a3 + 4 * a4;
}

static void move_predict(RefCtx* r) {
    const int64_t tmin = r->nriga, tmax = r->nliqa, nrig = r->nrig;
    for (int64_t i = tmin; i < tmax; ++i)
        for (int d = 0; d < 3; ++d)
            gear_predict(r->X[d][i], r->XD[0][d][i], r->XD[1][d][i], r->XD[2][d][i], r->XD[3][d][i]);
    double kp = 0.0;
    for (int64_t i = tmin; i < tmax; ++i)
        kp += r->mi[i] * (r->XD[0][0][i] * r->XD[0][0][i] + r->XD[0][1][i] * r->XD[0][1][i] +
                          r->XD[0][2][i] * r->XD[0][2][i]);
    for (int64_t i = 0; i < nrig; ++i)
        for (int d = 0; d < 3; ++d) gear_predict(r->C[0][d][i], r->C[1][d][i], r->C[2][d][i], r->C[3][d][i], r->C[4][d][i]);
    double sc[3] = {0, 0, 0};
    for (int d = 0; d < 3; ++d)
        for (int64_t i = 0; i < nrig; ++i) sc[d] += r->C[1][d][i] * r->C[1][d][i];
    kp = kp + r->body.mw * (sc[0] + sc[1] + sc[2]);
    for (int64_t i = 0; i < nrig; ++i)
        for (int d = 0; d < 3; ++d) gear_predict(r->W[0][d][i], r->W[1][d][i], r->W[2][d][i], r->W[3][d][i], r->W[4][d][i]);
    double sw[3] = {0, 0, 0};
    for (int d = 0; d < 3; ++d)
        for (int64_t i = 0; i < nrig; ++i) sw[d] += r->W[0][d][i] * r->W[0][d][i];
    const double kw = r->body.inxx * sw[0] + r->body.inyy * sw[1] + r->body.inzz * sw[2];
    for (int64_t i = 0; i < nrig; ++i) {
        for (int c = 0; c < 4; ++c) gear_predict(r->Q[c][0][i], r->Q[c][1][i], r->Q[c][2][i], r->Q[c][3][i], r->Q[c][4][i]);
        double& q1 = r->Q[0][0][i];
        double& q2 = r->Q[1][0][i];
        double& q3 = r->Q[2][0][i];
        double& q4 = r->Q[3][0][i];
        const double cr = 1.0 / std::sqrt(q1 * q1 + q2 * q2 + q3 * q3 + q4 * q4);
        q1 = q1 * cr; q2 = q2 * cr; q3 = q3 * cr; q4 = q4 * cr;
        r->A[0][i] = -q1 * q1 + q2 * q2 - q3 * q3 + q4 * q4;
        r->A[1][i] = 2.0 * (q3 * q4 - q1 * q2);
        r->A[2][i] = 2.0 * (q2 * q3 + q1 * q4);
        r->A[3][i] = -2.0 * (q1 * q2 + q3 * q4);
        r->A[4][i] = q1 * q1 - q2 * q2 - q3 * q3 + q4 * q4;
        r->A[5][i] = 2.0 * (q2 * q4 - q1 * q3);
        r->A[6][i] = 2.0 * (q2 * q3 - q1 * q4);
        r->A[7][i] = -2.0 * (q1 * q3 + q4 * q2);
        r->A[8][i] = -q1 * q1 - q2 * q2 + q3 * q3 + q4 * q4;
    }
    const mdg_rigid& b = r->body;
    for (int64_t i = 0; i < nrig; ++i) {
        const int64_t ix = 3 * i;
        for (int j = 0; j < 3; ++j) {
            r->X[0][ix + j] = r->C[0][0][i] + r->A[0][i] * b.xbody[j] + r->A[3][i] * b.ybody[j] + r->A[6][i] * b.zbody[j];
            r->X[1][ix + j] = r->C[0][1][i] + r->A[1][i] * b.xbody[j] + r->A[4][i] * b.ybody[j] + r->A[7][i] * b.zbody[j];
            r->X[2][ix + j] = r->C[0][2][i] + r->A[2][i] * b.xbody[j] + r->A[5][i] * b.ybody[j] + r->A[8][i] * b.zbody[j];
        }
        for (int j = 1; j < 3; ++j)
            for (int d = 0; d < 3; ++d) r->RS[d][ix + j] = r->X[d][ix + j] - r->X[d][ix];
    }
    if (b.temper == -1.0) {
        r->s[0] = r->s[1] = r->rs[0] = r->rs[1] = 0.0;
    } else {
        gear_predict(r->s[0], r->s[1], r->s[2], r->s[3], r->s[4]);
        gear_predict(r->rs[0], r->rs[1], r->rs[2], r->rs[3], r->rs[4]);
    }
    r->kp = kp;
    r->kw = kw;
    r->ke = kp + kw;
    const int64_t nfree = r->nliqa - r->nriga;
    const double tstar = PH_R * b.temper / 1000.0;
    double qmass = (double)(float)(3 * (nfree + nrig)) * tstar * F(2e3f);
    double rmass = (double)(float)(3 * nrig) * tstar * F(1e3f);
    qmass = qmass / 10.0;
    rmass = rmass / 10.0;
    r->htot = 0.5 * (r->ke + qmass * r->s[0] * r->s[0] + rmass * r->rs[0] * r->rs[0]) + r->uconf;
    r->sft = (kp - (double)(float)(3 * (nfree + nrig) - 2) * tstar) / qmass;
    r->sfr = (kw - (double)(float)(3 * nrig + 1) * tstar) / rmass;
}

static void move_correct(RefCtx* r, const std::vector<double>* ft, const std::vector<double>* fc,
                         const std::vector<double>* tq) {
    const int64_t tmin = r->nriga, tmax = r->nliqa, nrig = r->nrig;
    double rcorr = 0.5;
    const double s0i = r->s[0];
    for (int64_t i = tmin; i < tmax; ++i)
        for (int d = 0; d < 3; ++d) {
            const double cort = rcorr * ft[d][i - r->nriga] * r->mii[i] - r->XD[0][d][i] * s0i - r->XD[1][d][i];
            r->X[d][i] = r->X[d][i] + Gf02 * cort;
            r->XD[0][d][i] = r->XD[0][d][i] + Gf12 * cort;
            r->XD[1][d][i] = r->XD[1][d][i] + Gf22 * cort;
            r->XD[2][d][i] = r->XD[2][d][i] + Gf32 * cort;
            r->XD[3][d][i] = r->XD[3][d][i] + Gf42 * cort;
        }
    rcorr = rcorr / r->body.mw;
    for (int64_t i = 0; i < nrig; ++i)
        for (int d = 0; d < 3; ++d) {
            const double c1 = rcorr * fc[d][i] - r->C[1][d][i] * s0i - r->C[2][d][i];
            r->C[0][d][i] = r->C[0][d][i] + Gf02 * c1;
            r->C[1][d][i] = r->C[1][d][i] + Gf12 * c1;
            r->C[2][d][i] = r->C[2][d][i] + Gf22 * c1;
            r->C[3][d][i] = r->C[3][d][i] + Gf32 * c1;
            r->C[4][d][i] = r->C[4][d][i] + Gf42 * c1;
        }
    for (int64_t i = 0; i < nrig; ++i) {
        const double q1 = r->Q[0][0][i], q2 = r->Q[1][0][i], q3 = r->Q[2][0][i], q4 = r->Q[3][0][i];
        const double wx = r->W[0][0][i], wy = r->W[0][1][i], wz = r->W[0][2][i];
        double cq[4];
        cq[0] = 0.5 * (-q3 * wx - q4 * wy + q2 * wz);
        cq[1] = 0.5 * (q4 * wx - q3 * wy - q1 * wz);
        cq[2] = 0.5 * (q1 * wx + q2 * wy + q4 * wz);
        cq[3] = 0.5 * (-q2 * wx + q1 * wy - q3 * wz);
        for (int c = 0; c < 4; ++c) {
            const double co = cq[c] - r->Q[c][1][i];
            r->Q[c][0][i] = r->Q[c][0][i] + Gf01 * co;
            r->Q[c][1][i] = r->Q[c][1][i] + Gf11 * co;
            r->Q[c][2][i] = r->Q[c][2][i] + Gf21 * co;
            r->Q[c][3][i] = r->Q[c][3][i] + Gf31 * co;
            r->Q[c][4][i] = r->Q[c][4][i] + Gf41 * co;
        }
    }
    rcorr = 1.0;
    const double rs0i = r->rs[0];
    const mdg_rigid& b = r->body;
    const double inxxi = 1.0 / b.inxx, inyyi = 1.0 / b.inyy, inzzi = 1.0 / b.inzz;
    for (int64_t i = 0; i < nrig; ++i) {
        const double wx = r->W[0][0][i], wy = r->W[0][1][i], wz = r->W[0][2][i];
        double c1 = r->A[0][i] * tq[0][i] + r->A[1][i] * tq[1][i] + r->A[2][i] * tq[2][i];
        c1 = ((c1 * rcorr + wy * wz * (b.inyy - b.inzz)) * inxxi) - r->W[1][0][i] - rs0i * wx;
        double c2 = r->A[3][i] * tq[0][i] + r->A[4][i] * tq[1][i] + r->A[5][i] * tq[2][i];
        c2 = ((c2 * rcorr + wz * wx * (b.inzz - b.inxx)) * inyyi) - r->W[1][1][i] - rs0i * wy;
        double c3 = r->A[6][i] * tq[0][i] + r->A[7][i] * tq[1][i] + r->A[8][i] * tq[2][i];
        c3 = ((c3 * rcorr + wx * wy * (b.inxx - b.inyy)) * inzzi) - r->W[1][2][i] - rs0i * wz;
        const double cc[3] = {c1, c2, c3};
        for (int d = 0; d < 3; ++d) {
            r->W[0][d][i] = r->W[0][d][i] + Gf01 * cc[d];
            r->W[1][d][i] = r->W[1][d][i] + Gf11 * cc[d];
            r->W[2][d][i] = r->W[2][d][i] + Gf21 * cc[d];
            r->W[3][d][i] = r->W[3][d][i] + Gf31 * cc[d];
            r->W[4][d][i] = r->W[4][d][i] + Gf41 * cc[d];
        }
    }
    if (b.temper != -1.0) {
        double rc = r->sft - r->s[1];
        r->s[0] = r->s[0] + Gf01 * rc;
        r->s[1] = r->sft;
        r->s[2] = r->s[2] + Gf21 * rc;
        r->s[3] = r->s[3] + Gf31 * rc;
        r->s[4] = r->s[4] + Gf41 * rc;
        rc = r->sfr - r->rs[1];
        r->rs[0] = r->rs[0] + Gf01 * rc;
        r->rs[1] = r->sfr;
        r->rs[2] = r->rs[2] + Gf21 * rc;
        r->rs[3] = r->rs[3] + Gf31 * rc;
        r->rs[4] = r->rs[4] + Gf41 * rc;
    }
}

int ref_set_state(RefCtx* r, const mdg_rigid* b, const mdg_state* st) {
    const int64_t nt = r->ntota, nrig = r->nrig, nold = r->ntota - r->nliqa, nm = r->nmove;
    auto cpy = [](std::vector<double>& v, const double* p, int64_t n) { v.assign(p, p + n); };
    cpy(r->X[0], st->x0, nt); cpy(r->X[1], st->y0, nt); cpy(r->X[2], st->z0, nt);
    for (int k = 0; k < 4; ++k) {
        cpy(r->XD[k][0], st->xd[k], nt); cpy(r->XD[k][1], st->yd[k], nt); cpy(r->XD[k][2], st->zd[k], nt);
    }
    for (int k = 0; k < 5; ++k) {
        cpy(r->C[k][0], st->cx[k], nrig); cpy(r->C[k][1], st->cy[k], nrig); cpy(r->C[k][2], st->cz[k], nrig);
        cpy(r->W[k][0], st->wx[k], nrig); cpy(r->W[k][1], st->wy[k], nrig); cpy(r->W[k][2], st->wz[k], nrig);
        for (int c = 0; c < 4; ++c) cpy(r->Q[c][k], st->q[c][k], nrig);
    }
    cpy(r->OLD[0], st->xold, nold); cpy(r->OLD[1], st->yold, nold); cpy(r->OLD[2], st->zold, nold);
    cpy(r->RS[0], st->rsx, nm); cpy(r->RS[1], st->rsy, nm); cpy(r->RS[2], st->rsz, nm);
    for (int k = 0; k < 9; ++k) r->A[k].assign(nrig, 0.0);
    for (int k = 0; k < 5; ++k) {
        r->s[k] = st->s[k];
        r->rs[k] = st->rs[k];
    }
    r->body = *b;
    r->have_state = true;
    return MDG_OK;
}

int ref_get_state(RefCtx* r, mdg_state* st) {
    if (!r->have_state) return fail(r, MDG_E_ARG, "no state");
    const int64_t nt = r->ntota, nrig = r->nrig, nold = r->ntota - r->nliqa, nm = r->nmove;
    auto out = [](const std::vector<double>& v, double* p, int64_t n) {
        if (p) std::copy(v.begin(), v.begin() + n, p);
    };
    out(r->X[0], st->x0, nt); out(r->X[1], st->y0, nt); out(r->X[2], st->z0, nt);
    for (int k = 0; k < 4; ++k) {
        out(r->XD[k][0], st->xd[k], nt); out(r->XD[k][1], st->yd[k], nt); out(r->XD[k][2], st->zd[k], nt);
    }
    for (int k = 0; k < 5; ++k) {
        out(r->C[k][0], st->cx[k], nrig); out(r->C[k][1], st->cy[k], nrig); out(r->C[k][2], st->cz[k], nrig);
        out(r->W[k][0], st->wx[k], nrig); out(r->W[k][1], st->wy[k], nrig); out(r->W[k][2], st->wz[k], nrig);
        for (int c = 0; c < 4; ++c) out(r->Q[c][k], st->q[c][k], nrig);
    }
    out(r->OLD[0], st->xold, nold); out(r->OLD[1], st->yold, nold); out(r->OLD[2], st->zold, nold);
    out(r->RS[0], st->rsx, nm); out(r->RS[1], st->rsy, nm); out(r->RS[2], st->rsz, nm);
    for (int k = 0; k < 5; ++k) {
        st->s[k] = r->s[k];
        st->rs[k] = r->rs[k];
    }
    return MDG_OK;
}

// ---- measurement (src/measure.f90) ------------------------------------------------------------
// measure_init (src/measure.f90:66-176): bins of width rdel over the slab, lmax = int(lw/rdel+0.5)+1.
int ref_measure_init(RefCtx* r, const mdg_measure_params* p, mdg_measure_dims* d) {
    if (!p || !(p->rdel > 0.0)) return fail(r, MDG_E_ARG, "measure: rdel must be positive");
    Meas& m = r->ms;
    m = Meas();
    m.rdeli = 1.0 / p->rdel;
    m.lmax = (int64_t)(r->lw * m.rdeli + 0.5) + 1;
    m.ntz = std::max<int64_t>(r->nit - 2, 1);
    m.langmax = 201;
    m.l2d = p->l2d != 0;
    m.rfrst = p->rfrst;
    m.rscnd = p->rscnd;
    m.lgxmax = (int64_t)(4.0 * r->cx * m.rdeli + 1.0);
    m.lgymax = (int64_t)(2.0 * r->cy * m.rdeli + 1.0);
    const int64_t L = m.lmax + 1;
    m.ngc.assign(r->nijt * L, 0);
    m.efipos.assign(2 * L, 0.0);
    m.tefipos.assign(2 * L, 0.0);
    m.nefipos.assign(2 * L, 0);
    m.ngang.assign(m.ntz * (m.langmax + 1), 0);
    m.ngz.assign(m.ntz * L, 0);
    m.ndipx.assign(L, 0.0);
    m.ndipy.assign(L, 0.0);
    m.ndipz.assign(L, 0.0);
    m.ndipsq.assign(L, 0.0);
    if (m.l2d) {
        m.ng2d1.assign(m.ntz * (m.lgxmax + 1) * (m.lgymax + 1), 0);
        m.ng2d2.assign(m.ntz * (m.lgxmax + 1) * (m.lgymax + 1), 0);
    }
    m.force_hist = p->force_hist != 0;
    m.profiles = p->profiles != 0;
    m.init = true;
    if (d) {
        d->lmax = m.lmax; d->nijt = r->nijt; d->ntz = m.ntz; d->langmax = m.langmax;
        d->lgxmax = m.lgxmax; d->lgymax = m.lgymax;
    }
    return MDG_OK;
}

int ref_measure_enable(RefCtx* r, int force_hist, int profiles) {
    if (!r->ms.init) return fail(r, MDG_E_ARG, "measure: not initialised");
    r->ms.force_hist = force_hist != 0;
    r->ms.profiles = profiles != 0;
    return MDG_OK;
}

// measure_zero (src/measure.f90:178-262), the arrays this library keeps
int ref_measure_zero(RefCtx* r) {
    Meas& m = r->ms;
    if (!m.init) return fail(r, MDG_E_ARG, "measure: not initialised");
    for (auto* v : {&m.ngc, &m.nefipos, &m.ngang, &m.ngz, &m.ng2d1, &m.ng2d2}) std::fill(v->begin(), v->end(), 0);
    for (auto* v : {&m.efipos, &m.tefipos, &m.ndipx, &m.ndipy, &m.ndipz, &m.ndipsq})
        std::fill(v->begin(), v->end(), 0.0);
    for (int c = 0; c < 3; ++c)
        for (int k = 0; k < 3; ++k) m.ftot[c][k] = 0.0;
    m.calls_force = m.calls_do = m.oor = 0;
    return MDG_OK;
}

// measure_do (src/measure.f90:270-312): summed wall forces, site z-profile, water dipole profile
// and the near-wall 2-D maps, over the moving atoms.
static void measure_do(Ref* r, const double* x0, const double* y0, const double* z0) {
    Meas& m = r->ms;
    for (int c = 0; c < 3; ++c)
        for (int k = 0; k < 3; ++k) m.ftot[c][k] += m.fws[c][k];
    const int64_t L = m.lmax + 1;
    std::vector<double> mux(L, 0.0), muy(L, 0.0), muz(L, 0.0);
    const double lxh = 0.5 * r->lx, lyh = 0.5 * r->ly;
    for (int64_t i = 0; i < r->nmove; ++i) {
        const int64_t it = r->itype[i];
        double rij = z0[i] + r->lwh;
        int64_t l = (int64_t)(rij * m.rdeli + 0.5);
        if (l >= 0 && l <= m.lmax && it - 1 < m.ntz) {
            ++m.ngz[(it - 1) + m.ntz * l];
            if (it == 1 && i + 2 < r->nmove) {  // a water O and its two H (the reference assumes it)
                muz[l] += (z0[i] - 0.5 * (z0[i + 1] + z0[i + 2]));
                mux[l] += (x0[i] - 0.5 * (x0[i + 1] + x0[i + 2]));
                muy[l] += (y0[i] - 0.5 * (y0[i + 1] + y0[i + 2]));
            }
        } else {
            ++m.oor;
        }
        rij = r->lwh - std::fabs(z0[i]);
        if (m.l2d && rij < m.rscnd) {
            const int64_t lx2 = (int64_t)(0.5 * fmodulo(x0[i] + lxh + 4.0 * r->cx, 4.0 * r->cx) * m.rdeli + 0.5);
            const int64_t ky2 = (int64_t)(0.5 * fmodulo(y0[i] + lyh + 2.0 * r->cy, 2.0 * r->cy) * m.rdeli + 0.5);
            if (lx2 >= 0 && ky2 >= 0 && lx2 <= m.lgxmax && ky2 <= m.lgymax && it - 1 < m.ntz) {
                const int64_t k = (it - 1) + m.ntz * (lx2 + (m.lgxmax + 1) * ky2);
                if (rij < m.rfrst) ++m.ng2d1[k];
                else ++m.ng2d2[k];
            } else {
                ++m.oor;
            }
        }
    }
    for (int64_t l = 0; l < L; ++l) {
        m.ndipx[l] += mux[l];
        m.ndipy[l] += muy[l];
        m.ndipz[l] += muz[l];
        m.ndipsq[l] += mux[l] * mux[l] + muy[l] * muy[l] + muz[l] * muz[l];
    }
    ++m.calls_do;
}

int ref_measure_do(RefCtx* r, const double* x0, const double* y0, const double* z0) {
    if (!r->ms.init) return fail(r, MDG_E_ARG, "measure: not initialised");
    if (!x0) {
        if (!r->have_state) return fail(r, MDG_E_ARG, "measure: no positions");
        x0 = r->X[0].data(); y0 = r->X[1].data(); z0 = r->X[2].data();
    }
    measure_do(r, x0, y0, z0);
    return MDG_OK;
}

int ref_measure_get(RefCtx* r, mdg_measure_out* o) {
    const Meas& m = r->ms;
    if (!m.init) return fail(r, MDG_E_ARG, "measure: not initialised");
    auto cp = [](const auto& v, auto* p) {
        if (p) std::copy(v.begin(), v.end(), p);
    };
    cp(m.ngc, o->ngc); cp(m.efipos, o->efipos); cp(m.tefipos, o->tefipos); cp(m.nefipos, o->nefipos);
    cp(m.ngang, o->ngang); cp(m.ngz, o->ngz); cp(m.ndipx, o->ndipx); cp(m.ndipy, o->ndipy);
    cp(m.ndipz, o->ndipz); cp(m.ndipsq, o->ndipsq); cp(m.ng2d1, o->ng2d1); cp(m.ng2d2, o->ng2d2);
    for (int c = 0; c < 3; ++c)
        for (int k = 0; k < 3; ++k) o->ftot[c][k] = m.ftot[c][k];
    o->calls_force = m.calls_force;
    o->calls_do = m.calls_do;
    o->out_of_range = m.oor;
    return MDG_OK;
}

// ---- chempot (src/forcem.f90:1226-1507) with the generator of src/rndmod.f90:26-35 ------------
static double rnd(double& seed) {
    seed = std::fmod(8192.0 * seed, 67099547.0);
    return seed * 1.4903230270690e-8;
}

static double erfc_as(double alfar) {
    const double t = 1.0 / (1.0 + PP * alfar);
    const double exp2a = std::exp(-alfar * alfar);
    return ((((A5 * t + A4) * t + A3) * t + A2) * t + A1) * t * exp2a;
}

int ref_widom(RefCtx* r, const mdg_widom_params* p, double* seed, double* pave, int64_t* inave, int64_t* done) {
    if (r->variant != MDG_SLAB) return fail(r, MDG_E_UNSUPPORTED, "Widom insertion: slab variant only");
    if (r->wx0.empty()) return fail(r, MDG_E_ARG, "Widom insertion: no force evaluation yet");
    if (done) *done = 0;
    // measure_init (src/measure.f90:151-155)
    const double lwmin = r->lwh - p->lwmax, lwmax = r->lwh - p->lwmin;
    const double facbin = 1.0 / (lwmax - lwmin) * (double)(float)p->lchmax;
    const double chtemper = p->temper > 0.0 ? p->temper : 300.0;
    const double aco = F(-0.333333f), asi = F(0.942809f);
    const double rinsmin = 4.0, rwinsmin = (double)(2.35f * 2.35f);
    const double qsw[3] = {F(-0.8476f), F(0.4238f), F(0.4238f)};
    const double beta = 1000.0 / (PH_R * chtemper);
    const double crf = (p->flags & MDG_WIDOM_EW3DC)
                           ? 2.0 * (-2.0 * M_PI_R * r->lzi * r->lxi * r->lyi) * r->facq * r->wdipz : 0.0;
    const std::vector<double>&x0 = r->wx0, &y0 = r->wy0, &z0 = r->wz0;
    const int64_t ntota = r->ntota, KL = r->klmax, KM = r->kmmax, KN = r->knmax;
    double sd = *seed;
    int64_t n = 0;
    std::vector<int64_t> iarr;
    std::vector<double> xarr, yarr, zarr;
    for (int64_t ic = 0; ic < p->ichmax; ++ic) {
        const double oxr = (rnd(sd) - 0.5) * r->lx;
        const double oyr = (rnd(sd) - 0.5) * r->ly;
        double ozr;
        do {
            ozr = ((rnd(sd) - 0.5) * lwmax * 2.0);
        } while (!(std::fabs(ozr) > lwmin));
        const int64_t il = (int64_t)((std::fabs(ozr) - lwmin) * facbin) + 1;
        if (il < 1 || il > p->lchmax) return fail(r, MDG_E_ARG, "Widom insertion: bin outside lchmax");
        const int irot = il > p->ilmid ? 20 : 1;
        inave[il - 1] += irot;
        ++n;
        // the O of the probe (src/forcem.f90:1278-1340)
        double uchem = 0.0;
        int pins = 1;
        iarr.clear(); xarr.clear(); yarr.clear(); zarr.clear();
        for (int64_t j = 0; j < ntota; ++j) {
            if (r->itype[j] == 2) continue;
            const double zio = ozr - z0[j];
            if (std::fabs(zio) > r->rcut) continue;
            const double xio = r->mx(oxr - x0[j]);
            const double yio = r->my(oyr - y0[j]);
            const double rsq = xio * xio + yio * yio + zio * zio;
            if (rsq > r->rcutsq) continue;
            const int64_t jt = r->itype[j];
            const int ijt = r->ij(1, jt);
            if (rsq < rwinsmin) {
                if (jt == 1 || rsq < rinsmin) {
                    pins = 0;
                    break;
                }
            }
            const double rsqi = 1.0 / rsq;
            const double rij = std::sqrt(rsq);
            if (r->vdwnum[ijt] == 1) {
                const double r6 = r->sig[ijt] * pw3(rsqi);
                uchem += r->eps[ijt] * r6 * (r6 - 1.0);
            } else if (r->vdwnum[ijt] == 2) {
                const double r6 = r->cc[ijt] * pw3(rsqi);
                uchem += r->aa[ijt] * std::exp(-rij * r->rhoi[ijt]) - r6;
            }
            const double aux = r->facq * qsw[0] * r->qs[j] / rij;
            uchem += erfc_as(r->alfa * rij) * aux;
            iarr.push_back(j); xarr.push_back(xio); yarr.push_back(yio); zarr.push_back(zio);
        }
        const double uchemx = uchem;
        if (pins == 0 && !(p->flags & MDG_WIDOM_SKIP_OVERLAP)) {
            *seed = sd;
            if (done) *done = n;
            return MDG_OK;   // the reference leaves the insertion loop (src/forcem.f90:1342)
        }
        for (int ir = 0; ir < irot; ++ir) {
            double h1[3], ri;
            for (;;) {
                h1[0] = rnd(sd) - 0.5;
                h1[1] = rnd(sd) - 0.5;
                h1[2] = rnd(sd) - 0.5;
                ri = h1[0] * h1[0] + h1[1] * h1[1] + h1[2] * h1[2];
                if (ri < 0.25 && ri > F(0.001f)) break;
            }
            ri = 1.0 / std::sqrt(ri);
            for (double& hh : h1) hh = hh * ri;
            ri = 1.0 / std::sqrt(h1[0] * h1[0] + h1[1] * h1[1]);
            const double h2[3] = {-h1[1] * ri, h1[0] * ri, 0.0};
            const double mr[3] = {h2[1] * h1[2] - h2[2] * h1[1], h2[2] * h1[0] - h2[0] * h1[2],
                                  h2[0] * h1[1] - h2[1] * h1[0]};
            const double alph = 2.0 * M_PI_R * rnd(sd);
            const double cosa = std::cos(alph), sina = std::sin(alph);
            double rins[3][3];
            const double o[3] = {oxr, oyr, ozr};
            for (int d = 0; d < 3; ++d) {
                rins[0][d] = o[d];
                rins[1][d] = o[d] + aco * h1[d] + asi * (cosa * h2[d] + sina * mr[d]);
                rins[2][d] = o[d] + h1[d];
            }
            if (pins == 0) continue;  // skipped position: its orientations are drawn but not used
            // real space (src/forcem.f90:1378-1423)
            uchem = 0.0;
            for (size_t k = 0; k < iarr.size(); ++k) {
                const int64_t j = iarr[k];
                const double xio = xarr[k], yio = yarr[k], zio = zarr[k];
                const int64_t jt = r->itype[j];
                if (jt == 1) {
                    int64_t jmin = j + 1;
                    for (int ix = 0; ix < 3; ++ix) {
                        const double xi = xio + rins[ix][0] - oxr, yi = yio + rins[ix][1] - oyr,
                                     zi = zio + rins[ix][2] - ozr;
                        const double qx = r->facq * qsw[ix];
                        for (int64_t jx = jmin; jx < j + r->nsi[jt - 1]; ++jx) {
                            const double xd = xi - r->wrsx[jx], yd = yi - r->wrsy[jx], zd = zi - r->wrsz[jx];
                            const double rsq = xd * xd + yd * yd + zd * zd;
                            const double rij = std::sqrt(rsq);
                            uchem += erfc_as(r->alfa * rij) * (qx * r->qs[jx] / rij);
                        }
                        jmin = j;
                    }
                } else {
                    for (int ix = 1; ix < 3; ++ix) {
                        const double xi = xio + rins[ix][0] - oxr, yi = yio + rins[ix][1] - oyr,
                                     zi = zio + rins[ix][2] - ozr;
                        const double qx = r->facq * qsw[ix];
                        const double rsq = xi * xi + yi * yi + zi * zi;
                        const double rij = std::sqrt(rsq);
                        uchem += erfc_as(r->alfa * rij) * (qx * r->qs[j] / rij);
                    }
                }
            }
            uchem = uchem + uchemx;
            // reciprocal space (src/forcem.f90:1428-1475)
            std::vector<cplx> el(3 * (KL + 1)), em(3 * (2 * KM + 1)), en(3 * (2 * KN + 1));
            auto EL = [&](int q, int64_t l) -> cplx& { return el[q * (KL + 1) + l]; };
            auto EM = [&](int q, int64_t m) -> cplx& { return em[q * (2 * KM + 1) + m + KM]; };
            auto EN = [&](int q, int64_t nn) -> cplx& { return en[q * (2 * KN + 1) + nn + KN]; };
            for (int q = 0; q < 3; ++q) {
                EL(q, 0) = EM(q, 0) = EN(q, 0) = cplx(1.0, 0.0);
                EL(q, 1) = cplx(std::cos(r->pipix * rins[q][0]), std::sin(r->pipix * rins[q][0]));
                EM(q, 1) = cplx(std::cos(r->pipiy * rins[q][1]), std::sin(r->pipiy * rins[q][1]));
                EN(q, 1) = cplx(std::cos(r->pipiz * rins[q][2]), std::sin(r->pipiz * rins[q][2]));
                for (int64_t l = 2; l <= KL; ++l) EL(q, l) = EL(q, l - 1) * EL(q, 1);
                for (int64_t m = 2; m <= KM; ++m) EM(q, m) = EM(q, m - 1) * EM(q, 1);
                for (int64_t m = 1; m <= KM; ++m) EM(q, -m) = std::conj(EM(q, m));
                for (int64_t nn = 2; nn <= KN; ++nn) EN(q, nn) = EN(q, nn - 1) * EN(q, 1);
                for (int64_t nn = 1; nn <= KN; ++nn) EN(q, -nn) = std::conj(EN(q, nn));
            }
            for (size_t k = 0; k < r->Ak.size(); ++k) {
                const int kl = r->kl_[k], km = r->km_[k], kn = r->kn_[k];
                cplx sum(0.0, 0.0);
                for (int q = 0; q < 3; ++q) sum += (qsw[q] * EL(q, kl) * EM(q, km)) * EN(q, kn);
                uchem += 0.5 * r->Ak[k] * (sum * std::conj(r->wqsum[k])).real();
            }
            uchem = uchem - crf * (qsw[0] * rins[0][2] + qsw[1] * rins[1][2] + qsw[2] * rins[2][2]);
            // wall tail of the O (src/forcem.f90:1481-1494)
            for (int j = -1; j <= 1; j += 2) {
                const double dw = r->lwh - (double)j * rins[0][2];
                if (dw < r->rcut) {
                    uchem += r->ulr_w[0];
                } else {
                    uchem += r->ulr_l[0];
                    const double dw3 = dw * dw * dw;
                    uchem += (r->flr_lja[0] / (9.0 * (dw3 * dw3 * dw3)) - r->flr_ljc[0] / (3.0 * dw3));
                    const double t = r->flr_bur[0];
                    const double exp2a = r->flr_bua[0] * std::exp(-dw / t);
                    uchem += (t * (2.0 * t + dw) * exp2a - r->flr_buc[0] / (3.0 * dw3));
                }
            }
            pave[il - 1] += std::exp(-beta * uchem);
        }
    }
    *seed = sd;
    if (done) *done = n;
    return MDG_OK;
}

int ref_run(RefCtx* r, int64_t nsteps, mdg_report* rep) {
    if (!r->have_state) return fail(r, MDG_E_ARG, "mdg_run before mdg_set_state");
    const int64_t nm = r->nmove, nflex = r->nmove - r->nriga, nrig = std::max<int64_t>(r->nrig, 1);
    std::vector<double> ft[3], fc[3], tq[3];
    for (int d = 0; d < 3; ++d) {
        ft[d].assign(std::max<int64_t>(nflex, 1), 0.0);
        fc[d].assign(nrig, 0.0);
        tq[d].assign(nrig, 0.0);
    }
    std::vector<double> cx(nrig), cy(nrig), cz(nrig), elj(r->nijt), eqq(r->nijt);
    for (int64_t step = 0; step < nsteps; ++step) {
        move_predict(r);
        for (int64_t i = 0; i < r->nrig; ++i) {
            cx[i] = r->C[0][0][i]; cy[i] = r->C[0][1][i]; cz[i] = r->C[0][2][i];
        }
        mdg_energies e{};
        e.elj = elj.data();
        e.eqq = eqq.data();
        int rc = ref_force_get(r, r->X[0].data(), r->X[1].data(), r->X[2].data(), cx.data(), cy.data(), cz.data(),
                               r->RS[0].data(), r->RS[1].data(), r->RS[2].data(), ft[0].data(), ft[1].data(),
                               ft[2].data(), fc[0].data(), fc[1].data(), fc[2].data(), tq[0].data(), tq[1].data(),
                               tq[2].data(), nullptr, nullptr, nullptr, &e);
        if (rc) return rc;
        r->uconf = e.uconf;
        r->press = e.press;
        move_correct(r, ft, fc, tq);
        if (nm > r->nliqa) {
            int32_t sw = 0;
            double tk = 0.0;
            rc = ref_shake(r, r->X[0].data(), r->X[1].data(), r->X[2].data(), r->OLD[0].data(), r->OLD[1].data(),
                           r->OLD[2].data(), ft[0].data(), ft[1].data(), ft[2].data(), nullptr, &tk, &sw);
            if (rc) return rc;
            r->last_sweeps = sw;
            r->tkps = tk;
        }
        if (r->ms.init && r->ms.profiles) measure_do(r, r->X[0].data(), r->X[1].data(), r->X[2].data());
        const int64_t nfree = r->nliqa - r->nriga;
        r->tempnow = r->ke * 1000.0 / (3.0 * PH_R * (double)(float)(nfree + 2 * r->nrig));
    }
    if (rep) {
        rep->kp = r->kp; rep->kw = r->kw; rep->ke = r->ke; rep->htot = r->htot; rep->tempnow = r->tempnow;
        rep->uconf = r->uconf; rep->tkps = r->tkps; rep->press = r->press; rep->steps = nsteps;
        rep->rebuilds = 0; rep->last_sweeps = r->last_sweeps;
    }
    return MDG_OK;
}

}  // extern "C"
