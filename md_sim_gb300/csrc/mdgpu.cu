// mdgpu.cu - C ABI of the md_sim GB300 library (include/mdgpu.h).
//
// mdg_create plays force_init (src/forcem.f90:54-81) with nnlist_init (src/nnlist.f90:14-90) and
// move_shake_init (src/move.f90:385-406); mdg_force_get plays force_get (src/forcem.f90:93-129);
// mdg_nnlist_make plays nnlist_make; mdg_shake plays move_shake.  All per-step work runs on one
// CUDA stream per context; host arrays are copied in and out around it.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "ctx.h"

namespace mdg {

static thread_local std::string g_err;

int set_err(Ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    g_err = msg;
    return code;
}

void* dalloc(Ctx& c, size_t bytes) {
    void* p = nullptr;
    bytes = std::max<size_t>(bytes, 16);
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
        c.alloc_failed = true;
        return nullptr;
    }
    cudaMemset(p, 0, bytes);
    c.owned.push_back(p);
    return p;
}

static void dfree(Ctx& c, void* p) {
    if (!p) return;
    cudaFree(p);
    for (auto& q : c.owned)
        if (q == p) q = nullptr;
}

namespace {

const double kPi = (double)3.1415926535898f;
const double kPH_e = (double)1.6021892e-19f, kPH_Na = (double)6.022045e23f, kPH_4epi = (double)8.987551784952e+9f,
             kPH_A2m = (double)1.0e-10f;

template <typename T>
T* upload(Ctx& c, const std::vector<T>& h) {
    T* d = (T*)dalloc(c, sizeof(T) * std::max<size_t>(h.size(), 1));
    if (d && !h.empty()) cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
    return d;
}

// force_real_init long-range tables (src/forcem.f90:167-228), host side.
void lr_tables(Ctx& c, const mdg_sysdesc* s, double rcut, std::vector<double>& tab) {
    const int nit = (int)s->nit;
    const int64_t nstw = s->nst[s->ntype - 1];
    tab.assign(9 * nit, 0.0);
    double* flr_l = &tab[0 * nit];
    double* flr_w = &tab[1 * nit];
    double* flr_lja = &tab[2 * nit];
    double* flr_ljc = &tab[3 * nit];
    double* flr_bua = &tab[4 * nit];
    double* flr_buc = &tab[5 * nit];
    double* flr_bur = &tab[6 * nit];
    double* ulr_l = &tab[7 * nit];
    double* ulr_w = &tab[8 * nit];
    for (int t = 0; t < nit; ++t) flr_bur[t] = 1.0;
    if (c.variant != MDG_SLAB) return;
    const double rholiq = (double)s->nmove / (s->lx * s->ly * s->lw);
    int64_t nsum = 0;
    for (int64_t k = 0; k < nstw; ++k) nsum += s->nss_wall[k];
    const double rhowall = (double)nsum / (2.0 * s->cx * s->cy * s->cz);
    std::vector<double> xdens(nit, 0.0);
    for (int64_t i = 0; i < s->nmove; ++i) xdens[s->itype[i] - 1] += 1.0;
    for (int t = 0; t < nit - nstw; ++t) xdens[t] = xdens[t] / (double)(float)s->nmove * rholiq;
    const float nss12 = (float)(s->nss_wall[0] + s->nss_wall[1]);
    if (nit >= 2) {
        xdens[nit - 2] = (double)((float)s->nss_wall[0] / nss12) * rhowall;
        xdens[nit - 1] = (double)((float)s->nss_wall[1] / nss12) * rhowall;
    }
    const double rc = rcut;
    for (int it = 1; it <= nit - nstw; ++it) {
        for (int jt = 1; jt <= nit; ++jt) {
            const int k = (int)s->ijtype[(it - 1) + nit * (jt - 1)] - 1;
            const double sgn = (jt <= nit - nstw) ? -1.0 : 1.0;
            double flr = 0.0, ul = 0.0;
            const double e = s->eps[k], sg = s->sig[k];
            if (s->vdwnum[k] == 1) {
                flr = e * sg * (sg / (10.0 * std::pow(rc, 10)) - 1.0 / (4.0 * std::pow(rc, 4)));
                ul = e * sg * (sg / (90.0 * std::pow(rc, 9)) - 1.0 / (12.0 * rc * rc * rc));
                flr_lja[it - 1] += sgn * xdens[jt - 1] * e * (sg * sg) / 10.0;
                flr_ljc[it - 1] += sgn * xdens[jt - 1] * e * sg / 4.0;
            } else if (s->vdwnum[k] == 2) {
                const double ro = 1.0 / s->rhoi[k];
                flr = ro * (ro + rc) * s->aa[k] * std::exp(-rc / ro) - s->cc[k] / (4.0 * std::pow(rc, 4));
                ul = ro * ro * (2.0 * ro + rc) * s->aa[k] * std::exp(-rc / ro) - s->cc[k] / (12.0 * rc * rc * rc);
                flr_bua[it - 1] += sgn * xdens[jt - 1] * s->aa[k] * ro;
                flr_buc[it - 1] += sgn * xdens[jt - 1] * s->cc[k] / 4.0;
                flr_bur[it - 1] = ro;
            }
            if (sgn < 0.0) {
                flr_l[it - 1] += flr * xdens[jt - 1];
                ulr_l[it - 1] += ul * xdens[jt - 1];
            } else {
                flr_w[it - 1] += flr * xdens[jt - 1];
                ulr_w[it - 1] += ul * xdens[jt - 1];
            }
        }
    }
    for (int k = 0; k < 9 * nit; ++k)
        if (k < 6 * nit || k >= 7 * nit) tab[k] *= 2.0 * kPi;
}

// Self energy (src/forcem.f90:793-822); only reported, never part of uconf.
double self_energy(const mdg_sysdesc* s, const double* x0, const double* y0, const double* z0, double alfa,
                   double facq, double spii) {
    const double A1 = (double)0.254829592f, A2 = (double)-0.284496736f, A3 = (double)1.421413741f,
                 A4 = (double)-1.453152027f, A5 = (double)1.061405429f, P = (double)0.3275911f;
    double sq = 0.0;
    for (int64_t i = 0; i < s->ntota; ++i) sq += s->qs[i] * s->qs[i];
    double u = -0.5 * spii * facq * alfa * sq;
    int64_t ix = 0, ntprev = 0;
    for (int64_t it = 0; it < s->ntype; ++it) {
        if (s->moltypen[it] == 0) {
            const int64_t i0 = ntprev;
            for (int64_t a = i0; a < i0 + s->ns[it]; ++a)
                for (int64_t b = a + 1; b < i0 + s->ns[it]; ++b) {
                    const double dx = x0[a] - x0[b], dy = y0[a] - y0[b], dz = z0[a] - z0[b];
                    const double rij = std::sqrt(dx * dx + dy * dy + dz * dz);
                    const double t = 1.0 / (1.0 + P * alfa * rij), ar = alfa * rij;
                    const double erfv = 1.0 - ((((A5 * t + A4) * t + A3) * t + A2) * t + A1) * t * std::exp(-(ar * ar));
                    u -= (double)s->nt[it] * facq * s->qs[a] * s->qs[b] * erfv / rij;
                }
        } else if (s->moltypen[it] == 2) {
            for (int64_t iq = 0; iq < s->nt[it]; ++iq) {
                ++ix;
                for (int64_t is = 1; is <= s->nconst[it]; ++is) {
                    // constra(ix, is): transposed read of the (SMX, ncons) table, as the reference does
                    const int64_t flat = (ix - 1) + MDG_SMX * (is - 1);
                    if (flat >= MDG_SMX * s->ncons) continue;
                    const int64_t i = s->constra[flat], j = s->constrb[flat];
                    if (i <= 0 || j <= 0) continue;
                    const double rij = s->length[it + s->ntype * (is - 1)];
                    const double t = 1.0 / (1.0 + P * alfa * rij), ar = alfa * rij;
                    const double erfv = 1.0 - ((((A5 * t + A4) * t + A3) * t + A2) * t + A1) * t * std::exp(-(ar * ar));
                    u -= facq * s->qs[i - 1] * s->qs[j - 1] * erfv / rij;
                }
            }
        }
        ntprev = s->nt[it];
    }
    return u;
}

int alloc_lists(Ctx& c, int maxnb, int maxwnb) {
    View& v = c.v;
    dfree(c, v.nb);
    dfree(c, v.wnb);
    v.maxnb = std::max(maxnb, 8);
    v.maxwnb = std::max(maxwnb, 8);
    v.nb = (int*)dalloc(c, sizeof(int) * (size_t)std::max(v.nheads, 1) * v.maxnb);
    v.wnb = (int*)dalloc(c, sizeof(int) * (size_t)std::max(v.nheads, 1) * (v.nwall > 0 ? v.maxwnb : 1));
    if (!v.nb || !v.wnb) return set_err(&c, MDG_E_CUDA, "out of device memory for the neighbour lists");
    return MDG_OK;
}

int sync_check(Ctx& c, const char* where) {
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return set_err(&c, MDG_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
    return MDG_OK;
}

int read_status(Ctx& c) {
    MDG_CUDA(cudaMemcpyAsync(c.h_status, c.v.status, sizeof(int) * ST_NWORDS, cudaMemcpyDeviceToHost, c.stream));
    return sync_check(c, "status");
}

// Debug runs (MDG_DEBUG_SYNC=1 in the environment at mdg_create): synchronise after every
// phase and report the first phase that failed or saw an out-of-range index.
int phase_check(Ctx& c, const char* name) {
    if (!c.debug_sync) return MDG_OK;
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return set_err(&c, MDG_E_CUDA, std::string("phase ") + name + ": " + cudaGetErrorString(e));
    int st[ST_NWORDS];
    cudaMemcpy(st, c.v.status, sizeof(st), cudaMemcpyDeviceToHost);
    if (st[ST_OOB]) {
        char b[160];
        snprintf(b, sizeof b, "phase %s: out-of-range index at site %d", name, st[ST_OOB]);
        return set_err(&c, MDG_E_CUDA, b);
    }
    return MDG_OK;
}

#define PHASE(call, name)                   \
    do {                                    \
        call;                               \
        int prc_ = phase_check(c, name);    \
        if (prc_) return prc_;              \
    } while (0)

// Runs the force phases on device-resident positions.  Returns MDG_OK or an error.
int run_force(Ctx& c, bool force_rebuild) {
    View& v = c.v;
    for (int attempt = 0; attempt < 4; ++attempt) {
        cudaMemsetAsync(v.fx, 0, sizeof(double) * std::max(v.nmove, 1), c.stream);
        cudaMemsetAsync(v.fy, 0, sizeof(double) * std::max(v.nmove, 1), c.stream);
        cudaMemsetAsync(v.fz, 0, sizeof(double) * std::max(v.nmove, 1), c.stream);
        cudaMemsetAsync(v.acc, 0, sizeof(double) * (2 * v.nijt + ACC_NSLOT), c.stream);
        cudaMemsetAsync(v.status, 0, sizeof(int) * 2, c.stream);
        PHASE(nnlist_trigger(c, force_rebuild || attempt > 0), "trigger");
        PHASE(nnlist_build(c), "nnlist");
        PHASE(pair_forces_fp64(c), "pairs");
        PHASE(surf_partition(c), "surf_partition");
        PHASE(wall_forces_fp64(c), "walls");
        PHASE(lr_tail(c), "lr_tail");
        PHASE(recip_fp64(c), "reciprocal");
        PHASE(dipole_correction(c), "dipole");
        PHASE(angle_forces(c), "angles");
        PHASE(force_sum(c, c.d_ft, c.d_fc, c.d_tq), "force_sum");
        int rc = read_status(c);
        if (rc) return rc;
        const int ovf = c.h_status[ST_LIST_OVF], wovf = c.h_status[ST_WLIST_OVF];
        if (!ovf && !wovf) return MDG_OK;
        // the list outgrew its capacity: enlarge and redo this evaluation with a fresh list
        rc = alloc_lists(c, ovf ? ovf + ovf / 4 + 32 : v.maxnb, wovf ? wovf + wovf / 4 + 32 : v.maxwnb);
        if (rc) return rc;
    }
    return set_err(&c, MDG_E_LIST_OVERFLOW, "nnlist_make(): nnlist too big!");
}

}  // namespace
}  // namespace mdg

using namespace mdg;

struct mdg_ctx : Ctx {};

extern "C" {

const char* mdg_last_error(const mdg_ctx* ctx) { return ctx ? ctx->err.c_str() : g_err.c_str(); }

void mdg_destroy(mdg_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (void* p : c->owned)
        if (p) cudaFree(p);
    if (c->h_acc) cudaFreeHost(c->h_acc);
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int mdg_create(const mdg_sysdesc* s, const mdg_params* p, const double* x0, const double* y0, const double* z0,
               const double* cx0, const double* cy0, const double* cz0, mdg_ctx** out) {
    if (!s || !p || !out || !x0 || !y0 || !z0) return set_err(nullptr, MDG_E_ARG, "null argument");
    *out = nullptr;
    if (s->ngogo != s->nmove) return set_err(nullptr, MDG_E_UNSUPPORTED, "Couette-pulled walls (ngogo /= nmove)");
    if (s->nmove != s->nliqa + s->nsurf || s->ntota != s->nmove + s->nwall || s->nriga != 3 * s->nrig ||
        s->nijt != s->nit * (s->nit + 1) / 2 || s->ntype < 1)
        return set_err(nullptr, MDG_E_ARG, "inconsistent system sizes");
    if (s->nrig > 0 && (!cx0 || !cy0 || !cz0)) return set_err(nullptr, MDG_E_ARG, "null centre-of-mass array");
    if (s->ntota >= (1LL << 31)) return set_err(nullptr, MDG_E_UNSUPPORTED, "more than 2^31 atoms");
    for (int64_t k = 0; k < s->nijt; ++k)
        if (s->vdwnum[k] < 0 || s->vdwnum[k] > 2)
            return set_err(nullptr, MDG_E_ARG, "force_real(): unknown interaction type");
    for (int64_t i = 0; i < s->ntota; ++i)
        if (s->itype[i] < 1 || s->itype[i] > s->nit) return set_err(nullptr, MDG_E_ARG, "itype out of range");
    for (int64_t k = 0; k < s->nit * s->nit; ++k)
        if (s->ijtype[k] < 1 || s->ijtype[k] > s->nijt) return set_err(nullptr, MDG_E_ARG, "ijtype out of range");
    for (int64_t t = 0; t < s->nit; ++t)
        if (s->nsi[t] < 0 || s->nsi[t] > MDG_SMX) return set_err(nullptr, MDG_E_ARG, "nsi out of range");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_err(nullptr, MDG_E_CUDA, "no CUDA device");

    mdg_ctx* cp = new mdg_ctx();
    Ctx& c = *cp;
    cudaGetDevice(&c.device);
    c.sysc = *s;
    c.precision = p->precision;
    {
        const char* dbg = getenv("MDG_DEBUG_SYNC");
        c.debug_sync = dbg && dbg[0] == '1';
    }
    c.variant = p->variant;
    c.quirks = p->quirks;
    auto bail = [&](int code) {
        std::string m = c.err;
        mdg_destroy(cp);
        return set_err(nullptr, code, m.empty() ? "mdg_create failed" : m);
    };
    if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) {
        c.err = "cudaStreamCreate failed";
        return bail(MDG_E_CUDA);
    }
    View& v = c.v;
    v.nrig = (int)s->nrig;
    v.nriga = (int)s->nriga;
    v.nliqa = (int)s->nliqa;
    v.nmove = (int)s->nmove;
    v.nwall = (int)s->nwall;
    v.ntota = (int)s->ntota;
    v.nit = (int)s->nit;
    v.nijt = (int)s->nijt;
    v.nltype = (int)s->nltype;
    v.bulk = p->variant == MDG_BULK ? 1 : 0;
    v.pbcz = p->pbc_z_list ? 1 : 0;
    v.lx = s->lx;
    v.ly = s->ly;
    v.lz = s->lz;
    v.lxi = 1.0 / s->lx;
    v.lyi = 1.0 / s->ly;
    v.lzi = 1.0 / s->lz;
    v.lwh = 0.5 * s->lw;
    v.rcut = p->rcut;
    v.rcutsq = p->rcut * p->rcut;
    v.skin = p->skin;
    v.alfa = p->alpha > 0.0 ? p->alpha : (double)3.09f / p->rcut;
    v.spii = 2.0 / std::sqrt(kPi);
    v.facq = kPH_4epi * kPH_e * kPH_e * kPH_Na / (1000.0 * kPH_A2m);
    v.dshsq = p->dshsq;
    double rs = p->rcut + p->skin;
    if (s->nrig > 0) {
        const double dx = x0[0] - cx0[0], dy = y0[0] - cy0[0], dz = z0[0] - cz0[0];
        rs = rs + 2.0 * std::sqrt(dx * dx + dy * dy + dz * dz);
    }
    v.rskinsq = rs * rs;
    c.maxit = p->shake_maxit > 0 ? p->shake_maxit : 10;
    c.tol2 = p->shake_tol2 > 0.0 ? p->shake_tol2 : (double)1.e-8f;
    c.rptol = p->shake_rptol > 0.0 ? p->shake_rptol : (double)0.85f;

    // per-atom and per-type tables
    const int nt = v.ntota, nit = v.nit, nijt = v.nijt;
    std::vector<int> type(nt), nsi(nit), ijt(nit * nit), vdw(nijt);
    for (int i = 0; i < nt; ++i) type[i] = (int)s->itype[i] - 1;
    for (int t = 0; t < nit; ++t) nsi[t] = (int)s->nsi[t];
    for (int a = 0; a < nit; ++a)
        for (int b = 0; b < nit; ++b) ijt[a * nit + b] = (int)s->ijtype[a + nit * b] - 1;
    for (int k = 0; k < nijt; ++k) vdw[k] = (int)s->vdwnum[k];
    std::vector<double> q(s->qs, s->qs + nt), mi(s->mi, s->mi + nt), mii(s->mii, s->mii + nt);
    v.type = upload(c, type);
    v.nsi = upload(c, nsi);
    v.ijt = upload(c, ijt);
    v.vdw = upload(c, vdw);
    v.q = upload(c, q);
    v.mi = upload(c, mi);
    v.mii = upload(c, mii);
    v.eps = upload(c, std::vector<double>(s->eps, s->eps + nijt));
    v.sig = upload(c, std::vector<double>(s->sig, s->sig + nijt));
    v.aa = upload(c, std::vector<double>(s->aa, s->aa + nijt));
    v.rhoi = upload(c, std::vector<double>(s->rhoi, s->rhoi + nijt));
    v.cc = upload(c, std::vector<double>(s->cc, s->cc + nijt));
    c.h_qs_wall.assign(s->qs + v.nmove, s->qs + nt);
    // heads: moving atoms that carry a molecule (nsi /= 0)
    std::vector<int> heads;
    for (int i = 0; i < v.nmove; ++i)
        if (nsi[type[i]] != 0) {
            if (i + nsi[type[i]] > v.nmove || nsi[type[i]] > MDG_SMX) {
                c.err = "head atom with sites beyond nmove";
                return bail(MDG_E_ARG);
            }
            heads.push_back(i);
        }
    v.nheads = (int)heads.size();
    v.head_atom = upload(c, heads);
    // constrained pairs are not candidates (nnlist_constr, src/nnlist.f90:167-208)
    std::vector<std::vector<int>> ex(nt);
    for (int64_t ic = 0; ic < s->ncons; ++ic) {
        const int64_t it = s->ictype[ic] - 1;
        for (int64_t k = 0; k < s->nconst[it]; ++k) {
            const int64_t a = s->constra[k + MDG_SMX * ic] - 1, b = s->constrb[k + MDG_SMX * ic] - 1;
            if (a < 0 || b < 0 || a >= nt || b >= nt) {
                c.err = "constraint atom out of range";
                return bail(MDG_E_ARG);
            }
            ex[a].push_back((int)b);
            ex[b].push_back((int)a);
        }
    }
    std::vector<int> eoff(nt + 1, 0), el;
    for (int i = 0; i < nt; ++i) {
        eoff[i + 1] = eoff[i] + (int)ex[i].size();
        el.insert(el.end(), ex[i].begin(), ex[i].end());
    }
    v.excl_off = upload(c, eoff);
    v.excl = upload(c, el);
    // state arrays
    v.x = upload(c, std::vector<double>(x0, x0 + nt));
    v.y = upload(c, std::vector<double>(y0, y0 + nt));
    v.z = upload(c, std::vector<double>(z0, z0 + nt));
    v.rsx = (double*)dalloc(c, sizeof(double) * std::max(v.nmove, 1));
    v.rsy = (double*)dalloc(c, sizeof(double) * std::max(v.nmove, 1));
    v.rsz = (double*)dalloc(c, sizeof(double) * std::max(v.nmove, 1));
    v.cx = (double*)dalloc(c, sizeof(double) * std::max(v.nrig, 1));
    v.cy = (double*)dalloc(c, sizeof(double) * std::max(v.nrig, 1));
    v.cz = (double*)dalloc(c, sizeof(double) * std::max(v.nrig, 1));
    if (v.nrig > 0) {
        cudaMemcpy(v.cx, cx0, sizeof(double) * v.nrig, cudaMemcpyHostToDevice);
        cudaMemcpy(v.cy, cy0, sizeof(double) * v.nrig, cudaMemcpyHostToDevice);
        cudaMemcpy(v.cz, cz0, sizeof(double) * v.nrig, cudaMemcpyHostToDevice);
    }
    v.ocx = (double*)dalloc(c, sizeof(double) * std::max(v.nrig, 1));
    v.ocy = (double*)dalloc(c, sizeof(double) * std::max(v.nrig, 1));
    v.ocz = (double*)dalloc(c, sizeof(double) * std::max(v.nrig, 1));
    const int nflex = v.nmove - v.nriga;
    v.ox = (double*)dalloc(c, sizeof(double) * std::max(nflex, 1));
    v.oy = (double*)dalloc(c, sizeof(double) * std::max(nflex, 1));
    v.oz = (double*)dalloc(c, sizeof(double) * std::max(nflex, 1));
    v.fx = (double*)dalloc(c, sizeof(double) * std::max(v.nmove, 1));
    v.fy = (double*)dalloc(c, sizeof(double) * std::max(v.nmove, 1));
    v.fz = (double*)dalloc(c, sizeof(double) * std::max(v.nmove, 1));
    v.nbcnt = (int*)dalloc(c, sizeof(int) * std::max(v.nheads, 1));
    v.wnbcnt = (int*)dalloc(c, sizeof(int) * std::max(v.nheads, 1));
    v.acc = (double*)dalloc(c, sizeof(double) * (2 * nijt + ACC_NSLOT));
    v.status = (int*)dalloc(c, sizeof(int) * ST_NWORDS);
    c.d_ft = (double*)dalloc(c, sizeof(double) * 3 * std::max(nflex, 1));
    c.d_fc = (double*)dalloc(c, sizeof(double) * 3 * std::max(v.nrig, 1));
    c.d_tq = (double*)dalloc(c, sizeof(double) * 3 * std::max(v.nrig, 1));
    if (cudaMallocHost(&c.h_acc, sizeof(double) * (2 * nijt + ACC_NSLOT)) != cudaSuccess ||
        cudaMallocHost(&c.h_status, sizeof(int) * ST_NWORDS) != cudaSuccess)
        c.alloc_failed = true;
    if (c.alloc_failed) {
        c.err = "out of device memory";
        return bail(MDG_E_CUDA);
    }
    // LR tables, self energy
    std::vector<double> lr;
    lr_tables(c, s, p->rcut, lr);
    c.d_lr = upload(c, lr);
    c.uself = self_energy(s, x0, y0, z0, v.alfa, v.facq, v.spii);
    int rc = recip_setup(c, p->kmax, x0, y0, z0);
    if (rc) return bail(rc);
    rc = nnlist_setup(c, x0, y0, z0);
    if (rc) return bail(rc);
    rc = shake_setup(c, s);
    if (rc) return bail(rc);
    // angles
    {
        std::vector<int4> terms;
        std::vector<double> kt, th;
        for (int64_t ia = 0; ia < s->nang; ++ia) {
            const int64_t it = s->iatype[ia] - 1;
            for (int64_t k = 0; k < s->nangt[it]; ++k) {
                const int64_t a = s->ang1[k + MDG_SMX * ia] - 1, b = s->ang2[k + MDG_SMX * ia] - 1,
                              d = s->ang3[k + MDG_SMX * ia] - 1;
                if (a < 0 || b < 0 || d < 0 || a >= nt || b >= nt || d >= nt) {
                    c.err = "angle atom out of range";
                    return bail(MDG_E_ARG);
                }
                terms.push_back(make_int4((int)a, (int)b, (int)d, (int)kt.size()));
                kt.push_back(s->kt[it + s->ntype * k]);
                th.push_back(s->theta[it + s->ntype * k]);
            }
        }
        c.nang_terms = (int)terms.size();
        c.d_ang = reinterpret_cast<int*>(upload(c, terms));
        c.d_ang_kt = upload(c, kt);
        c.d_ang_th = upload(c, th);
    }
    c.nfreed = 3 * (s->nmove - s->nliqa);
    for (int64_t it = s->nltype; it < s->ntype; ++it)
        if (s->moltypen[it] == 2) c.nfreed -= s->nt[it] * s->nconst[it];

    // first list: size the capacity from the actual neighbour counts (a capacity given in the
    // parameters is only the starting size; the list never stays truncated)
    {
        const double vol = s->lx * s->ly * s->lz;
        const double sph = 4.0 / 3.0 * kPi * rs * rs * rs;
        const int est = (int)(sph * v.nheads / vol) + 64;
        const bool user = p->list_capacity > 0 || p->wlist_capacity > 0;
        rc = alloc_lists(c, p->list_capacity > 0 ? (int)std::min<int64_t>(p->list_capacity, 1 << 28) : est,
                         p->wlist_capacity > 0 ? (int)std::min<int64_t>(p->wlist_capacity, 1 << 28) : 2 * est);
        if (rc) return bail(rc);
        cudaMemsetAsync(v.acc, 0, sizeof(double) * (2 * nijt + ACC_NSLOT), c.stream);
        for (int attempt = 0;; ++attempt) {
            cudaMemsetAsync(v.status, 0, sizeof(int) * ST_NWORDS, c.stream);
            nnlist_trigger(c, true);
            nnlist_build(c);
            rc = read_status(c);
            if (rc) return bail(rc);
            std::vector<int> cnt(std::max(v.nheads, 1)), wcnt(std::max(v.nheads, 1));
            cudaMemcpy(cnt.data(), v.nbcnt, sizeof(int) * std::max(v.nheads, 1), cudaMemcpyDeviceToHost);
            cudaMemcpy(wcnt.data(), v.wnbcnt, sizeof(int) * std::max(v.nheads, 1), cudaMemcpyDeviceToHost);
            const int mx = std::max(*std::max_element(cnt.begin(), cnt.end()), c.h_status[ST_LIST_OVF]);
            const int mw = std::max(*std::max_element(wcnt.begin(), wcnt.end()), c.h_status[ST_WLIST_OVF]);
            const bool ovf = c.h_status[ST_LIST_OVF] || c.h_status[ST_WLIST_OVF];
            const int want = mx + mx / 3 + 32, wwant = mw + mw / 3 + 32;
            const bool roomy = want <= v.maxnb && (v.nwall == 0 || wwant <= v.maxwnb);
            if (!ovf && (user || roomy)) break;
            if (attempt >= 4) {
                c.err = "nnlist_init(): could not size the neighbour list";
                return bail(MDG_E_LIST_OVERFLOW);
            }
            rc = alloc_lists(c, std::max(want, v.maxnb), std::max(wwant, v.maxwnb));
            if (rc) return bail(rc);
        }
    }
    rc = sync_check(c, "mdg_create");
    if (rc) return bail(rc);
    *out = cp;
    return MDG_OK;
}

int mdg_nnlist_make(mdg_ctx* cp, const double* x0, const double* y0, const double* z0, const double* cx0,
                    const double* cy0, const double* cz0, int64_t* ipack, int64_t* wpack) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    View& v = c.v;
    MDG_CUDA(cudaMemcpyAsync(v.x, x0, sizeof(double) * v.nmove, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(v.y, y0, sizeof(double) * v.nmove, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(v.z, z0, sizeof(double) * v.nmove, cudaMemcpyHostToDevice, c.stream));
    if (v.nrig > 0) {
        MDG_CUDA(cudaMemcpyAsync(v.cx, cx0, sizeof(double) * v.nrig, cudaMemcpyHostToDevice, c.stream));
        MDG_CUDA(cudaMemcpyAsync(v.cy, cy0, sizeof(double) * v.nrig, cudaMemcpyHostToDevice, c.stream));
        MDG_CUDA(cudaMemcpyAsync(v.cz, cz0, sizeof(double) * v.nrig, cudaMemcpyHostToDevice, c.stream));
    }
    for (int attempt = 0; attempt < 4; ++attempt) {
        cudaMemsetAsync(v.status, 0, sizeof(int) * 2, c.stream);
        nnlist_trigger(c, true);
        nnlist_build(c);
        int rc = read_status(c);
        if (rc) return rc;
        const int ovf = c.h_status[ST_LIST_OVF], wovf = c.h_status[ST_WLIST_OVF];
        if (!ovf && !wovf) break;
        rc = alloc_lists(c, ovf ? ovf + ovf / 4 + 32 : v.maxnb, wovf ? wovf + wovf / 4 + 32 : v.maxwnb);
        if (rc) return rc;
        if (attempt == 3) return set_err(&c, MDG_E_LIST_OVERFLOW, "nnlist_make(): nnlist too big!");
    }
    return mdg_get_lists(cp, nullptr, nullptr, 0, nullptr, nullptr, 0, ipack, wpack);
}

int mdg_get_lists(mdg_ctx* cp, int64_t* li, int64_t* lj, int64_t cap, int64_t* wi, int64_t* wj, int64_t wcap,
                  int64_t* ipack, int64_t* wpack) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    View& v = c.v;
    const int nh = std::max(v.nheads, 1);
    std::vector<int> cnt(nh, 0), wcnt(nh, 0), heads(nh, 0);
    MDG_CUDA(cudaMemcpy(cnt.data(), v.nbcnt, sizeof(int) * nh, cudaMemcpyDeviceToHost));
    MDG_CUDA(cudaMemcpy(wcnt.data(), v.wnbcnt, sizeof(int) * nh, cudaMemcpyDeviceToHost));
    MDG_CUDA(cudaMemcpy(heads.data(), v.head_atom, sizeof(int) * nh, cudaMemcpyDeviceToHost));
    int64_t n = 0, nw = 0;
    for (int h = 0; h < v.nheads; ++h) {
        n += cnt[h];
        nw += wcnt[h];
    }
    if (ipack) *ipack = n;
    if (wpack) *wpack = nw;
    if (li && lj && cap > 0) {
        std::vector<int> nb((size_t)nh * v.maxnb);
        MDG_CUDA(cudaMemcpy(nb.data(), v.nb, sizeof(int) * nb.size(), cudaMemcpyDeviceToHost));
        int64_t k = 0;
        for (int h = 0; h < v.nheads && k < cap; ++h)
            for (int t = 0; t < cnt[h] && k < cap; ++t, ++k) {
                li[k] = heads[h] + 1;
                lj[k] = nb[(size_t)h * v.maxnb + t] + 1;
            }
    }
    if (wi && wj && wcap > 0 && v.nwall > 0) {
        std::vector<int> nb((size_t)nh * v.maxwnb);
        MDG_CUDA(cudaMemcpy(nb.data(), v.wnb, sizeof(int) * nb.size(), cudaMemcpyDeviceToHost));
        int64_t k = 0;
        for (int h = 0; h < v.nheads && k < wcap; ++h)
            for (int t = 0; t < wcnt[h] && k < wcap; ++t, ++k) {
                wi[k] = heads[h] + 1;
                wj[k] = nb[(size_t)h * v.maxwnb + t] + 1;
            }
    }
    return MDG_OK;
}

int mdg_force_get(mdg_ctx* cp, const double* x0, const double* y0, const double* z0, const double* cx0,
                  const double* cy0, const double* cz0, double* rsx, double* rsy, double* rsz, double* ftx,
                  double* fty, double* ftz, double* fcx, double* fcy, double* fcz, double* tx, double* ty,
                  double* tz, double* fx, double* fy, double* fz, mdg_energies* e) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    View& v = c.v;
    const int nm = v.nmove, nrig = v.nrig, nflex = v.nmove - v.nriga;
    if (!x0 || !y0 || !z0 || !rsx || !rsy || !rsz) return set_err(&c, MDG_E_ARG, "null position array");
    MDG_CUDA(cudaMemcpyAsync(v.x, x0, sizeof(double) * nm, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(v.y, y0, sizeof(double) * nm, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(v.z, z0, sizeof(double) * nm, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(v.rsx, rsx, sizeof(double) * nm, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(v.rsy, rsy, sizeof(double) * nm, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(v.rsz, rsz, sizeof(double) * nm, cudaMemcpyHostToDevice, c.stream));
    if (nrig > 0) {
        MDG_CUDA(cudaMemcpyAsync(v.cx, cx0, sizeof(double) * nrig, cudaMemcpyHostToDevice, c.stream));
        MDG_CUDA(cudaMemcpyAsync(v.cy, cy0, sizeof(double) * nrig, cudaMemcpyHostToDevice, c.stream));
        MDG_CUDA(cudaMemcpyAsync(v.cz, cz0, sizeof(double) * nrig, cudaMemcpyHostToDevice, c.stream));
    }
    int rc = run_force(c, false);
    if (rc) return rc;
    if (ftx && nflex > 0) {
        MDG_CUDA(cudaMemcpyAsync(ftx, c.d_ft, sizeof(double) * nflex, cudaMemcpyDeviceToHost, c.stream));
        MDG_CUDA(cudaMemcpyAsync(fty, c.d_ft + nflex, sizeof(double) * nflex, cudaMemcpyDeviceToHost, c.stream));
        MDG_CUDA(cudaMemcpyAsync(ftz, c.d_ft + 2 * nflex, sizeof(double) * nflex, cudaMemcpyDeviceToHost, c.stream));
    }
    if (nrig > 0) {
        if (fcx) {
            MDG_CUDA(cudaMemcpyAsync(fcx, c.d_fc, sizeof(double) * nrig, cudaMemcpyDeviceToHost, c.stream));
            MDG_CUDA(cudaMemcpyAsync(fcy, c.d_fc + nrig, sizeof(double) * nrig, cudaMemcpyDeviceToHost, c.stream));
            MDG_CUDA(cudaMemcpyAsync(fcz, c.d_fc + 2 * nrig, sizeof(double) * nrig, cudaMemcpyDeviceToHost, c.stream));
        }
        if (tx) {
            MDG_CUDA(cudaMemcpyAsync(tx, c.d_tq, sizeof(double) * nrig, cudaMemcpyDeviceToHost, c.stream));
            MDG_CUDA(cudaMemcpyAsync(ty, c.d_tq + nrig, sizeof(double) * nrig, cudaMemcpyDeviceToHost, c.stream));
            MDG_CUDA(cudaMemcpyAsync(tz, c.d_tq + 2 * nrig, sizeof(double) * nrig, cudaMemcpyDeviceToHost, c.stream));
        }
        MDG_CUDA(cudaMemcpyAsync(rsx, v.rsx, sizeof(double) * 3, cudaMemcpyDeviceToHost, c.stream));
        MDG_CUDA(cudaMemcpyAsync(rsy, v.rsy, sizeof(double) * 3, cudaMemcpyDeviceToHost, c.stream));
        MDG_CUDA(cudaMemcpyAsync(rsz, v.rsz, sizeof(double) * 3, cudaMemcpyDeviceToHost, c.stream));
    }
    if (fx) {
        MDG_CUDA(cudaMemcpyAsync(fx, v.fx, sizeof(double) * nm, cudaMemcpyDeviceToHost, c.stream));
        MDG_CUDA(cudaMemcpyAsync(fy, v.fy, sizeof(double) * nm, cudaMemcpyDeviceToHost, c.stream));
        MDG_CUDA(cudaMemcpyAsync(fz, v.fz, sizeof(double) * nm, cudaMemcpyDeviceToHost, c.stream));
    }
    const int nacc = 2 * v.nijt + ACC_NSLOT;
    MDG_CUDA(cudaMemcpyAsync(c.h_acc, v.acc, sizeof(double) * nacc, cudaMemcpyDeviceToHost, c.stream));
    rc = sync_check(c, "mdg_force_get");
    if (rc) return rc;
    const double* a = c.h_acc;
    const double* sl = a + 2 * v.nijt;
    double sumlj = 0.0, sumqq = 0.0;
    for (int k = 0; k < v.nijt; ++k) {
        sumlj += a[k];
        sumqq += a[v.nijt + k];
    }
    const double uewa = 0.5 * sl[ACC_UEWA];
    const double ewqLL = 0.5 * sl[ACC_EWQLL];
    const double ulr = c.variant == MDG_SLAB ? sl[ACC_ULR] : 0.0;
    double urf = 0.0;
    if (c.variant == MDG_SLAB) {
        const double crf = -2.0 * kPi * v.lzi * v.lxi * v.lyi;
        urf = -crf * v.facq * sl[ACC_DIPZ] * sl[ACC_DIPZ];
    }
    if (!std::isfinite(sumlj) || !std::isfinite(sumqq) || !std::isfinite(uewa))
        return set_err(&c, MDG_E_NAN, "non-finite energy");
    if (e) {
        if (e->elj)
            for (int k = 0; k < v.nijt; ++k) e->elj[k] = a[k];
        if (e->eqq)
            for (int k = 0; k < v.nijt; ++k) e->eqq[k] = a[v.nijt + k];
        e->uewa = uewa;
        e->urf = urf;
        e->ulr = ulr;
        e->uself = c.uself;
        e->uconf = (sumlj + sumqq + uewa + c.uself + urf) - c.uself;
        e->uavex = sumlj + sumqq + ulr + uewa + urf;
        e->vir = 0.0;
        e->ewqLL = ewqLL;
        e->ewqWW = c.ewqWW;
        e->ewqWL = uewa - c.ewqWW - ewqLL;
        for (int k = 0; k < 3; ++k) {
            e->fwsx[k] = sl[ACC_FWS + k];
            e->fwsy[k] = sl[ACC_FWS + 3 + k];
            e->fwsz[k] = sl[ACC_FWS + 6 + k];
        }
        e->fwsx[1] = sl[ACC_FWS0 + 0];
        e->fwsy[1] = sl[ACC_FWS0 + 1];
        e->fwsz[1] = sl[ACC_FWS0 + 2];
        e->press = (e->fwsz[2] - e->fwsz[0]) / (2.0 * v.lx * v.ly) * 1000.0 / (kPH_Na * (double)1e-30f) *
                   (double)1e-5f;
    }
    return MDG_OK;
}

int mdg_shake(mdg_ctx* cp, double* x0, double* y0, double* z0, double* xold, double* yold, double* zold,
              const double* ftx, const double* fty, const double* ftz, double* kps, double* tkps, int32_t* sweeps) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    View& v = c.v;
    const int nl = v.nliqa, ns = v.nmove - v.nliqa, nold = v.ntota - v.nliqa, nflex = v.nmove - v.nriga;
    if (ns <= 0) return MDG_OK;
    MDG_CUDA(cudaMemcpyAsync(v.x + nl, x0 + nl, sizeof(double) * ns, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(v.y + nl, y0 + nl, sizeof(double) * ns, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(v.z + nl, z0 + nl, sizeof(double) * ns, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(c.d_xold, xold, sizeof(double) * nold, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(c.d_yold, yold, sizeof(double) * nold, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(c.d_zold, zold, sizeof(double) * nold, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(c.d_ft_in, ftx, sizeof(double) * nflex, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(c.d_ft_in + nflex, fty, sizeof(double) * nflex, cudaMemcpyHostToDevice, c.stream));
    MDG_CUDA(cudaMemcpyAsync(c.d_ft_in + 2 * nflex, ftz, sizeof(double) * nflex, cudaMemcpyHostToDevice, c.stream));
    cudaMemsetAsync(v.status + ST_SHAKE_MAXIT, 0, sizeof(int) * 2, c.stream);
    shake_launch(c);
    MDG_CUDA(cudaMemcpyAsync(x0 + nl, v.x + nl, sizeof(double) * ns, cudaMemcpyDeviceToHost, c.stream));
    MDG_CUDA(cudaMemcpyAsync(y0 + nl, v.y + nl, sizeof(double) * ns, cudaMemcpyDeviceToHost, c.stream));
    MDG_CUDA(cudaMemcpyAsync(z0 + nl, v.z + nl, sizeof(double) * ns, cudaMemcpyDeviceToHost, c.stream));
    MDG_CUDA(cudaMemcpyAsync(xold, c.d_xold, sizeof(double) * nold, cudaMemcpyDeviceToHost, c.stream));
    MDG_CUDA(cudaMemcpyAsync(yold, c.d_yold, sizeof(double) * nold, cudaMemcpyDeviceToHost, c.stream));
    MDG_CUDA(cudaMemcpyAsync(zold, c.d_zold, sizeof(double) * nold, cudaMemcpyDeviceToHost, c.stream));
    std::vector<double> hk(std::max(v.nit, 1));
    int sw[2] = {0, 1};
    MDG_CUDA(cudaMemcpyAsync(hk.data(), c.d_kps, sizeof(double) * v.nit, cudaMemcpyDeviceToHost, c.stream));
    if (c.ncons > 0) MDG_CUDA(cudaMemcpyAsync(sw, c.d_sweeps, sizeof(sw), cudaMemcpyDeviceToHost, c.stream));
    int rc = read_status(c);
    if (rc) return rc;
    double ks = 0.0;
    for (int t = 0; t < v.nit; ++t) {
        ks += hk[t];
        if (kps) kps[t] = hk[t];
    }
    if (tkps) *tkps = c.nfreed > 0 ? ks * 1000.0 / ((double)8.31441f * (double)(float)c.nfreed) : 0.0;
    if (sweeps) *sweeps = sw[0];
    if (c.h_status[ST_SHAKE_RPTOL]) {
        const int code = c.h_status[ST_SHAKE_RPTOL] - 1;
        char b[128];
        snprintf(b, sizeof b, "Constraint failure: molecule %d", code / 8 + 1);
        return set_err(&c, MDG_E_SHAKE_RPTOL, b);
    }
    if (c.ncons > 0 && !sw[1]) return set_err(&c, MDG_E_SHAKE_MAXIT, "shake(): Too many constraint iterations!");
    return MDG_OK;
}

}  // extern "C"
