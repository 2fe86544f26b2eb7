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
    drop_graphs(c);
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
    int rc = sync_check(c, "status");
    if (rc) return rc;
    if (c.h_status[ST_TC_TIMEOUT]) {
        char b[128];
        snprintf(b, sizeof b, "tensor-core reciprocal phase timed out waiting (site %d)", c.h_status[ST_TC_TIMEOUT]);
        return set_err(&c, MDG_E_CUDA, b);
    }
    return MDG_OK;
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

// The mixed form ends in one kernel that merges the force parts and does force_sum, when no bend
// angles or histograms need the merged site forces first.
static bool merge_fusable(const Ctx& c) {
    return c.precision == MDG_MIXED && c.nang_terms == 0 && !(c.meas.init && c.meas.force_hist);
}

// Queues the force phases on device-resident positions (no synchronisation).  acc_clear: the
// energy sums were zeroed by the kernel before (the predictor of a resident step).  In the mixed
// form the packing kernel clears them (and the overflow words), which keeps memset nodes, slow
// to start inside a graph, off the critical path.  defer_merge: leave that final merge kernel to
// the caller (the resident step fuses it into the corrector).  packed: the records were written by
// the kernel before (the predictor of a resident step), so the packing kernel is left out.
// batch_stage (replica batches in phase order, mixed form with walls and no surface atoms): 1 stops
// after the rebuild decision with the list build and the head-head and head-wall loops left to the
// batch's kernels, 2 goes on from there (0: the whole evaluation).
static bool batch_phased(const Ctx& c) {
    const View& v = c.v;
    return c.precision == MDG_MIXED && v.nliqa == v.nmove && v.nwall > 0 && v.nheads > 0;
}

int launch_force(Ctx& c, bool force_rebuild, bool reset_status, bool acc_clear = false, bool defer_merge = false,
                 bool packed = false) {
    View& v = c.v;
    const bool hist = c.meas.init && c.meas.force_hist;
    const bool fused = merge_fusable(c);
    if (c.precision != MDG_MIXED) {
        if (!acc_clear) cudaMemsetAsync(v.acc, 0, sizeof(double) * (2 * v.nijt + ACC_NSLOT), c.stream);
        if (reset_status) cudaMemsetAsync(v.status, 0, sizeof(int) * 2, c.stream);
    }
    if (c.precision == MDG_MIXED && c.batch_stage != 2) {
        // The tensor-core reciprocal sum needs only the packed atom records: it runs on a side
        // stream while the main stream does the list, the real-space loops and the wall tail.
        // Without surface atoms (whose z forces after the head-head loop are booked to the walls,
        // src/forcem.f90:408-413) the head-wall loop runs on a third stream beside the head-head
        // loop; both add into F with vector reductions.  Fork and join go through events, so the
        // same dependencies hold inside a captured graph.  The reciprocal forces (d_frc), F and the
        // slab dipole term join the FP64 forces in one merge at the end.
        if (!packed) PHASE(pack_mixed(c, force_rebuild, reset_status, true), "pack");
        const cudaStream_t s0 = c.stream;
        MDG_CUDA(cudaEventRecord(c.ev_fork, s0));
        MDG_CUDA(cudaStreamWaitEvent(c.side, c.ev_fork, 0));
        c.stream = c.side;
        recip_tc(c);
        c.stream = s0;
        MDG_CUDA(cudaEventRecord(c.ev_join, c.side));
        // the packing's close (dipole, rebuild decision) runs here, ahead of the list it decides
        if (packed) step_close_launch(c);
        else pack_close_launch(c);
        const bool conc = v.nliqa == v.nmove && v.nwall > 0 && v.nheads > 0;
        if (conc) {
            // third branch: the wall tail (positions only) while the list is checked and rebuilt,
            // then the head-wall loop once the list is there
            MDG_CUDA(cudaStreamWaitEvent(c.side2, c.ev_fork, 0));
            c.stream = c.side2;
            lr_tail(c);
            c.stream = s0;
        }
        if (conc && c.batch_stage == 1) {
            // the list build and the loops run in the batch's kernels once every system has its
            // rebuild decision
            MDG_CUDA(cudaEventRecord(c.ev_join2, c.side2));
            MDG_CUDA(cudaStreamWaitEvent(s0, c.ev_join2, 0));
            return MDG_OK;
        }
        PHASE(nnlist_build(c), "nnlist");
        if (conc) {
            MDG_CUDA(cudaEventRecord(c.ev_list, s0));
            MDG_CUDA(cudaStreamWaitEvent(c.side2, c.ev_list, 0));
            c.stream = c.side2;
            walls_mixed(c, true);
            c.stream = s0;
            MDG_CUDA(cudaEventRecord(c.ev_join2, c.side2));
            PHASE(pairs_mixed(c, false), "pairs");
            MDG_CUDA(cudaStreamWaitEvent(s0, c.ev_join2, 0));
        } else {
            PHASE(pairs_mixed(c, true), "pairs");
            PHASE(surf_partition(c), "surf_partition");
            PHASE(walls_mixed(c), "walls");
            PHASE(lr_tail(c), "lr_tail");
        }
    }
    if (c.precision == MDG_MIXED) {
        MDG_CUDA(cudaStreamWaitEvent(c.stream, c.ev_join, 0));
        if (fused) {
            if (!defer_merge) PHASE(merge_force_sum(c, c.d_frc), "merge + force_sum");
        } else {
            PHASE(merge_mixed(c, c.d_frc, true), "merge");
        }
    } else {
        cudaMemsetAsync(v.fx, 0, sizeof(double) * std::max(v.nmove, 1), c.stream);
        cudaMemsetAsync(v.fy, 0, sizeof(double) * std::max(v.nmove, 1), c.stream);
        cudaMemsetAsync(v.fz, 0, sizeof(double) * std::max(v.nmove, 1), c.stream);
        PHASE(nnlist_trigger(c, force_rebuild), "trigger");
        PHASE(nnlist_build(c), "nnlist");
        PHASE(pair_forces_fp64(c), "pairs");
        PHASE(surf_partition(c), "surf_partition");
        PHASE(wall_forces_fp64(c), "walls");
        PHASE(lr_tail(c), "lr_tail");
        PHASE(recip_fp64(c), "reciprocal");
        PHASE(dipole_correction(c), "dipole");
    }
    if (hist) {
        measure_force_real(c);
        measure_force_fouri(c);
    }
    if (!fused) {
        PHASE(angle_forces(c), "angles");
        if (hist) measure_force_intra(c);
        PHASE(force_sum(c, c.d_ft, c.d_fc, c.d_tq), "force_sum");
    }
    if (hist) measure_force_sum(c);
    return MDG_OK;
}

// Runs the force phases and checks the list capacity; regrows and redoes on overflow.
int run_force(Ctx& c, bool force_rebuild) {
    View& v = c.v;
    for (int attempt = 0; attempt < 4; ++attempt) {
        int rc = launch_force(c, force_rebuild || attempt > 0, true);
        if (rc) return rc;
        rc = read_status(c);
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

extern "C" {

const char* mdg_last_error(const mdg_ctx* ctx) { return ctx ? ctx->err.c_str() : g_err.c_str(); }

void mdg_destroy(mdg_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->side) cudaStreamSynchronize(c->side);
    if (c->side2) cudaStreamSynchronize(c->side2);
    for (void* p : c->owned)
        if (p) cudaFree(p);
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    if (c->force_exec) cudaGraphExecDestroy(c->force_exec);
    if (c->h_acc) cudaFreeHost(c->h_acc);
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->h_small) cudaFreeHost(c->h_small);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    else if (c->stream) cudaStreamDestroy(c->stream);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->side2) cudaStreamDestroy(c->side2);
    for (cudaEvent_t e : {c->ev_fork, c->ev_join, c->ev_fork2, c->ev_join2, c->ev_list})
        if (e) cudaEventDestroy(e);
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
    c.h_moltypen.assign(s->moltypen, s->moltypen + s->ntype);
    c.h_nt.assign(s->nt, s->nt + s->ntype);
    c.h_ns.assign(s->ns, s->ns + s->ntype);
    c.h_itype.assign(s->itype, s->itype + s->ntota);
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
    // The reciprocal branch is the longest of a force evaluation: its stream gets the highest
    // priority, so that its kernels' blocks are placed first when the real-space loops fill the
    // SMs (graphs are instantiated to keep the priority of the stream each node was captured on).
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithPriority(&c.side, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c.side2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c.ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c.ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c.ev_fork2, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c.ev_join2, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c.ev_list, cudaEventDisableTiming) != cudaSuccess) {
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
        cudaMallocHost(&c.h_status, sizeof(int) * ST_NWORDS) != cudaSuccess ||
        cudaMallocHost(&c.h_small, sizeof(double) * (std::max(v.nit, 1) + 1)) != cudaSuccess)
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
    if (c.precision == MDG_MIXED) {
        rc = recip_tc_setup(c);
        if (rc) return bail(rc);
        pack_setup(c);
        c.pk.tc = c.d_tc_atoms;
        c.pk.cmax = c.d_tc_cmax;
        std::vector<float> parf(6 * (size_t)std::max<int64_t>(nijt, 1), 0.f);
        for (int64_t k = 0; k < nijt; ++k) {
            int bits = (int)s->vdwnum[k];
            std::memcpy(&parf[6 * k + 0], &bits, 4);
            parf[6 * k + 1] = (float)s->sig[k];
            parf[6 * k + 2] = (float)s->eps[k];
            parf[6 * k + 3] = (float)s->aa[k];
            parf[6 * k + 4] = (float)s->rhoi[k];
            parf[6 * k + 5] = (float)s->cc[k];
        }
        c.pk.par = upload(c, parf);
    }
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
                c.h_ang_mt.push_back((int)it);
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

// k set of the context (src/forcem.f90:743-776): kl, km, kn per valid k in the reference's order and
// Ak; returns the number of k vectors, or a negative error code.
int64_t mdg_kvectors(mdg_ctx* cp, int32_t* kl, int32_t* km, int32_t* kn, double* ak, int64_t cap) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    const KSet& ks = c.ks;
    const int64_t n = std::min<int64_t>(ks.nk, std::max<int64_t>(cap, 0));
    if (n > 0 && (kl || km || kn)) {
        std::vector<int3> kv((size_t)n);
        MDG_CUDA(cudaMemcpy(kv.data(), ks.kvec, sizeof(int3) * n, cudaMemcpyDeviceToHost));
        for (int64_t k = 0; k < n; ++k) {
            if (kl) kl[k] = kv[k].x;
            if (km) km[k] = kv[k].y;
            if (kn) kn[k] = kv[k].z;
        }
    }
    if (n > 0 && ak) MDG_CUDA(cudaMemcpy(ak, ks.ak, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return ks.nk;
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
    if (nrig > 0 && (!cx0 || !cy0 || !cz0)) return set_err(&c, MDG_E_ARG, "null centre array");
    // inputs: pinned host arrays through one gather kernel, others by copy
    IoBatch io;
    MDG_CUDA(io_add(c, io, v.x, x0, nm, true));
    MDG_CUDA(io_add(c, io, v.y, y0, nm, true));
    MDG_CUDA(io_add(c, io, v.z, z0, nm, true));
    MDG_CUDA(io_add(c, io, v.rsx, rsx, nm, true));
    MDG_CUDA(io_add(c, io, v.rsy, rsy, nm, true));
    MDG_CUDA(io_add(c, io, v.rsz, rsz, nm, true));
    if (nrig > 0) {
        MDG_CUDA(io_add(c, io, v.cx, cx0, nrig, true));
        MDG_CUDA(io_add(c, io, v.cy, cy0, nrig, true));
        MDG_CUDA(io_add(c, io, v.cz, cz0, nrig, true));
    }
    io_flush(c, io);
    // The force phases run as one captured graph (launched per call; host launch cost of one
    // graph instead of ~20 kernels), and the results are queued right behind it with the status
    // words, so the call waits once.  A list overflow (rare: the capacity grows at create) is
    // handled afterwards by regrowing and redoing the evaluation the eager way.
    int rc;
    bool graph_ok = false;
    if (!c.debug_sync) {
        if (!c.force_exec) {
            cudaGraph_t g;
            MDG_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
            rc = launch_force(c, false, true);
            const cudaError_t ce = cudaStreamEndCapture(c.stream, &g);
            if (rc) return rc;
            if (ce != cudaSuccess) return set_err(&c, MDG_E_CUDA, std::string("force graph capture: ") + cudaGetErrorString(ce));
            const cudaError_t ie = cudaGraphInstantiate(&c.force_exec, g, cudaGraphInstantiateFlagUseNodePriority);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess) return set_err(&c, MDG_E_CUDA, std::string("force graph: ") + cudaGetErrorString(ie));
        }
        MDG_CUDA(cudaGraphLaunch(c.force_exec, c.stream));
        graph_ok = true;
    } else {
        rc = run_force(c, false);
        if (rc) return rc;
    }
    for (int pass = 0; pass < 2; ++pass) {
    // results and the status words, one scatter kernel for the pinned ones
    if (ftx && nflex > 0) {
        MDG_CUDA(io_add(c, io, ftx, c.d_ft, nflex, false));
        MDG_CUDA(io_add(c, io, fty, c.d_ft + nflex, nflex, false));
        MDG_CUDA(io_add(c, io, ftz, c.d_ft + 2 * nflex, nflex, false));
    }
    if (nrig > 0) {
        if (fcx) {
            MDG_CUDA(io_add(c, io, fcx, c.d_fc, nrig, false));
            MDG_CUDA(io_add(c, io, fcy, c.d_fc + nrig, nrig, false));
            MDG_CUDA(io_add(c, io, fcz, c.d_fc + 2 * nrig, nrig, false));
        }
        if (tx) {
            MDG_CUDA(io_add(c, io, tx, c.d_tq, nrig, false));
            MDG_CUDA(io_add(c, io, ty, c.d_tq + nrig, nrig, false));
            MDG_CUDA(io_add(c, io, tz, c.d_tq + 2 * nrig, nrig, false));
        }
        MDG_CUDA(io_add(c, io, rsx, v.rsx, 3, false));
        MDG_CUDA(io_add(c, io, rsy, v.rsy, 3, false));
        MDG_CUDA(io_add(c, io, rsz, v.rsz, 3, false));
    }
    if (fx) {
        MDG_CUDA(io_add(c, io, fx, v.fx, nm, false));
        MDG_CUDA(io_add(c, io, fy, v.fy, nm, false));
        MDG_CUDA(io_add(c, io, fz, v.fz, nm, false));
    }
    const int nacc = 2 * v.nijt + ACC_NSLOT;
    MDG_CUDA(io_add(c, io, c.h_acc, v.acc, nacc, false));
    static_assert(ST_NWORDS % 2 == 0, "status words move as 8-byte pairs");
    MDG_CUDA(io_add(c, io, c.h_status, v.status, ST_NWORDS / 2, false));
    io_flush(c, io);
    rc = sync_check(c, "mdg_force_get");
    if (rc) return rc;
    if (!graph_ok || pass == 1) break;
    // status of the graph's evaluation (read_status's checks, on the copy queued above)
    if (c.h_status[ST_TC_TIMEOUT]) {
        rc = read_status(c);
        if (rc) return rc;
    }
    if (!c.h_status[ST_LIST_OVF] && !c.h_status[ST_WLIST_OVF]) break;
    rc = alloc_lists(c, c.h_status[ST_LIST_OVF] ? c.h_status[ST_LIST_OVF] + c.h_status[ST_LIST_OVF] / 4 + 32 : v.maxnb,
                     c.h_status[ST_WLIST_OVF] ? c.h_status[ST_WLIST_OVF] + c.h_status[ST_WLIST_OVF] / 4 + 32 : v.maxwnb);
    if (rc) return rc;
    rc = run_force(c, true);
    if (rc) return rc;
    }
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
    if (!x0 || !y0 || !z0 || !xold || !yold || !zold || !ftx || !fty || !ftz)
        return set_err(&c, MDG_E_ARG, "null array");
    IoBatch io;  // pinned host arrays move through one gather and one scatter kernel
    MDG_CUDA(io_add(c, io, v.x + nl, x0 + nl, ns, true));
    MDG_CUDA(io_add(c, io, v.y + nl, y0 + nl, ns, true));
    MDG_CUDA(io_add(c, io, v.z + nl, z0 + nl, ns, true));
    MDG_CUDA(io_add(c, io, c.d_xold, xold, nold, true));
    MDG_CUDA(io_add(c, io, c.d_yold, yold, nold, true));
    MDG_CUDA(io_add(c, io, c.d_zold, zold, nold, true));
    MDG_CUDA(io_add(c, io, c.d_ft_in, ftx, nflex, true));
    MDG_CUDA(io_add(c, io, c.d_ft_in + nflex, fty, nflex, true));
    MDG_CUDA(io_add(c, io, c.d_ft_in + 2 * nflex, ftz, nflex, true));
    io_flush(c, io);
    cudaMemsetAsync(v.status + ST_SHAKE_MAXIT, 0, sizeof(int) * 2, c.stream);
    shake_launch(c, c.d_ft_in);
    MDG_CUDA(io_add(c, io, x0 + nl, v.x + nl, ns, false));
    MDG_CUDA(io_add(c, io, y0 + nl, v.y + nl, ns, false));
    MDG_CUDA(io_add(c, io, z0 + nl, v.z + nl, ns, false));
    MDG_CUDA(io_add(c, io, xold, c.d_xold, nold, false));
    MDG_CUDA(io_add(c, io, yold, c.d_yold, nold, false));
    MDG_CUDA(io_add(c, io, zold, c.d_zold, nold, false));
    double* hk = c.h_small;
    int* sw = reinterpret_cast<int*>(c.h_small + std::max(v.nit, 1));
    sw[0] = 0;
    sw[1] = 1;
    MDG_CUDA(io_add(c, io, hk, c.d_kps, v.nit, false));
    if (c.ncons > 0) MDG_CUDA(io_add(c, io, sw, c.d_sweeps, 1, false));  // two int words
    MDG_CUDA(io_add(c, io, c.h_status, v.status, ST_NWORDS / 2, false));
    io_flush(c, io);
    int rc = sync_check(c, "mdg_shake");
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

int mdg_pin_host(void* p, int64_t bytes) {
    if (!p || bytes <= 0) return set_err(nullptr, MDG_E_ARG, "mdg_pin_host: null pointer or empty range");
    const cudaError_t e = pin_host_range(p, (size_t)bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(nullptr, MDG_E_CUDA, std::string("mdg_pin_host: ") + cudaGetErrorString(e));
    }
    return MDG_OK;
}

int mdg_unpin_host(void* p) {
    if (!p) return set_err(nullptr, MDG_E_ARG, "mdg_unpin_host: null pointer");
    const cudaError_t e = unpin_host_range(p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(nullptr, MDG_E_CUDA, std::string("mdg_unpin_host: ") + cudaGetErrorString(e));
    }
    return MDG_OK;
}

// ---------------------------------------------------------------------------------------------
// Resident mode
// ---------------------------------------------------------------------------------------------
static int resident_alloc_impl(Ctx& c) {
    if (c.d_thermo) return MDG_OK;
    View& v = c.v;
    const int nion = std::max(v.nliqa - v.nriga, 1), nr = std::max(v.nrig, 1);
    c.d_xd = (double*)dalloc(c, sizeof(double) * 12 * nion);
    c.d_c = (double*)dalloc(c, sizeof(double) * 15 * nr);
    c.d_q = (double*)dalloc(c, sizeof(double) * 20 * nr);
    c.d_w = (double*)dalloc(c, sizeof(double) * 15 * nr);
    c.d_a = (double*)dalloc(c, sizeof(double) * 9 * nr);
    c.d_thermo = (double*)dalloc(c, sizeof(double) * TH_N);
    c.d_isum = (double*)dalloc(c, sizeof(double) * 8);
    c.d_done = (unsigned*)dalloc(c, sizeof(unsigned) * 4);
    if (c.alloc_failed) return set_err(&c, MDG_E_CUDA, "out of device memory for the integrator state");
    // the centres of mass of the force phases become the first Gear slice
    v.cx = c.d_c;
    v.cy = c.d_c + nr;
    v.cz = c.d_c + 2 * nr;
    // regions saved before each chunk of steps (restored when the list must grow)
    const int nold = v.ntota - v.nliqa, nflex = v.nmove - v.nriga;
    auto add = [&](void* p, size_t b) {
        if (p && b) c.snap_regions.push_back({p, b});
    };
    for (double* p : {v.x, v.y, v.z}) add(p, sizeof(double) * v.nmove);
    for (double* p : {v.rsx, v.rsy, v.rsz}) add(p, sizeof(double) * v.nmove);
    for (double* p : {c.d_xold, c.d_yold, c.d_zold}) add(p, sizeof(double) * nold);
    for (double* p : {v.ocx, v.ocy, v.ocz}) add(p, sizeof(double) * v.nrig);
    for (double* p : {v.ox, v.oy, v.oz}) add(p, sizeof(double) * nflex);
    add(c.d_xd, sizeof(double) * 12 * nion);
    add(c.d_c, sizeof(double) * 15 * nr);
    add(c.d_q, sizeof(double) * 20 * nr);
    add(c.d_w, sizeof(double) * 15 * nr);
    add(c.d_thermo, sizeof(double) * TH_N);
    size_t tot = 0;
    for (auto& r : c.snap_regions) tot += (r.second + 255) / 256 * 256;
    c.d_snap = (char*)dalloc(c, tot);
    if (c.alloc_failed) return set_err(&c, MDG_E_CUDA, "out of device memory for the step snapshot");
    return MDG_OK;
}

static void snapshot(Ctx& c, bool restore) {
    size_t off = 0;
    for (auto& r : c.snap_regions) {
        if (restore)
            cudaMemcpyAsync(r.first, c.d_snap + off, r.second, cudaMemcpyDeviceToDevice, c.stream);
        else
            cudaMemcpyAsync(c.d_snap + off, r.first, r.second, cudaMemcpyDeviceToDevice, c.stream);
        off += (r.second + 255) / 256 * 256;
    }
}

// One MD step (src/main.f90:60-64): predict, forces, correct, SHAKE.
static int step_launch(Ctx& c) {
    const bool fp64 = c.precision != MDG_MIXED, shake = c.v.nmove > c.v.nliqa, fuse = merge_fusable(c);
    const bool pack = !fp64 && !shake;  // surface atoms move in SHAKE, after the predictor
    if (c.batch_stage != 2) predict_launch(c, fp64, shake, pack);
    int rc = launch_force(c, false, false, fp64, fuse, pack);
    if (rc || c.batch_stage == 1) return rc;
    correct_launch(c, fuse);
    if (shake) shake_launch(c, c.d_ft, true);
    if (c.meas.init && c.meas.profiles) measure_do_launch(c, c.v.x, c.v.y, c.v.z);
    return MDG_OK;
}

int mdg_set_state(mdg_ctx* cp, const mdg_rigid* b, const mdg_state* st) {
    if (!cp || !b || !st) return set_err(cp, MDG_E_ARG, "null argument");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    View& v = c.v;
    MDG_CUDA(cudaStreamSynchronize(c.stream));
    int rc = resident_alloc_impl(c);
    if (rc) return rc;
    c.body = *b;
    const int nm = v.nmove, nr = v.nrig, nion = v.nliqa - v.nriga, nold = v.ntota - v.nliqa;
    MDG_CUDA(cudaMemcpy(v.x, st->x0, sizeof(double) * nm, cudaMemcpyHostToDevice));
    MDG_CUDA(cudaMemcpy(v.y, st->y0, sizeof(double) * nm, cudaMemcpyHostToDevice));
    MDG_CUDA(cudaMemcpy(v.z, st->z0, sizeof(double) * nm, cudaMemcpyHostToDevice));
    for (int k = 0; k < 4 && nion > 0; ++k) {
        const double* src[3] = {st->xd[k], st->yd[k], st->zd[k]};
        for (int d = 0; d < 3; ++d)
            MDG_CUDA(cudaMemcpy(c.d_xd + (k * 3 + d) * nion, src[d] + v.nriga, sizeof(double) * nion,
                                cudaMemcpyHostToDevice));
    }
    for (int k = 0; k < 5 && nr > 0; ++k) {
        const double* cs[3] = {st->cx[k], st->cy[k], st->cz[k]};
        const double* ws[3] = {st->wx[k], st->wy[k], st->wz[k]};
        for (int d = 0; d < 3; ++d) {
            MDG_CUDA(cudaMemcpy(c.d_c + (k * 3 + d) * nr, cs[d], sizeof(double) * nr, cudaMemcpyHostToDevice));
            MDG_CUDA(cudaMemcpy(c.d_w + (k * 3 + d) * nr, ws[d], sizeof(double) * nr, cudaMemcpyHostToDevice));
        }
        for (int q = 0; q < 4; ++q)
            MDG_CUDA(cudaMemcpy(c.d_q + (q * 5 + k) * nr, st->q[q][k], sizeof(double) * nr, cudaMemcpyHostToDevice));
    }
    if (nold > 0) {
        MDG_CUDA(cudaMemcpy(c.d_xold, st->xold, sizeof(double) * nold, cudaMemcpyHostToDevice));
        MDG_CUDA(cudaMemcpy(c.d_yold, st->yold, sizeof(double) * nold, cudaMemcpyHostToDevice));
        MDG_CUDA(cudaMemcpy(c.d_zold, st->zold, sizeof(double) * nold, cudaMemcpyHostToDevice));
    }
    MDG_CUDA(cudaMemcpy(v.rsx, st->rsx, sizeof(double) * nm, cudaMemcpyHostToDevice));
    MDG_CUDA(cudaMemcpy(v.rsy, st->rsy, sizeof(double) * nm, cudaMemcpyHostToDevice));
    MDG_CUDA(cudaMemcpy(v.rsz, st->rsz, sizeof(double) * nm, cudaMemcpyHostToDevice));
    double th[TH_N] = {0};
    for (int k = 0; k < 5; ++k) {
        th[TH_S + k] = st->s[k];
        th[TH_RS + k] = st->rs[k];
    }
    MDG_CUDA(cudaMemcpy(c.d_thermo, th, sizeof(th), cudaMemcpyHostToDevice));
    const int one = 1;
    MDG_CUDA(cudaMemcpy(v.status + ST_FORCE_RB, &one, sizeof(int), cudaMemcpyHostToDevice));
    c.resident = true;
    return MDG_OK;
}

int mdg_get_state(mdg_ctx* cp, mdg_state* st) {
    if (!cp || !st) return set_err(cp, MDG_E_ARG, "null argument");
    Ctx& c = *cp;
    if (!c.resident) return set_err(&c, MDG_E_ARG, "mdg_get_state before mdg_set_state");
    cudaSetDevice(c.device);
    View& v = c.v;
    MDG_CUDA(cudaStreamSynchronize(c.stream));
    const int nm = v.nmove, nr = v.nrig, nion = v.nliqa - v.nriga, nold = v.ntota - v.nliqa;
    auto get = [&](double* dst, const double* src, size_t n) -> cudaError_t {
        if (!dst || n == 0) return cudaSuccess;
        return cudaMemcpy(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost);
    };
    MDG_CUDA(get(st->x0, v.x, nm));
    MDG_CUDA(get(st->y0, v.y, nm));
    MDG_CUDA(get(st->z0, v.z, nm));
    for (int k = 0; k < 4 && nion > 0; ++k) {
        double* dst[3] = {st->xd[k], st->yd[k], st->zd[k]};
        for (int d = 0; d < 3; ++d)
            if (dst[d]) MDG_CUDA(get(dst[d] + v.nriga, c.d_xd + (k * 3 + d) * nion, nion));
    }
    for (int k = 0; k < 5 && nr > 0; ++k) {
        double* cs[3] = {st->cx[k], st->cy[k], st->cz[k]};
        double* ws[3] = {st->wx[k], st->wy[k], st->wz[k]};
        for (int d = 0; d < 3; ++d) {
            MDG_CUDA(get(cs[d], c.d_c + (k * 3 + d) * nr, nr));
            MDG_CUDA(get(ws[d], c.d_w + (k * 3 + d) * nr, nr));
        }
        for (int q = 0; q < 4; ++q) MDG_CUDA(get(st->q[q][k], c.d_q + (q * 5 + k) * nr, nr));
    }
    MDG_CUDA(get(st->xold, c.d_xold, nold));
    MDG_CUDA(get(st->yold, c.d_yold, nold));
    MDG_CUDA(get(st->zold, c.d_zold, nold));
    MDG_CUDA(get(st->rsx, v.rsx, nm));
    MDG_CUDA(get(st->rsy, v.rsy, nm));
    MDG_CUDA(get(st->rsz, v.rsz, nm));
    double th[TH_N];
    MDG_CUDA(cudaMemcpy(th, c.d_thermo, sizeof(th), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 5; ++k) {
        st->s[k] = th[TH_S + k];
        st->rs[k] = th[TH_RS + k];
    }
    return MDG_OK;
}

// One resident step captured as a graph (not instantiated); the caller owns *out.
static int capture_step_graph(Ctx& c, cudaGraph_t* out) {
    MDG_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    const int rc = step_launch(c);
    const cudaError_t e = cudaStreamEndCapture(c.stream, out);
    if (rc) return rc;
    if (e != cudaSuccess) return set_err(&c, MDG_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    return MDG_OK;
}

static int ensure_graph(Ctx& c, int nstep) {
    if (c.graph_exec) return MDG_OK;
    cudaGraph_t g;
    MDG_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    int rc = MDG_OK;
    for (int t = 0; t < nstep && rc == MDG_OK; ++t) rc = step_launch(c);
    cudaError_t e = cudaStreamEndCapture(c.stream, &g);
    if (rc) return rc;
    if (e != cudaSuccess) return set_err(&c, MDG_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    size_t nn = 0;
    cudaGraphGetNodes(g, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn) cudaGraphGetNodes(g, nodes.data(), &nn);
    int64_t kern = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kern;
    }
    c.kernels_per_step = kern / std::max(nstep, 1);
    e = cudaGraphInstantiate(&c.graph_exec, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_err(&c, MDG_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    c.graph_steps = nstep;
    return MDG_OK;
}

static void fill_report(Ctx& c, const double* th, mdg_report* rep) {
    View& v = c.v;
    rep->kp = th[TH_KP];
    rep->kw = th[TH_KW];
    rep->ke = th[TH_KE];
    rep->htot = th[TH_HTOT];
    rep->tempnow = th[TH_TEMPNOW];
    rep->uconf = th[TH_UCONF];
    rep->press = th[TH_PRESS];
    rep->steps = (int64_t)th[TH_STEPS];
    rep->rebuilds = (int64_t)th[TH_REBUILDS];
    rep->last_sweeps = c.h_status[ST_SWEEPS];
    double hk[64] = {0};
    cudaMemcpy(hk, c.d_kps, sizeof(double) * std::min(v.nit, 64), cudaMemcpyDeviceToHost);
    double ks = 0.0;
    for (int t = 0; t < std::min(v.nit, 64); ++t) ks += hk[t];
    rep->tkps = c.nfreed > 0 ? ks * 1000.0 / ((double)8.31441f * (double)(float)c.nfreed) : 0.0;
}

int mdg_run_async(mdg_ctx* cp, int64_t nsteps) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    if (!c.resident) return set_err(&c, MDG_E_ARG, "mdg_run_async before mdg_set_state");
    cudaSetDevice(c.device);
    if (c.debug_sync) {
        for (int64_t k = 0; k < nsteps; ++k) {
            int rc = step_launch(c);
            if (rc) return rc;
        }
        return MDG_OK;
    }
    int rc = ensure_graph(c, 1);
    if (rc) return rc;
    for (int64_t k = 0; k < nsteps; ++k) MDG_CUDA(cudaGraphLaunch(c.graph_exec, c.stream));
    return MDG_OK;
}

int mdg_check(mdg_ctx* cp, mdg_report* rep) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    int rc = read_status(c);
    if (rc) return rc;
    MDG_CUDA(cudaMemsetAsync(c.v.status, 0, sizeof(int) * 4, c.stream));
    if (c.h_status[ST_LIST_OVF] || c.h_status[ST_WLIST_OVF])
        return set_err(&c, MDG_E_LIST_OVERFLOW, "nnlist_make(): nnlist too big! (rerun with mdg_run)");
    if (c.h_status[ST_SHAKE_RPTOL]) return set_err(&c, MDG_E_SHAKE_RPTOL, "Constraint failure");
    if (c.h_status[ST_SHAKE_MAXIT]) return set_err(&c, MDG_E_SHAKE_MAXIT, "shake(): Too many constraint iterations!");
    if (c.resident) {
        double th[TH_N];
        MDG_CUDA(cudaMemcpy(th, c.d_thermo, sizeof(th), cudaMemcpyDeviceToHost));
        if (!std::isfinite(th[TH_HTOT]) || !std::isfinite(th[TH_UCONF]))
            return set_err(&c, MDG_E_NAN, "non-finite energy");
        if (rep) fill_report(c, th, rep);
    }
    return MDG_OK;
}

int64_t mdg_kernels_per_step(const mdg_ctx* cp) { return cp ? cp->kernels_per_step : 0; }

int mdg_run(mdg_ctx* cp, int64_t nsteps, mdg_report* rep) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    if (!c.resident) return set_err(&c, MDG_E_ARG, "mdg_run before mdg_set_state");
    cudaSetDevice(c.device);
    View& v = c.v;
    const int kGraph = 1;     // steps per captured graph (relaunched; launch cost is a few us)
    const int kChunk = 64;    // steps between status checks
    const bool graphs = !c.debug_sync;
    int64_t done = 0;
    int retries = 0;
    while (done < nsteps) {
        const int64_t chunk = std::min<int64_t>(kChunk, nsteps - done);
        snapshot(c, false);
        MDG_CUDA(cudaMemsetAsync(v.status, 0, sizeof(int) * 4, c.stream));
        int64_t k = 0;
        if (graphs && chunk >= kGraph) {
            int rc = ensure_graph(c, kGraph);
            if (rc) return rc;
            for (; k + kGraph <= chunk; k += kGraph) MDG_CUDA(cudaGraphLaunch(c.graph_exec, c.stream));
        }
        for (; k < chunk; ++k) {
            int rc = step_launch(c);
            if (rc) return rc;
        }
        int rc = read_status(c);
        if (rc) return rc;
        const int ovf = c.h_status[ST_LIST_OVF], wovf = c.h_status[ST_WLIST_OVF];
        if (ovf || wovf) {
            if (++retries > 4) return set_err(&c, MDG_E_LIST_OVERFLOW, "nnlist_make(): nnlist too big!");
            rc = alloc_lists(c, ovf ? ovf + ovf / 4 + 32 : v.maxnb, wovf ? wovf + wovf / 4 + 32 : v.maxwnb);
            if (rc) return rc;
            snapshot(c, true);
            const int one = 1;
            MDG_CUDA(cudaMemcpyAsync(v.status + ST_FORCE_RB, &one, sizeof(int), cudaMemcpyHostToDevice, c.stream));
            MDG_CUDA(cudaStreamSynchronize(c.stream));
            continue;
        }
        if (c.h_status[ST_SHAKE_RPTOL]) return set_err(&c, MDG_E_SHAKE_RPTOL, "Constraint failure");
        if (c.h_status[ST_SHAKE_MAXIT]) return set_err(&c, MDG_E_SHAKE_MAXIT, "shake(): Too many constraint iterations!");
        done += chunk;
    }
    double th[TH_N];
    MDG_CUDA(cudaMemcpy(th, c.d_thermo, sizeof(th), cudaMemcpyDeviceToHost));
    if (!std::isfinite(th[TH_HTOT]) || !std::isfinite(th[TH_UCONF])) return set_err(&c, MDG_E_NAN, "non-finite energy");
    if (rep) fill_report(c, th, rep);
    return MDG_OK;
}

int mdg_set_stream(mdg_ctx* cp, void* stream) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    MDG_CUDA(cudaStreamSynchronize(c.stream));
    if (!c.own_stream) c.own_stream = c.stream;
    c.stream = stream ? (cudaStream_t)stream : c.own_stream;
    drop_graphs(c);
    return MDG_OK;
}

int mdg_phase_times(mdg_ctx* cp, int reps, double* ms) {
    if (!cp || !ms || reps < 1) return set_err(cp, MDG_E_ARG, "bad argument");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    View& v = c.v;
    cudaEvent_t ev[8];
    for (auto& e : ev) MDG_CUDA(cudaEventCreate(&e));
    double acc[MDG_NPHASE] = {0};
    for (int r = 0; r < reps; ++r) {
        cudaMemsetAsync(v.fx, 0, sizeof(double) * std::max(v.nmove, 1), c.stream);
        cudaMemsetAsync(v.fy, 0, sizeof(double) * std::max(v.nmove, 1), c.stream);
        cudaMemsetAsync(v.fz, 0, sizeof(double) * std::max(v.nmove, 1), c.stream);
        cudaMemsetAsync(v.acc, 0, sizeof(double) * (2 * v.nijt + ACC_NSLOT), c.stream);
        cudaMemsetAsync(v.status, 0, sizeof(int) * 2, c.stream);
        cudaEventRecord(ev[0], c.stream);
        nnlist_trigger(c, true);
        nnlist_build(c);
        cudaEventRecord(ev[1], c.stream);
        if (c.precision == MDG_MIXED) {
            pack_mixed(c, false);
            pairs_mixed(c, true);
        } else {
            pair_forces_fp64(c);
        }
        surf_partition(c);
        cudaEventRecord(ev[2], c.stream);
        if (c.precision == MDG_MIXED) {
            walls_mixed(c);
            merge_mixed(c, nullptr, false);
        } else {
            wall_forces_fp64(c);
        }
        cudaEventRecord(ev[3], c.stream);
        if (c.precision == MDG_MIXED) {
            recip_tc(c);
            merge_mixed(c, c.d_frc, true);
        } else {
            recip_fp64(c);
        }
        cudaEventRecord(ev[4], c.stream);
        lr_tail(c);
        if (c.precision != MDG_MIXED) dipole_correction(c);
        angle_forces(c);
        force_sum(c, c.d_ft, c.d_fc, c.d_tq);
        cudaEventRecord(ev[5], c.stream);
        if (c.resident) {
            predict_launch(c);
            correct_launch(c);
        }
        cudaEventRecord(ev[6], c.stream);
        if (v.nmove > v.nliqa && c.ncons > 0 && c.resident) shake_launch(c, c.d_ft);
        cudaEventRecord(ev[7], c.stream);
        MDG_CUDA(cudaEventSynchronize(ev[7]));
        for (int k = 0; k < MDG_NPHASE; ++k) {
            float t = 0.f;
            cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
            acc[k] += t;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    for (int k = 0; k < MDG_NPHASE; ++k) ms[k] = acc[k] / reps;
    return sync_check(c, "mdg_phase_times");
}

int mdg_recip_forces_noalloc(const double* x, const double* y, const double* z, const double* q, int64_t n,
                             double lx, double ly, double lz, double alpha, int64_t kmax, double* fx, double* fy,
                             double* fz, double* uewa, void* stream) {
    const int rc = recip_forces_noalloc(x, y, z, q, n, lx, ly, lz, alpha, kmax, fx, fy, fz, uewa, (cudaStream_t)stream);
    if (rc) g_err = recip_noalloc_error();
    return rc;
}

int mdg_selftest_umma(int n, int k, const float* a, const float* b, float* d) {
    std::string err;
    const int rc = umma_selftest(n, k, a, b, d, err);
    if (rc) g_err = err;
    return rc;
}

// ---------------------------------------------------------------------------------------------
// Learned SHAKE seed
// ---------------------------------------------------------------------------------------------
int mdg_mlp_nw(void) { return mlp_nw(); }

int mdg_shake_set_model(mdg_ctx* cp, const float* w, int64_t n) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    if (n == 0 || !w) {
        c.shake_model = false;
    } else {
        if (n != mlp_nw()) return set_err(&c, MDG_E_ARG, "mdg_shake_set_model: parameter count differs from mdg_mlp_nw()");
        MDG_CUDA(cudaStreamSynchronize(c.stream));
        MDG_CUDA(cudaMemcpy(c.d_mlpw, w, sizeof(float) * n, cudaMemcpyHostToDevice));
        c.shake_model = true;
    }
    drop_graphs(c);
    return MDG_OK;
}

int mdg_shake_record(mdg_ctx* cp, int enable) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    c.shake_record = enable != 0;
    drop_graphs(c);
    return MDG_OK;
}

int mdg_shake_samples(mdg_ctx* cp, float* out) {
    if (!cp || !out) return set_err(cp, MDG_E_ARG, "null argument");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    MDG_CUDA(cudaStreamSynchronize(c.stream));
    MDG_CUDA(cudaMemcpy(out, c.d_shake_rec, sizeof(float) * 16 * c.ncons, cudaMemcpyDeviceToHost));
    return MDG_OK;
}

int mdg_mlp_forward(const float* w, const float* x, int64_t n, float* y) {
    std::string err;
    const int rc = mlp_forward_host(w, x, n, y, err);
    if (rc) g_err = err;
    return rc;
}

int mdg_mlp_grad(const float* w, const float* x, const float* y, int64_t n, float* grad, float* loss) {
    std::string err;
    const int rc = mlp_grad_host(w, x, y, n, grad, loss, err);
    if (rc) g_err = err;
    return rc;
}

int mdg_mlp_train(const float* x, const float* y, int64_t n, int epochs, int batch, float lr, uint64_t seed,
                  float* w_out, float* loss_out) {
    std::string err;
    const int rc = mlp_train_host(x, y, n, epochs, batch, lr, seed, w_out, loss_out, err);
    if (rc) g_err = err;
    return rc;
}

// ---------------------------------------------------------------------------------------------
// Replica batches: independent contexts stepped by one graph launch.  Two graph forms:
//   MDG_BATCH_GRAPHS  every replica's step graph is a parallel child graph of one graph, so the
//                     kernels of small systems fill the GPU together;
//   MDG_BATCH_PHASES  phase order: every replica's predictor, packing close (rebuild decision),
//                     wall tail and reciprocal branch as in its own step, then, for the replicas
//                     in the concurrent mixed form (walls, no surface atoms), the list build as
//                     five launches in all and the head-head and head-wall loops as one persistent
//                     kernel each over all their heads, then every replica's merge, corrector and
//                     SHAKE.  Other replicas keep their whole step in the graph.
// ---------------------------------------------------------------------------------------------
struct mdg_batch {
    std::vector<mdg_ctx*> ctx;
    cudaStream_t stream = nullptr;      // stream the batch graph is launched on
    cudaStream_t own_stream = nullptr;  // the batch's own stream (the only one it destroys)
    cudaStream_t cs = nullptr, cs2 = nullptr;  // capture streams of the phase-ordered graph
    std::vector<cudaEvent_t> ev;        // its fork and join events: 4 + 2 per replica
    RsBatch rb;                         // descriptors of the batched real-space loops
    LsBatch lb;                         // and of the batched list build
    int mode = MDG_BATCH_PHASES;
    int phased = 0;                     // replicas in the batched loops (last graph build)
    cudaGraphExec_t exec = nullptr;
    int device = 0;
    std::string err;
};

static int batch_err(mdg_batch* b, int code, const std::string& m) {
    if (b) b->err = m;
    g_err = m;
    return code;
}

static int batch_graph_phases(mdg_batch* b) {
    const size_t n = b->ctx.size();
    if (!b->cs) {
        // the batched loops hold up every replica's merge: as urgent as the reciprocal branches
        int prio_lo = 0, prio_hi = 0;
        cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
        if (cudaStreamCreateWithPriority(&b->cs, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
            cudaStreamCreateWithPriority(&b->cs2, cudaStreamNonBlocking, prio_hi) != cudaSuccess)
            return batch_err(b, MDG_E_CUDA, "batch: capture streams");
    }
    while (b->ev.size() < 4 + 2 * n) {
        cudaEvent_t e;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return batch_err(b, MDG_E_CUDA, "batch: events");
        b->ev.push_back(e);
    }
    std::vector<Ctx*> ph;
    std::vector<char> is_ph(n, 0);
    for (size_t i = 0; i < n; ++i)
        if (batch_phased(*b->ctx[i])) {
            ph.push_back(b->ctx[i]);
            is_ph[i] = 1;
        }
    std::string err;
    int rc = rs_batch_setup(b->rb, ph, err);
    if (!rc) rc = ls_batch_setup(b->lb, ph, err);
    if (rc) return batch_err(b, rc, err);
    b->phased = (int)ph.size();
    cudaEvent_t ev0 = b->ev[0], evf = b->ev[1], evw = b->ev[2], evrs = b->ev[3];
    auto ev_pre = [&](size_t i) { return b->ev[4 + 2 * i]; };
    auto ev_post = [&](size_t i) { return b->ev[5 + 2 * i]; };
    if (cudaStreamBeginCapture(b->cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return batch_err(b, MDG_E_CUDA, "batch: capture");
    auto fail = [&](int code, const std::string& m) {
        cudaGraph_t gg = nullptr;
        cudaStreamEndCapture(b->cs, &gg);
        if (gg) cudaGraphDestroy(gg);
        cudaGetLastError();
        for (auto* cp : b->ctx) cp->batch_stage = 0;
        return batch_err(b, code, m);
    };
    bool ok = cudaEventRecord(ev0, b->cs) == cudaSuccess;
    for (size_t i = 0; i < n && ok; ++i) {
        Ctx& c = *b->ctx[i];
        ok = cudaStreamWaitEvent(c.stream, ev0, 0) == cudaSuccess;
        c.batch_stage = is_ph[i] ? 1 : 0;
        rc = step_launch(c);
        c.batch_stage = 0;
        if (rc) return fail(rc, "replica " + std::to_string(i) + ": " + c.err);
        ok = ok && cudaEventRecord(ev_pre(i), c.stream) == cudaSuccess;
    }
    if (ok && !ph.empty()) {
        for (size_t i = 0; i < n && ok; ++i)
            if (is_ph[i]) ok = cudaStreamWaitEvent(b->cs, ev_pre(i), 0) == cudaSuccess;
        if (ok) ls_batch_launch(b->lb, b->cs);
        ok = ok && cudaEventRecord(evf, b->cs) == cudaSuccess && cudaStreamWaitEvent(b->cs2, evf, 0) == cudaSuccess;
        if (ok) rs_batch_launch(b->rb, b->cs, b->cs2);
        ok = ok && cudaEventRecord(evw, b->cs2) == cudaSuccess && cudaStreamWaitEvent(b->cs, evw, 0) == cudaSuccess &&
             cudaEventRecord(evrs, b->cs) == cudaSuccess;
        for (size_t i = 0; i < n && ok; ++i) {
            if (!is_ph[i]) continue;
            Ctx& c = *b->ctx[i];
            ok = cudaStreamWaitEvent(c.stream, evrs, 0) == cudaSuccess;
            c.batch_stage = 2;
            rc = step_launch(c);
            c.batch_stage = 0;
            if (rc) return fail(rc, "replica " + std::to_string(i) + ": " + c.err);
            ok = ok && cudaEventRecord(ev_post(i), c.stream) == cudaSuccess;
        }
    }
    for (size_t i = 0; i < n && ok; ++i)
        ok = cudaStreamWaitEvent(b->cs, is_ph[i] ? ev_post(i) : ev_pre(i), 0) == cudaSuccess;
    if (!ok) return fail(MDG_E_CUDA, std::string("batch capture: ") + cudaGetErrorString(cudaGetLastError()));
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(b->cs, &g);
    if (ce != cudaSuccess) return batch_err(b, MDG_E_CUDA, std::string("batch capture: ") + cudaGetErrorString(ce));
    const cudaError_t e = cudaGraphInstantiate(&b->exec, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return batch_err(b, MDG_E_CUDA, std::string("batch instantiate: ") + cudaGetErrorString(e));
    return MDG_OK;
}

// Replicas in a batch share the GPU, so their tensor-core passes take the fewest CTAs (each CTA
// holds an SM for its set-up; one system alone instead spreads its passes over every SM).
static int batch_plans(mdg_batch* b, bool on) {
    for (size_t i = 0; i < b->ctx.size(); ++i) {
        Ctx& c = *b->ctx[i];
        if (c.precision != MDG_MIXED || !c.tcp.ready) continue;
        const int rc = recip_tc_throughput(c, on);
        if (rc) return batch_err(b, rc, "replica " + std::to_string(i) + ": " + c.err);
    }
    return MDG_OK;
}

static int batch_graph(mdg_batch* b) {
    if (b->exec) return MDG_OK;
    const int prc = batch_plans(b, true);
    if (prc) return prc;
    if (b->mode == MDG_BATCH_PHASES) return batch_graph_phases(b);
    b->phased = 0;
    cudaGraph_t g;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) return batch_err(b, MDG_E_CUDA, "cudaGraphCreate failed");
    for (size_t i = 0; i < b->ctx.size(); ++i) {
        Ctx& c = *b->ctx[i];
        cudaGraph_t child;
        int rc = capture_step_graph(c, &child);
        if (rc) {
            cudaGraphDestroy(g);
            return batch_err(b, rc, "replica " + std::to_string(i) + ": " + c.err);
        }
        cudaGraphNode_t node;
        const cudaError_t e = cudaGraphAddChildGraphNode(&node, g, nullptr, 0, child);
        cudaGraphDestroy(child);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            return batch_err(b, MDG_E_CUDA, std::string("child graph: ") + cudaGetErrorString(e));
        }
    }
    const cudaError_t e = cudaGraphInstantiate(&b->exec, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return batch_err(b, MDG_E_CUDA, std::string("batch instantiate: ") + cudaGetErrorString(e));
    return MDG_OK;
}

int mdg_batch_create(mdg_ctx* const* ctxs, int n, mdg_batch** out) {
    if (!ctxs || n < 1 || !out) return batch_err(nullptr, MDG_E_ARG, "mdg_batch_create: bad argument");
    auto* b = new mdg_batch();
    b->device = ctxs[0]->device;
    for (int i = 0; i < n; ++i) {
        if (!ctxs[i] || !ctxs[i]->resident || ctxs[i]->device != b->device) {
            delete b;
            return batch_err(nullptr, MDG_E_ARG, "mdg_batch_create: every context needs mdg_set_state, one device");
        }
        b->ctx.push_back(ctxs[i]);
    }
    cudaSetDevice(b->device);
    if (cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        return batch_err(nullptr, MDG_E_CUDA, "mdg_batch_create: stream");
    }
    b->stream = b->own_stream;
    *out = b;
    return MDG_OK;
}

void mdg_batch_destroy(mdg_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    batch_plans(b, false);  // the contexts step alone again with their own plans
    if (b->own_stream) cudaStreamDestroy(b->own_stream);  // a caller's stream stays the caller's
    if (b->cs) cudaStreamDestroy(b->cs);
    if (b->cs2) cudaStreamDestroy(b->cs2);
    for (cudaEvent_t e : b->ev) cudaEventDestroy(e);
    rs_batch_free(b->rb);
    ls_batch_free(b->lb);
    delete b;
}

const char* mdg_batch_last_error(const mdg_batch* b) { return b ? b->err.c_str() : g_err.c_str(); }

int mdg_batch_set_stream(mdg_batch* b, void* stream) {
    if (!b) return batch_err(nullptr, MDG_E_ARG, "null batch");
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    b->stream = stream ? (cudaStream_t)stream : b->own_stream;
    return MDG_OK;
}

int mdg_batch_set_mode(mdg_batch* b, int mode, int pair_blocks, int wall_blocks) {
    if (!b) return batch_err(nullptr, MDG_E_ARG, "null batch");
    if ((mode != MDG_BATCH_GRAPHS && mode != MDG_BATCH_PHASES) || pair_blocks < 0 || wall_blocks < 0)
        return batch_err(b, MDG_E_ARG, "mdg_batch_set_mode: bad argument");
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->mode = mode;
    b->rb.blocks_p = pair_blocks > 0 ? pair_blocks : RsBatch().blocks_p;
    b->rb.blocks_w = wall_blocks > 0 ? wall_blocks : RsBatch().blocks_w;
    return MDG_OK;
}

int mdg_batch_phased(const mdg_batch* b) { return b ? b->phased : 0; }

int mdg_batch_run_async(mdg_batch* b, int64_t nsteps) {
    if (!b) return batch_err(nullptr, MDG_E_ARG, "null batch");
    cudaSetDevice(b->device);
    int rc = batch_graph(b);
    if (rc) return rc;
    for (int64_t k = 0; k < nsteps; ++k)
        if (cudaGraphLaunch(b->exec, b->stream) != cudaSuccess) return batch_err(b, MDG_E_CUDA, "batch graph launch");
    return MDG_OK;
}

// Steps every replica nsteps times.  Status is checked every 64 steps; a replica whose neighbour
// list overflowed in a chunk is rolled back and redoes that chunk alone with larger lists
// (mdg_run), after which the batch graph is rebuilt.  reps: n reports or NULL.
int mdg_batch_run(mdg_batch* b, int64_t nsteps, mdg_report* reps) {
    if (!b) return batch_err(nullptr, MDG_E_ARG, "null batch");
    cudaSetDevice(b->device);
    const int64_t kChunk = 64;
    int64_t done = 0;
    while (done < nsteps) {
        const int64_t chunk = std::min<int64_t>(kChunk, nsteps - done);
        for (auto* cp : b->ctx) {
            snapshot(*cp, false);
            cudaMemsetAsync(cp->v.status, 0, sizeof(int) * 4, cp->stream);
        }
        for (auto* cp : b->ctx) cudaStreamSynchronize(cp->stream);
        int rc = mdg_batch_run_async(b, chunk);
        if (rc) return rc;
        if (cudaStreamSynchronize(b->stream) != cudaSuccess) return batch_err(b, MDG_E_CUDA, "batch step failed");
        bool rebuild = false;
        for (size_t i = 0; i < b->ctx.size(); ++i) {
            Ctx& c = *b->ctx[i];
            rc = read_status(c);
            if (rc) return batch_err(b, rc, "replica " + std::to_string(i) + ": " + c.err);
            const int ovf = c.h_status[ST_LIST_OVF], wovf = c.h_status[ST_WLIST_OVF];
            if (ovf || wovf) {
                rc = alloc_lists(c, ovf ? ovf + ovf / 4 + 32 : c.v.maxnb, wovf ? wovf + wovf / 4 + 32 : c.v.maxwnb);
                if (rc) return batch_err(b, rc, "replica " + std::to_string(i) + ": " + c.err);
                snapshot(c, true);
                const int one = 1;
                cudaMemcpyAsync(c.v.status + ST_FORCE_RB, &one, sizeof(int), cudaMemcpyHostToDevice, c.stream);
                cudaStreamSynchronize(c.stream);
                rc = mdg_run(b->ctx[i], chunk, nullptr);
                if (rc) return batch_err(b, rc, "replica " + std::to_string(i) + ": " + c.err);
                rebuild = true;
                continue;
            }
            if (c.h_status[ST_SHAKE_RPTOL])
                return batch_err(b, MDG_E_SHAKE_RPTOL, "replica " + std::to_string(i) + ": Constraint failure");
            if (c.h_status[ST_SHAKE_MAXIT])
                return batch_err(b, MDG_E_SHAKE_MAXIT, "replica " + std::to_string(i) + ": shake(): Too many constraint iterations!");
        }
        if (rebuild && b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        done += chunk;
    }
    if (reps) {
        for (size_t i = 0; i < b->ctx.size(); ++i) {
            Ctx& c = *b->ctx[i];
            double th[TH_N];
            if (cudaMemcpy(th, c.d_thermo, sizeof(th), cudaMemcpyDeviceToHost) != cudaSuccess)
                return batch_err(b, MDG_E_CUDA, "batch report");
            fill_report(c, th, &reps[i]);
        }
    }
    return MDG_OK;
}

// ---------------------------------------------------------------------------------------------
// Autotuner: launch parameters of the force phases timed on this context's own system
// ---------------------------------------------------------------------------------------------
// One candidate's force evaluation time, replayed as the captured graph the calls run (branches
// overlap and the reciprocal stream's priority holds there, not in eager launches); eager when
// the capture fails.
static float time_force(Ctx& c, int reps) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaGraphExec_t ge = nullptr;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const int rc = launch_force(c, false, true);
        const cudaError_t ce = cudaStreamEndCapture(c.stream, &g);
        if (rc == MDG_OK && ce == cudaSuccess &&
            cudaGraphInstantiate(&ge, g, cudaGraphInstantiateFlagUseNodePriority) != cudaSuccess)
            ge = nullptr;
        if (g) cudaGraphDestroy(g);
    }
    cudaGetLastError();
    auto once = [&]() {
        if (ge) cudaGraphLaunch(ge, c.stream);
        else launch_force(c, false, true);
    };
    once();
    cudaEventRecord(a, c.stream);
    for (int r = 0; r < reps; ++r) once();
    cudaEventRecord(b, c.stream);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ge) cudaGraphExecDestroy(ge);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms / std::max(reps, 1);
}

// A candidate replaces the current choice only when it is at least 2 % faster: differences below
// that are within the spread of repeated timings, and the defaults are chosen for the resident
// step (whose branches overlap differently from the force evaluation timed here).
constexpr float kTuneGain = 0.98f;

int mdg_autotune(mdg_ctx* cp, int32_t reps, mdg_tuning* out) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    reps = std::max(reps, 1);
    const float t0 = time_force(c, reps);
    // real-space grid (blocks of 8 warps; 0 = one warp per head up to 16 blocks per SM)
    int best_pb = c.pair_blocks;
    float best = t0;
    for (int pb : {0, 152 * 2, 152 * 4, 152 * 8}) {
        c.pair_blocks = pb;
        const float t = time_force(c, reps);
        if (t < best * kTuneGain) {
            best = t;
            best_pb = pb;
        }
    }
    c.pair_blocks = best_pb;
    // structure-factor split: row tiles per CTA x atom splits
    if (c.precision == MDG_MIXED && c.tcp.ready) {
        const int trc = recip_tc_throughput(c, false);  // tune the plan for the system alone
        if (trc) return trc;
    }
    int best_tpc = c.tcp.tpc1, best_mult = c.tcp.mult1;
    if (c.precision == MDG_MIXED && c.tcp.ready) {
        best = time_force(c, reps);
        // the n-side form when it applies (its accumulation chains are short), its atom split tuned
        const bool nside = c.tcp.tpc1 == 1;
        for (int tpc : {1, 4, 2})
            for (int m : {1, 2, 4}) {
                if ((tpc == 1) != nside) continue;
                if (tc_plan_pass1(c, tpc, m)) continue;
                const float t = time_force(c, reps);
                if (t < best * kTuneGain) {
                    best = t;
                    best_tpc = tpc;
                    best_mult = m;
                }
            }
        tc_plan_pass1(c, best_tpc, best_mult);
    }
    drop_graphs(c);
    const float t1 = time_force(c, reps);
    MDG_CUDA(cudaStreamSynchronize(c.stream));
    int rc = read_status(c);
    if (rc) return rc;
    if (out) {
        out->pair_blocks = best_pb;
        out->tc_rows_per_cta = best_tpc == 1 ? 256 : 128 * best_tpc;
        out->tc_atom_splits = c.tcp.nsplit1;
        out->ms_before = t0;
        out->ms_after = t1;
    }
    return MDG_OK;
}

// ---------------------------------------------------------------------------------------------
// Measurement histograms (measure.cu)
// ---------------------------------------------------------------------------------------------
static void drop_graph(Ctx& c) {
    drop_graphs(c);
}

int mdg_measure_init(mdg_ctx* cp, const mdg_measure_params* p, mdg_measure_dims* d) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    MDG_CUDA(cudaStreamSynchronize(c.stream));
    const int rc = measure_init(c, p, d);
    if (rc) return rc;
    drop_graph(c);
    return MDG_OK;
}

int mdg_measure_enable(mdg_ctx* cp, int force_hist, int profiles) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    if (!c.meas.init) return set_err(&c, MDG_E_ARG, "measure: mdg_measure_init first");
    if (c.meas.force_hist != (force_hist != 0) || c.meas.profiles != (profiles != 0)) {
        cudaSetDevice(c.device);
        MDG_CUDA(cudaStreamSynchronize(c.stream));
        drop_graph(c);
    }
    c.meas.force_hist = force_hist != 0;
    c.meas.profiles = profiles != 0;
    return MDG_OK;
}

int mdg_measure_zero(mdg_ctx* cp) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    if (!c.meas.init) return set_err(&c, MDG_E_ARG, "measure: mdg_measure_init first");
    cudaSetDevice(c.device);
    measure_zero(c);
    MDG_CUDA(cudaStreamSynchronize(c.stream));
    return MDG_OK;
}

int mdg_measure_do(mdg_ctx* cp, const double* x0, const double* y0, const double* z0) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    if (!c.meas.init) return set_err(&c, MDG_E_ARG, "measure: mdg_measure_init first");
    if ((x0 == nullptr) != (y0 == nullptr) || (x0 == nullptr) != (z0 == nullptr))
        return set_err(&c, MDG_E_ARG, "measure: give all of x0, y0, z0 or none");
    cudaSetDevice(c.device);
    const View& v = c.v;
    if (x0) {
        const size_t n = (size_t)std::max(v.nmove, 1);
        double* pos = c.meas.m.pos;
        MDG_CUDA(cudaMemcpyAsync(pos, x0, sizeof(double) * v.nmove, cudaMemcpyHostToDevice, c.stream));
        MDG_CUDA(cudaMemcpyAsync(pos + n, y0, sizeof(double) * v.nmove, cudaMemcpyHostToDevice, c.stream));
        MDG_CUDA(cudaMemcpyAsync(pos + 2 * n, z0, sizeof(double) * v.nmove, cudaMemcpyHostToDevice, c.stream));
        measure_do_launch(c, pos, pos + n, pos + 2 * n);
    } else {
        if (!c.resident) return set_err(&c, MDG_E_ARG, "measure: no positions and no resident state");
        measure_do_launch(c, v.x, v.y, v.z);
    }
    MDG_CUDA(cudaStreamSynchronize(c.stream));
    MDG_CUDA(cudaGetLastError());
    return MDG_OK;
}

int mdg_measure_get(mdg_ctx* cp, mdg_measure_out* o) {
    if (!cp || !o) return set_err(cp, MDG_E_ARG, "null argument");
    Ctx& c = *cp;
    if (!c.meas.init) return set_err(&c, MDG_E_ARG, "measure: mdg_measure_init first");
    cudaSetDevice(c.device);
    return measure_get(c, o);
}

// ---------------------------------------------------------------------------------------------
// Widom insertion (widom.cu)
// ---------------------------------------------------------------------------------------------
int mdg_widom(mdg_ctx* cp, const mdg_widom_params* prm, double* seed, double* pave, int64_t* inave, int64_t* done) {
    if (!cp) return set_err(nullptr, MDG_E_ARG, "null context");
    Ctx& c = *cp;
    cudaSetDevice(c.device);
    MDG_CUDA(cudaStreamSynchronize(c.stream));
    return widom(c, prm, seed, pave, inave, done);
}

}  // extern "C"

namespace mdg {
int resident_alloc(Ctx& c) { return resident_alloc_impl(c); }
}  // namespace mdg
