// shake.cu - move_shake (src/move.f90:408-529) on the GPU.
//
// Verlet step of the surface atoms (:416-439) with the per-type kinetic sums kps, then SHAKE.
// The reference sweeps molecules in order (Gauss-Seidel), skips a constraint when neither atom
// moved in the previous sweep, and resets `done` per molecule (:458), so the loop length is
// decided by the last molecule alone (stop after its first sweep without an update, at most
// maxit+1 sweeps).  When no moving atom belongs to two constrained molecules, molecules evolve
// independently; then
//   k_shake_last  replays the last molecule on private copies to get that sweep count, and
//   k_shake_mol   runs every molecule for exactly that many sweeps, one thread per molecule,
// which gives the reference's positions exactly.  Frozen atoms (index >= nmove) never count as
// moved, as moved(ismax+1:ntota) = 1 in the reference.  Topologies that share moving atoms
// between molecules fall back to k_shake_seq, a single-thread copy of the reference loop.
// Every loop is bounded by maxit+1 sweeps.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "ctx.h"
#include "mlp.cuh"

namespace mdg {

namespace {

constexpr int kNT = 128;
constexpr int kMolNT = 64;
constexpr int kMaxAt = 6;

struct ShakeArgs {
    int ncons, maxit, clean, nliqa, nmove;
    double tol2, rptol;
    const int* cons;      // ncons * 6: (a0,b0,a1,b1,a2,b2), -1 unused
    const double* clen2;  // ncons * 3
    const int* cons_n;    // ncons
    double *xo, *yo, *zo; // xold(nliqa:ntota)
    int* sweeps_out;      // [0] sweeps decided, [1] done flag
    const float* mlpw;    // seeding network (mlp.cuh blob) or nullptr
    float* rec;           // ncons x 16: features, accumulated multipliers, sweeps of this call, or nullptr
};

__global__ void k_verlet(View v, const double* ft, double* xo, double* yo, double* zo, double* kps) {
    const int i = v.nliqa + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nmove) return;
    const int k = i - v.nliqa, f = i - v.nriga;
    const int nflex = v.nmove - v.nriga;
    const double m = v.mii[i];
    double aux = v.x[i] - xo[k];
    xo[k] = v.x[i];
    aux = minimg(aux, v.lx, v.lxi);
    v.x[i] = v.x[i] + aux + ft[f] * m;
    double kaux = aux * aux;
    aux = v.y[i] - yo[k];
    yo[k] = v.y[i];
    aux = minimg(aux, v.ly, v.lyi);
    v.y[i] = v.y[i] + aux + ft[nflex + f] * m;
    kaux = kaux + aux * aux;
    aux = v.z[i] - zo[k];
    zo[k] = v.z[i];
    v.z[i] = v.z[i] + aux + ft[2 * nflex + f] * m;
    kaux = kaux + aux * aux;
    atomicAdd(&kps[v.type[i]], v.mi[i] * kaux);
}

// One molecule's state in registers.
struct Mol {
    int n;               // constraints
    int at[kMaxAt];      // distinct atoms
    int na;
    int ca[3], cb[3];    // local slots of the constraint atoms
    double l2[3];
};

__device__ __forceinline__ int slot_of(Mol& m, int a) {
    for (int s = 0; s < m.na; ++s)
        if (m.at[s] == a) return s;
    m.at[m.na] = a;
    return m.na++;
}

__device__ void load_mol(const ShakeArgs& A, int ic, Mol& m) {
    m.n = A.cons_n[ic];
    m.na = 0;
    for (int s = 0; s < m.n; ++s) {
        m.ca[s] = slot_of(m, A.cons[ic * 6 + 2 * s]);
        m.cb[s] = slot_of(m, A.cons[ic * 6 + 2 * s + 1]);
        m.l2[s] = A.clen2[ic * 3 + s];
    }
}

// One sweep over the molecule; returns true when some constraint was corrected.
// moved bit s = 1: atom in slot s was NOT moved in the previous sweep (reference `moved` = 1).
__device__ bool sweep(const View& v, const ShakeArgs& A, const Mol& m, double* px, double* py, double* pz,
                      const double* ox, const double* oy, const double* oz, unsigned& moved, int* fail,
                      double* gacc = nullptr) {
    unsigned moving = (1u << kMaxAt) - 1u;
    bool upd = false;
    for (int s = 0; s < m.n; ++s) {
        const int a = m.ca[s], b = m.cb[s];
        if (((moved >> a) & 1u) && ((moved >> b) & 1u)) continue;
        double pxab = minimg(px[a] - px[b], v.lx, v.lxi);
        double pyab = minimg(py[a] - py[b], v.ly, v.lyi);
        double pzab = minimg(pz[a] - pz[b], v.lz, v.lzi);
        const double rabsq = m.l2[s];
        const double diffsq = rabsq - (pxab * pxab + pyab * pyab + pzab * pzab);
        if (fabs(diffsq) > rabsq * A.tol2) {
            const double rx = minimg(ox[a] - ox[b], v.lx, v.lxi);
            const double ry = minimg(oy[a] - oy[b], v.ly, v.lyi);
            const double rz = minimg(oz[a] - oz[b], v.lz, v.lzi);
            const double rpab = rx * pxab + ry * pyab + rz * pzab;
            if (rpab < rabsq * A.rptol) {
                *fail = 1;
                return upd;
            }
            double rma = v.mii[m.at[a]], rmb = v.mii[m.at[b]];
            const double aux = diffsq / (2.0 * (rma + rmb) * rpab);
            if (gacc) gacc[s] += aux;
            rma = rma * aux;
            rmb = rmb * aux;
            px[a] = px[a] + rx * rma; py[a] = py[a] + ry * rma; pz[a] = pz[a] + rz * rma;
            px[b] = px[b] - rx * rmb; py[b] = py[b] - ry * rmb; pz[b] = pz[b] - rz * rmb;
            moving &= ~((1u << a) | (1u << b));
            upd = true;
        }
    }
    // frozen atoms keep moved = 1
    unsigned frozen = 0;
    for (int s = 0; s < m.na; ++s)
        if (m.at[s] >= A.nmove) frozen |= 1u << s;
    moved = moving | frozen;
    return upd;
}

__device__ void gather(const View& v, const ShakeArgs& A, const Mol& m, double* px, double* py, double* pz,
                       double* ox, double* oy, double* oz, unsigned& moved) {
    moved = 0;
    for (int s = 0; s < m.na; ++s) {
        const int a = m.at[s];
        px[s] = v.x[a]; py[s] = v.y[a]; pz[s] = v.z[a];
        const int k = a - A.nliqa;
        ox[s] = A.xo[k]; oy[s] = A.yo[k]; oz[s] = A.zo[k];
        if (a >= A.nmove) moved |= 1u << s;
    }
}

// Bonds of a 3-constraint molecule after the Verlet step (p) and before it (r), minimum-imaged.
__device__ void bonds(const View& v, const Mol& m, const double* px, const double* py, const double* pz,
                      const double* ox, const double* oy, const double* oz, double p[3][3], double r[3][3]) {
    for (int c = 0; c < 3; ++c) {
        const int a = m.ca[c], b = m.cb[c];
        p[c][0] = minimg(px[a] - px[b], v.lx, v.lxi);
        p[c][1] = minimg(py[a] - py[b], v.ly, v.lyi);
        p[c][2] = minimg(pz[a] - pz[b], v.lz, v.lzi);
        r[c][0] = minimg(ox[a] - ox[b], v.lx, v.lxi);
        r[c][1] = minimg(oy[a] - oy[b], v.ly, v.lyi);
        r[c][2] = minimg(oz[a] - oz[b], v.lz, v.lzi);
    }
}

// Network seed: predicted accumulated multipliers applied along the old bonds, the same update as a
// SHAKE correction (src/move.f90:498-510) with all three constraints at once.
__device__ void apply_seed(const View& v, const Mol& m, const float y[3], double* px, double* py, double* pz,
                           const double r[3][3], double* gacc) {
    for (int c = 0; c < 3; ++c) {
        const int a = m.ca[c], b = m.cb[c];
        const double ma = v.mii[m.at[a]], mb = v.mii[m.at[b]];
        if (ma + mb <= 0.0) continue;
        const double g = (double)y[c] / (ma + mb);
        gacc[c] += g;
        px[a] += r[c][0] * ma * g; py[a] += r[c][1] * ma * g; pz[a] += r[c][2] * ma * g;
        px[b] -= r[c][0] * mb * g; py[b] -= r[c][1] * mb * g; pz[b] -= r[c][2] * mb * g;
    }
}

__device__ void seed_mol(const View& v, const Mol& m, const float* W, const float f[9], double* px, double* py,
                         double* pz, const double r[3][3], double* gacc) {
    float y[3];
    mlp::forward(W, f, y);
    apply_seed(v, m, y, px, py, pz, r, gacc);
}

__device__ void load_weights(const float* mlpw, float* W) {
    for (int i = threadIdx.x; i < mlp::NW; i += blockDim.x) W[i] = i < mlp::NPARAM ? mlp::bf16r(mlpw[i]) : mlpw[i];
}

__global__ void k_shake_init(ShakeArgs A) {
    A.sweeps_out[0] = 0;
    A.sweeps_out[1] = 1;
}

__global__ void k_shake_last(View v, ShakeArgs A) {
    // one block: the seeding network's forward pass for the last molecule runs on the block's
    // threads (identical outputs to the one-thread form of k_shake_mol); its sweeps on thread 0
    __shared__ float W[mlp::NW];
    __shared__ float fin[mlp::NI], hid[2 * mlp::NH], yout[mlp::NO];
    __shared__ int seeded;
    if (A.mlpw) load_weights(A.mlpw, W);
    Mol m;
    load_mol(A, A.ncons - 1, m);
    double px[kMaxAt], py[kMaxAt], pz[kMaxAt], ox[kMaxAt], oy[kMaxAt], oz[kMaxAt];
    unsigned moved = 0;
    double r[3][3];
    if (threadIdx.x == 0) {
        gather(v, A, m, px, py, pz, ox, oy, oz, moved);
        seeded = A.mlpw && m.n == 3 ? 1 : 0;
        if (seeded) {
            double p[3][3];
            float f[9];
            bonds(v, m, px, py, pz, ox, oy, oz, p, r);
            mlp::features(p, r, m.l2, f);
            for (int k = 0; k < mlp::NI; ++k) fin[k] = f[k];
        }
    }
    __syncthreads();
    if (seeded) mlp::forward_block(W, fin, hid, yout);
    if (threadIdx.x != 0) return;
    if (seeded) {
        double g[3] = {0, 0, 0};
        const float y[3] = {yout[0], yout[1], yout[2]};
        apply_seed(v, m, y, px, py, pz, r, g);
    }
    int fail = 0, s = 0;
    bool done = false;
    while (!done && s <= A.maxit) {
        done = !sweep(v, A, m, px, py, pz, ox, oy, oz, moved, &fail);
        ++s;
        if (fail) break;
    }
    A.sweeps_out[0] = s;
    A.sweeps_out[1] = done ? 1 : 0;
}

__global__ void k_shake_mol(View v, ShakeArgs A) {
    __shared__ float W[mlp::NW];
    if (A.mlpw) load_weights(A.mlpw, W);
    __syncthreads();
    const int ic = blockIdx.x * blockDim.x + threadIdx.x;
    if (ic >= A.ncons) return;
    Mol m;
    load_mol(A, ic, m);
    double px[kMaxAt], py[kMaxAt], pz[kMaxAt], ox[kMaxAt], oy[kMaxAt], oz[kMaxAt];
    unsigned moved;
    gather(v, A, m, px, py, pz, ox, oy, oz, moved);
    double gacc[3] = {0.0, 0.0, 0.0};
    float feat[9];
    const bool model = m.n == 3 && (A.mlpw || A.rec);
    if (model) {
        double p[3][3], r[3][3];
        bonds(v, m, px, py, pz, ox, oy, oz, p, r);
        mlp::features(p, r, m.l2, feat);
        if (A.mlpw) seed_mol(v, m, W, feat, px, py, pz, r, gacc);
    }
    int fail = 0;
    int s = 0;
    const int nsw = A.clean ? A.maxit + 1 : A.sweeps_out[0];
    bool converged = false;
    for (; s < nsw; ++s) {
        const bool upd = sweep(v, A, m, px, py, pz, ox, oy, oz, moved, &fail, gacc);
        if (fail) {
            atomicCAS(&v.status[ST_SHAKE_RPTOL], 0, 1 + ic * 8 + 0);
            break;
        }
        if (!upd) {
            converged = true;
            if (A.clean) break;
        }
    }
    if (A.clean) {
        atomicMax(&A.sweeps_out[0], s + (converged ? 1 : 0));
        if (!converged) atomicAnd(&A.sweeps_out[1], 0);
    }
    for (int t = 0; t < m.na; ++t) {
        const int a = m.at[t];
        if (a < A.nmove) {
            v.x[a] = px[t]; v.y[a] = py[t]; v.z[a] = pz[t];
        }
    }
    if (A.rec) {
        float* o = A.rec + (size_t)ic * 16;
        for (int k = 0; k < 9; ++k) o[k] = model ? feat[k] : 0.f;
        for (int c = 0; c < 3; ++c)
            o[9 + c] = model ? (float)(gacc[c] * (v.mii[m.at[m.ca[c]]] + v.mii[m.at[m.cb[c]]])) : 0.f;
        o[12] = (float)(s + (converged && A.clean ? 1 : 0));
        o[13] = o[14] = o[15] = 0.f;
    }
}

// Single-thread copy of the reference loop for topologies with shared moving atoms.
__global__ void k_shake_seq(View v, ShakeArgs A, int* moving, int* movd) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int nsurf = A.nmove - A.nliqa;
    for (int i = 0; i < nsurf; ++i) {
        moving[i] = 1;
        movd[i] = 0;
    }
    bool done = false;
    int ite = 0;
    while (!(done || ite > A.maxit)) {
        bool any = false;
        for (int ic = 0; ic < A.ncons; ++ic) {
            done = true;
            for (int s = 0; s < A.cons_n[ic]; ++s) {
                const int ia = A.cons[ic * 6 + 2 * s], ib = A.cons[ic * 6 + 2 * s + 1];
                const int ma = ia < A.nmove ? movd[ia - A.nliqa] : 1;
                const int mb = ib < A.nmove ? movd[ib - A.nliqa] : 1;
                if (ma * mb != 0) continue;
                const double pxab = minimg(v.x[ia] - v.x[ib], v.lx, v.lxi);
                const double pyab = minimg(v.y[ia] - v.y[ib], v.ly, v.lyi);
                const double pzab = minimg(v.z[ia] - v.z[ib], v.lz, v.lzi);
                const double rabsq = A.clen2[ic * 3 + s];
                const double diffsq = rabsq - (pxab * pxab + pyab * pyab + pzab * pzab);
                if (fabs(diffsq) > rabsq * A.tol2) {
                    const int ka = ia - A.nliqa, kb = ib - A.nliqa;
                    const double rx = minimg(A.xo[ka] - A.xo[kb], v.lx, v.lxi);
                    const double ry = minimg(A.yo[ka] - A.yo[kb], v.ly, v.lyi);
                    const double rz = minimg(A.zo[ka] - A.zo[kb], v.lz, v.lzi);
                    const double rpab = rx * pxab + ry * pyab + rz * pzab;
                    if (rpab < rabsq * A.rptol) {
                        v.status[ST_SHAKE_RPTOL] = 1 + ic * 8 + s;
                        A.sweeps_out[0] = ite + 1;
                        A.sweeps_out[1] = 0;
                        return;
                    }
                    double rma = v.mii[ia], rmb = v.mii[ib];
                    const double aux = diffsq / (2.0 * (rma + rmb) * rpab);
                    rma *= aux;
                    rmb *= aux;
                    v.x[ia] += rx * rma; v.y[ia] += ry * rma; v.z[ia] += rz * rma;
                    v.x[ib] -= rx * rmb; v.y[ib] -= ry * rmb; v.z[ib] -= rz * rmb;
                    if (ia < A.nmove) moving[ia - A.nliqa] = 0;
                    if (ib < A.nmove) moving[ib - A.nliqa] = 0;
                    done = false;
                    any = true;
                }
            }
        }
        if (A.clean) done = !any;
        ++ite;
        for (int i = 0; i < nsurf; ++i) {
            movd[i] = moving[i];
            moving[i] = 1;
        }
    }
    A.sweeps_out[0] = ite;
    A.sweeps_out[1] = done ? 1 : 0;
}

}  // namespace

int shake_setup(Ctx& c, const mdg_sysdesc* s) {
    const View& v = c.v;
    c.ncons = (int)s->ncons;
    const int nsurfold = v.ntota - v.nliqa;
    c.d_xold = (double*)dalloc(c, sizeof(double) * std::max(nsurfold, 1));
    c.d_yold = (double*)dalloc(c, sizeof(double) * std::max(nsurfold, 1));
    c.d_zold = (double*)dalloc(c, sizeof(double) * std::max(nsurfold, 1));
    c.d_kps = (double*)dalloc(c, sizeof(double) * std::max(v.nit, 1));
    c.d_ft_in = (double*)dalloc(c, sizeof(double) * 3 * std::max(v.nmove - v.nriga, 1));
    c.d_sweeps = (int*)dalloc(c, sizeof(int) * 2);
    c.d_seq_flags = (int*)dalloc(c, sizeof(int) * 2 * std::max(v.nmove - v.nliqa, 1));
    c.d_mlpw = (float*)dalloc(c, sizeof(float) * mlp::NW);
    c.d_shake_rec = (float*)dalloc(c, sizeof(float) * 16 * std::max<int64_t>(s->ncons, 1));
    if (c.ncons == 0) return MDG_OK;
    std::vector<int> cons(6 * c.ncons, -1), cn(c.ncons, 0);
    std::vector<double> l2(3 * c.ncons, 0.0);
    std::vector<int> owner(v.nmove, -1);
    c.shake_seq = 0;
    for (int ic = 0; ic < c.ncons; ++ic) {
        const int64_t it = s->ictype[ic] - 1;
        if (it < 0 || it >= s->ntype) return set_err(&c, MDG_E_ARG, "ictype out of range");
        const int nc = (int)s->nconst[it];
        if (nc > MDG_SMX) return set_err(&c, MDG_E_ARG, "more than 3 constraints per molecule");
        cn[ic] = nc;
        for (int k = 0; k < nc; ++k) {
            const int64_t a = s->constra[k + MDG_SMX * ic] - 1, b = s->constrb[k + MDG_SMX * ic] - 1;
            if (a < v.nliqa || b < v.nliqa || a >= v.ntota || b >= v.ntota)
                return set_err(&c, MDG_E_ARG, "constraint atom outside the surface/wall range");
            cons[ic * 6 + 2 * k] = (int)a;
            cons[ic * 6 + 2 * k + 1] = (int)b;
            const double L = s->length[it + s->ntype * k];
            l2[ic * 3 + k] = L * L;
            for (int64_t at : {a, b})
                if (at < v.nmove) {
                    if (owner[at] >= 0 && owner[at] != ic) c.shake_seq = 1;
                    owner[at] = ic;
                }
        }
    }
    c.d_cons = (int*)dalloc(c, sizeof(int) * cons.size());
    c.d_clen2 = (double*)dalloc(c, sizeof(double) * l2.size());
    c.d_cons_n = (int*)dalloc(c, sizeof(int) * cn.size());
    MDG_CUDA(cudaMemcpy(c.d_cons, cons.data(), sizeof(int) * cons.size(), cudaMemcpyHostToDevice));
    MDG_CUDA(cudaMemcpy(c.d_clen2, l2.data(), sizeof(double) * l2.size(), cudaMemcpyHostToDevice));
    MDG_CUDA(cudaMemcpy(c.d_cons_n, cn.data(), sizeof(int) * cn.size(), cudaMemcpyHostToDevice));
    return MDG_OK;
}

__global__ void k_shake_status(View v, const int* sweeps) {
    if (!sweeps[1]) v.status[ST_SHAKE_MAXIT] = 1;
    v.status[ST_SWEEPS] = sweeps[0];
}

// Verlet + SHAKE on the device state (x/y/z, xold) with forces d_ft (3 x (nmove - nriga)).
void shake_launch(Ctx& c, const double* d_ft, bool kps_clear) {
    const View& v = c.v;
    const int nsurf = v.nmove - v.nliqa;
    if (!kps_clear) cudaMemsetAsync(c.d_kps, 0, sizeof(double) * v.nit, c.stream);
    if (nsurf > 0)
        k_verlet<<<(nsurf + kNT - 1) / kNT, kNT, 0, c.stream>>>(v, d_ft, c.d_xold, c.d_yold, c.d_zold, c.d_kps);
    if (c.ncons == 0) return;
    const int clean = (c.quirks & MDG_QUIRK_CLEAN_SHAKE_DONE) ? 1 : 0;
    ShakeArgs A{c.ncons, c.maxit, clean, v.nliqa, v.nmove, c.tol2, c.rptol, c.d_cons, c.d_clen2,
                c.d_cons_n, c.d_xold, c.d_yold, c.d_zold, c.d_sweeps, c.shake_model ? c.d_mlpw : nullptr,
                c.shake_record ? c.d_shake_rec : nullptr};
    if (c.shake_seq) {
        k_shake_seq<<<1, 1, 0, c.stream>>>(v, A, c.d_seq_flags, c.d_seq_flags + std::max(nsurf, 1));
        k_shake_status<<<1, 1, 0, c.stream>>>(v, c.d_sweeps);
        return;
    }
    if (clean) {
        k_shake_init<<<1, 1, 0, c.stream>>>(A);
    } else {
        k_shake_last<<<1, 128, 0, c.stream>>>(v, A);
    }
    // one thread per molecule, 64 per block: the molecules are few (8,192 at most in the benchmark
    // systems) and their sweeps are chains of FP64 operations, so they are spread over the SMs
    k_shake_mol<<<(c.ncons + kMolNT - 1) / kMolNT, kMolNT, 0, c.stream>>>(v, A);
    k_shake_status<<<1, 1, 0, c.stream>>>(v, c.d_sweeps);
}

}  // namespace mdg
