// recip.cu - reciprocal-space Ewald sum (force_fouri_init / force_fouri,
// src/forcem.f90:657-825 and :827-937), FP64.
//
// k vectors keep the reference's order and selection: l = 0..klmax outer, m, n innermost over
// the half space, kept when  real(l^2+m^2) + real(n^2 kmax^2)/real(knmax^2) < real(kmax^2)+2.01
// in single precision (src/forcem.f90:756-759).  For a fixed (l, m) the kept n form the
// contiguous range -nmax..nmax (1..nmax when l = m = 0), so the list is a sequence of rows.
//
//   k_sfac       S(k) = sum_j q_j e^{i k.r_j} over moving atoms.  Work item = (row, chunk of 8 n);
//                phase factors el/em/en of a tile of atoms are built in shared memory by the
//                same recurrences as the reference (el(l) = el(l-1)*el(1), negative powers by
//                conjugation); partial sums over atom splits meet in FP64 atomics.
//   k_kenergy    uewa, ewqLL and C(k) = Ak conj(S(k) + Sw(k)) (Sw: static walls)
//   k_kforce     f_j += sum_k Ak Im(conj(S) q_j e^{ik.r_j}) k; one thread per atom walks the rows
//                with its own phase tables in shared memory and reads C(k) as warp broadcasts.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "ctx.h"

namespace mdg {

namespace {

constexpr int kChunk = 8;     // n per work item in k_sfac
constexpr int kSfacNT = 256;
constexpr int kForceNT = 128;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 conjd(double2 a) { return make_double2(a.x, -a.y); }

struct KDims {
    int KL, KM, KN;        // table extents (positive powers 0..K)
    double px, py, pz;     // 2 pi / L
};

// Phase tables of one atom: el[0..KL], em[0..KM], en[0..KN] by recurrence.
__device__ void phase_tables(double x, double y, double z, const KDims& d, double2* el, double2* em,
                             double2* en, int which) {
    double s, c;
    if (which == 0) {
        sincos(d.px * x, &s, &c);
        const double2 e1 = make_double2(c, s);
        el[0] = make_double2(1.0, 0.0);
        if (d.KL >= 1) el[1] = e1;
        for (int l = 2; l <= d.KL; ++l) el[l] = cmul(el[l - 1], e1);
    } else if (which == 1) {
        sincos(d.py * y, &s, &c);
        const double2 e1 = make_double2(c, s);
        em[0] = make_double2(1.0, 0.0);
        if (d.KM >= 1) em[1] = e1;
        for (int m = 2; m <= d.KM; ++m) em[m] = cmul(em[m - 1], e1);
    } else {
        sincos(d.pz * z, &s, &c);
        const double2 e1 = make_double2(c, s);
        en[0] = make_double2(1.0, 0.0);
        if (d.KN >= 1) en[1] = e1;
        for (int n = 2; n <= d.KN; ++n) en[n] = cmul(en[n - 1], e1);
    }
}

__device__ __forceinline__ double2 pw(const double2* t, int k) { return k >= 0 ? t[k] : conjd(t[-k]); }
#ifdef MDG_DEBUG_BOUNDS
#define PW(t, k, lim, tag) pw((t), ((k) > (lim) || (k) < -(lim)) ? (atomicCAS(&v.status[ST_OOB], 0, (tag)), 0) : (k))
#else
#define PW(t, k, lim, tag) pw((t), (k))
#endif

// rows: (l, m, n_first, k_first); nlen: kept n in the row (n = n_first .. n_first + nlen - 1)
__global__ void __launch_bounds__(kSfacNT) k_sfac(View v, KDims d, int nrow, const int4* rows,
                                                  const int* nlen, const int* witem_row,
                                                  const int* witem_n0, int nwork, int tile,
                                                  int atoms_per_split, double2* S, int nk_total) {
    extern __shared__ double2 sm[];
    const int per = d.KL + 1 + d.KM + 1 + d.KN + 1;
    double2* tab = sm;                                  // tile * per
    double* qt = reinterpret_cast<double*>(sm + (size_t)tile * per);  // tile
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    int l = 0, m = 0, n0 = 0, nn = 0, k0 = 0;
    if (w < nwork) {
        const int r = CK(witem_row[w], nrow, 201);
        const int4 rw = rows[r];
        l = rw.x;
        m = rw.y;
        const int off = witem_n0[w];
        n0 = rw.z + off;
        k0 = rw.w + off;
        nn = min(kChunk, nlen[r] - off);
    }
    double2 acc[kChunk];
#pragma unroll
    for (int c = 0; c < kChunk; ++c) acc[c] = make_double2(0.0, 0.0);
    const int a_begin = blockIdx.y * atoms_per_split;
    const int a_end = min(v.nmove, a_begin + atoms_per_split);
    for (int t0 = a_begin; t0 < a_end; t0 += tile) {
        const int nt = min(tile, a_end - t0);
        __syncthreads();
        for (int s = threadIdx.x; s < nt * 3; s += blockDim.x) {
            const int a = s % nt, which = s / nt;
            const int at = CK(t0 + a, v.nmove, 202);
            double2* base = tab + (size_t)CK(a, tile, 203) * per;
            phase_tables(v.x[at], v.y[at], v.z[at], d, base, base + d.KL + 1, base + d.KL + 1 + d.KM + 1, which);
            if (which == 0) qt[a] = v.q[at];
        }
        __syncthreads();
        if (nn > 0) {
            for (int a = 0; a < nt; ++a) {
                const double2* base = tab + (size_t)a * per;
                const double2 el = base[CK(l, d.KL + 1, 204)];
                const double2 em = PW(base + d.KL + 1, m, d.KM, 209);
                const double2* en = base + d.KL + 1 + d.KM + 1;
                // elm = q*el*em (src/forcem.f90:874), elmn = elm*en (:879)
                const double q = qt[a];
                const double2 elm = cmul(make_double2(q * el.x, q * el.y), em);
#pragma unroll
                for (int c = 0; c < kChunk; ++c) {
                    if (c < nn) {
                        const double2 e = cmul(elm, PW(en, n0 + c, d.KN, 210));
                        acc[c].x += e.x;
                        acc[c].y += e.y;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < kChunk; ++c) {
        if (c < nn) {
            atomicAdd(&S[CK(k0 + c, nk_total, 205)].x, acc[c].x);
            atomicAdd(&S[CK(k0 + c, nk_total, 205)].y, acc[c].y);
        }
    }
}

__global__ void k_kenergy(View v, int nk, const double* ak, const double2* S, const double2* qw, double2* C) {
    double ew = 0.0, ll = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nk; k += gridDim.x * blockDim.x) {
        const double2 s = S[k];
        const double2 st = make_double2(s.x + qw[k].x, s.y + qw[k].y);
        const double a = ak[k];
        ll += a * (s.x * s.x + s.y * s.y);
        ew += a * (st.x * st.x + st.y * st.y);
        C[k] = make_double2(a * st.x, -a * st.y);
    }
    block_atomic_sum<256>(ew, &v.acc[2 * v.nijt + ACC_UEWA]);
    block_atomic_sum<256>(ll, &v.acc[2 * v.nijt + ACC_EWQLL]);
}

__global__ void __launch_bounds__(kForceNT) k_kforce(View v, KDims d, int nrow, const int4* rows,
                                                     const int* nlen, const double2* C, int nk_total) {
    extern __shared__ double2 sm[];
    const int per = d.KM + 1 + d.KN + 1;
    double2* em = sm + (size_t)CK(threadIdx.x, blockDim.x, 206) * per;
    double2* en = em + d.KM + 1;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = j < v.nmove;
    const int jj = active ? j : 0;
    phase_tables(0, v.y[jj], 0, d, nullptr, em, nullptr, 1);
    phase_tables(0, 0, v.z[jj], d, nullptr, nullptr, en, 2);
    double s, c;
    sincos(d.px * v.x[jj], &s, &c);
    const double2 el1 = make_double2(c, s);
    double2 el = make_double2(1.0, 0.0);
    int lcur = 0;
    const double q = v.q[jj];
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int r = 0; r < nrow; ++r) {
        const int4 rw = rows[r];
        while (lcur < rw.x) {
            el = cmul(el, el1);
            ++lcur;
        }
        const double2 emm = PW(em, rw.y, d.KM, 211);
        const double2 elm = cmul(make_double2(q * el.x, q * el.y), emm);
        const int n0 = rw.z, cnt = nlen[r];
        const double2* Ck = C + CK(rw.w, nk_total, 207);
        double st = 0.0, stn = 0.0;
        for (int t = 0; t < cnt; ++t) {
            const int n = n0 + t;
            const double2 e = cmul(elm, PW(en, n, d.KN, 212));
            const double2 ck = Ck[CK(t, nk_total - rw.w, 208)];
            const double f = ck.x * e.y + ck.y * e.x;  // Im(C * e), C = Ak conj(S)
            st += f;
            stn += f * (double)n;
        }
        fx += st * (d.px * (double)rw.x);
        fy += st * (d.py * (double)rw.y);
        fz += stn * d.pz;
    }
    if (active) {
        v.fx[j] += fx;
        v.fy[j] += fy;
        v.fz[j] += fz;
    }
}

}  // namespace

// Host side: k set in reference order, rows, Ak, static wall structure factors, work items.
int recip_setup(Ctx& c, int64_t kmax, const double* x0, const double* y0, const double* z0) {
    View& v = c.v;
    KSet& ks = c.ks;
    typedef std::complex<double> cd;
    const double pi_r = (double)3.1415926535898f;
    const double PH_e = (double)1.6021892e-19f, PH_Na = (double)6.022045e23f,
                 PH_eps0 = (double)8.85418782e-12f, PH_A2m = (double)1.0e-10f;
    ks.pipix = 2.0 * pi_r / v.lx;
    ks.pipiy = 2.0 * pi_r / v.ly;
    ks.pipiz = 2.0 * pi_r / v.lz;
    const double alf4i = -1.0 / (4.0 * v.alfa * v.alfa);
    const double fac = 2.0 * PH_e * PH_e * PH_Na / (PH_eps0 * PH_A2m * 1000.0 * v.lx * v.ly * v.lz);
    const double lmin = std::min(v.lx, std::min(v.ly, v.lz));
    const double rk = (double)(float)kmax;
    const int KL = (int)std::lround(rk * v.lx / lmin), KM = (int)std::lround(rk * v.ly / lmin),
              KN = (int)std::lround(rk * v.lz / lmin);
    ks.klmax = KL;
    ks.kmmax = KM;
    ks.knmax = KN;
    std::vector<int4> rows;
    std::vector<int> nlen;
    std::vector<int3> kvec;
    std::vector<double> ak;
    const float lim = (float)(kmax * kmax) + 2.01f;
    int kmmin = 0, knmin = 1;
    for (int kl = 0; kl <= KL; ++kl) {
        const double rl = ks.pipix * (double)(float)kl;
        for (int km = kmmin; km <= KM; ++km) {
            const double rm = ks.pipiy * (double)(float)km;
            int first = 0, cnt = 0;
            for (int kn = knmin; kn <= KN; ++kn) {
                volatile float a = (float)(kl * kl + km * km);
                volatile float b = (float)((int64_t)kn * kn * kmax * kmax) / (float)((int64_t)KN * KN);
                volatile float ksq = a + b;
                if (!(ksq < lim)) continue;
                const double rn = ks.pipiz * (double)(float)kn;
                const double rksq = rl * rl + rm * rm + rn * rn;
                if (cnt == 0) first = kn;
                ++cnt;
                kvec.push_back(make_int3(kl, km, kn));
                ak.push_back(fac * std::exp(rksq * alf4i) / rksq);
            }
            if (cnt > 0) {
                rows.push_back(make_int4(kl, km, first, (int)kvec.size() - cnt));
                nlen.push_back(cnt);
            }
            knmin = -KN;
        }
        kmmin = -KM;
    }
    ks.nk = (int)kvec.size();
    ks.nrow = (int)rows.size();
    // static wall structure factor, two halves summed separately as Qsumw1/Qsumw2
    std::vector<cd> q1(ks.nk, cd(0, 0)), q2(ks.nk, cd(0, 0));
    {
        std::vector<cd> el(KL + 1), em(2 * KM + 1), en(2 * KN + 1);
        const int nw = v.nwall;
        for (int w = 0; w < nw; ++w) {
            const int i = v.nmove + w;
            el[0] = em[KM] = en[KN] = cd(1, 0);
            const double tx = ks.pipix * x0[i], ty = ks.pipiy * y0[i], tz = ks.pipiz * z0[i];
            if (KL >= 1) el[1] = cd(std::cos(tx), std::sin(tx));
            if (KM >= 1) em[KM + 1] = cd(std::cos(ty), std::sin(ty));
            if (KN >= 1) en[KN + 1] = cd(std::cos(tz), std::sin(tz));
            for (int l = 2; l <= KL; ++l) el[l] = el[l - 1] * el[1];
            for (int m = 2; m <= KM; ++m) em[KM + m] = em[KM + m - 1] * em[KM + 1];
            for (int m = 1; m <= KM; ++m) em[KM - m] = std::conj(em[KM + m]);
            for (int n = 2; n <= KN; ++n) en[KN + n] = en[KN + n - 1] * en[KN + 1];
            for (int n = 1; n <= KN; ++n) en[KN - n] = std::conj(en[KN + n]);
            const double qw = c.h_qs_wall[w];
            std::vector<cd>& dst = (w < nw / 2) ? q1 : q2;
            for (int r = 0; r < ks.nrow; ++r) {
                const int4 rw = rows[r];
                const cd elm = qw * el[rw.x] * em[KM + rw.y];
                for (int t = 0; t < nlen[r]; ++t) dst[rw.w + t] += elm * en[KN + rw.z + t];
            }
        }
    }
    std::vector<double2> qw(ks.nk);
    c.ewqWW = 0.0;
    for (int k = 0; k < ks.nk; ++k) {
        const cd s = q1[k] + q2[k];
        qw[k] = make_double2(s.real(), s.imag());
        c.ewqWW += (ak[k] * s * std::conj(s)).real();
    }
    c.ewqWW *= 0.5;
    // work items of k_sfac: (row, n offset) in chunks of kChunk
    std::vector<int> wr, wn;
    for (int r = 0; r < ks.nrow; ++r)
        for (int off = 0; off < nlen[r]; off += kChunk) {
            wr.push_back(r);
            wn.push_back(off);
        }
    ks.nwork = (int)wr.size();
    const int nk1 = std::max(ks.nk, 1), nr1 = std::max(ks.nrow, 1), nw1 = std::max(ks.nwork, 1);
    ks.row = (int4*)dalloc(c, sizeof(int4) * nr1);
    ks.row_nlen = (int*)dalloc(c, sizeof(int) * nr1);
    ks.ak = (double*)dalloc(c, sizeof(double) * nk1);
    ks.qw = (double2*)dalloc(c, sizeof(double2) * nk1);
    ks.s = (double2*)dalloc(c, sizeof(double2) * nk1);
    ks.c = (double2*)dalloc(c, sizeof(double2) * nk1);
    ks.kvec = (int3*)dalloc(c, sizeof(int3) * nk1);
    ks.witem_row = (int*)dalloc(c, sizeof(int) * nw1);
    ks.witem_n0 = (int*)dalloc(c, sizeof(int) * nw1);
    ks.h_row = rows;
    ks.h_nlen = nlen;
    if (ks.nk > 0) {
        MDG_CUDA(cudaMemcpy(ks.row, rows.data(), sizeof(int4) * ks.nrow, cudaMemcpyHostToDevice));
        MDG_CUDA(cudaMemcpy(ks.row_nlen, nlen.data(), sizeof(int) * ks.nrow, cudaMemcpyHostToDevice));
        MDG_CUDA(cudaMemcpy(ks.ak, ak.data(), sizeof(double) * ks.nk, cudaMemcpyHostToDevice));
        MDG_CUDA(cudaMemcpy(ks.qw, qw.data(), sizeof(double2) * ks.nk, cudaMemcpyHostToDevice));
        MDG_CUDA(cudaMemcpy(ks.kvec, kvec.data(), sizeof(int3) * ks.nk, cudaMemcpyHostToDevice));
        MDG_CUDA(cudaMemcpy(ks.witem_row, wr.data(), sizeof(int) * ks.nwork, cudaMemcpyHostToDevice));
        MDG_CUDA(cudaMemcpy(ks.witem_n0, wn.data(), sizeof(int) * ks.nwork, cudaMemcpyHostToDevice));
    }
    // launch geometry of k_sfac: atom tile in shared memory, atom splits to fill the GPU
    const int per = (KL + 1 + KM + 1 + KN + 1) * (int)sizeof(double2) + (int)sizeof(double);
    ks.tile = std::max(8, std::min(64, (96 * 1024) / per));
    const int kblocks = (ks.nwork + kSfacNT - 1) / kSfacNT;
    int splits = std::max(1, (152 * 4 + kblocks - 1) / std::max(kblocks, 1));
    splits = std::min(splits, std::max(1, (v.nmove + ks.tile - 1) / ks.tile));
    ks.atoms_per_split = (v.nmove + splits - 1) / splits;
    ks.splits = splits;
    ks.sfac_smem = ks.tile * ((KL + 1 + KM + 1 + KN + 1) * (int)sizeof(double2) + (int)sizeof(double));
    ks.force_smem = kForceNT * (KM + 1 + KN + 1) * (int)sizeof(double2);
    MDG_CUDA(allow_max_smem(k_sfac));
    MDG_CUDA(allow_max_smem(k_kforce));
    if (ks.force_smem > 200 * 1024 || ks.sfac_smem > 200 * 1024)
        return set_err(&c, MDG_E_UNSUPPORTED, "kmax too large for the shared-memory phase tables");
    return MDG_OK;
}

void recip_energy_launch(Ctx& c) {
    KSet& ks = c.ks;
    k_kenergy<<<std::min((ks.nk + 255) / 256, 256), 256, 0, c.stream>>>(c.v, ks.nk, ks.ak, ks.s, ks.qw, ks.c);
}

void recip_fp64(Ctx& c) {
    const View& v = c.v;
    KSet& ks = c.ks;
    if (ks.nk == 0 || v.nmove == 0) return;
    KDims d{ks.klmax, ks.kmmax, ks.knmax, ks.pipix, ks.pipiy, ks.pipiz};
    cudaMemsetAsync(ks.s, 0, sizeof(double2) * ks.nk, c.stream);
    dim3 g((ks.nwork + kSfacNT - 1) / kSfacNT, ks.splits);
    k_sfac<<<g, kSfacNT, ks.sfac_smem, c.stream>>>(v, d, ks.nrow, ks.row, ks.row_nlen, ks.witem_row,
                                                   ks.witem_n0, ks.nwork, ks.tile, ks.atoms_per_split, ks.s, ks.nk);
    k_kenergy<<<std::min((ks.nk + 255) / 256, 256), 256, 0, c.stream>>>(v, ks.nk, ks.ak, ks.s, ks.qw, ks.c);
    k_kforce<<<(v.nmove + kForceNT - 1) / kForceNT, kForceNT, ks.force_smem, c.stream>>>(v, d, ks.nrow, ks.row,
                                                                                        ks.row_nlen, ks.c, ks.nk);
}

// ---------------------------------------------------------------------------------------------
// Allocation-free reciprocal sum (mdg_recip_forces_noalloc).
//
// Some callers cannot allocate device memory while they run: a host that has sized its device
// memory once at start-up and forbids later driver allocations, a framework whose caching
// allocator owns all device memory (a cudaMalloc behind its back fragments the pool and
// synchronises the device).  For them the
// structure-factor sum runs here with all of its scratch in one static device array that the
// library carries (every GPU that loads the library holds it until the process exits).  The caller
// passes device arrays in and out; nothing is allocated by this path.
// ---------------------------------------------------------------------------------------------
namespace {

constexpr int kNaMaxK = MDG_NOALLOC_MAX_K;
constexpr int kNaMaxRows = MDG_NOALLOC_MAX_ROWS;
constexpr int kNaMaxWork = kNaMaxK / kChunk + kNaMaxRows;

// byte offsets of the regions inside the scratch array
constexpr size_t kNaS = 0;                                              // double2 [MAX_K]  S(k)
constexpr size_t kNaC = kNaS + sizeof(double2) * kNaMaxK;               // double2 [MAX_K]  C(k)
constexpr size_t kNaQw = kNaC + sizeof(double2) * kNaMaxK;              // double2 [MAX_K]  zeros
constexpr size_t kNaAk = kNaQw + sizeof(double2) * kNaMaxK;             // double  [MAX_K]
constexpr size_t kNaRows = kNaAk + sizeof(double) * kNaMaxK;            // int4    [MAX_ROWS]
constexpr size_t kNaNlen = kNaRows + sizeof(int4) * kNaMaxRows;         // int     [MAX_ROWS]
constexpr size_t kNaWr = kNaNlen + sizeof(int) * kNaMaxRows;            // int     [MAX_WORK]
constexpr size_t kNaWn = kNaWr + sizeof(int) * kNaMaxWork;              // int     [MAX_WORK]
constexpr size_t kNaAcc = (kNaWn + sizeof(int) * kNaMaxWork + 255) / 256 * 256;  // double [64]
constexpr size_t kNaStatus = kNaAcc + sizeof(double) * 64;              // int [ST_NWORDS]
constexpr size_t kNaBytes = (kNaStatus + sizeof(int) * ST_NWORDS + 255) / 256 * 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

__global__ void k_noalloc_energy(const double* acc, double* uewa) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && uewa) *uewa = 0.5 * acc[ACC_UEWA];
}

std::mutex g_na_mutex;
constexpr int kNaMaxDev = 64;
unsigned char* g_na_ptr[kNaMaxDev] = {nullptr};
// host-side k tables, reused by every call (calls are serialised by g_na_mutex)
int4 g_na_rows[kNaMaxRows];
int g_na_nlen[kNaMaxRows];
double g_na_ak[kNaMaxK];
int g_na_wr[kNaMaxWork], g_na_wn[kNaMaxWork];
thread_local char g_na_err[256] = "";

int na_fail(int code, const char* msg) {
    std::snprintf(g_na_err, sizeof g_na_err, "%s", msg);
    return code;
}

}  // namespace

const char* recip_noalloc_error() { return g_na_err; }

int recip_forces_noalloc(const double* x, const double* y, const double* z, const double* q, int64_t n,
                         double lx, double ly, double lz, double alpha, int64_t kmax, double* fx, double* fy,
                         double* fz, double* uewa, cudaStream_t st) {
    if (!x || !y || !z || !q || !fx || !fy || !fz || n < 1 || n >= (1LL << 31) || kmax < 1 || alpha <= 0.0 ||
        lx <= 0.0 || ly <= 0.0 || lz <= 0.0)
        return na_fail(MDG_E_ARG, "mdg_recip_forces_noalloc: bad argument");
    std::lock_guard<std::mutex> lock(g_na_mutex);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDev)
        return na_fail(MDG_E_CUDA, "mdg_recip_forces_noalloc: no current CUDA device");
    if (!g_na_ptr[dev]) {
        // once per device, with that device current: the device address of the static scratch
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return na_fail(MDG_E_CUDA, "mdg_recip_forces_noalloc: cudaGetSymbolAddress failed");
        g_na_ptr[dev] = static_cast<unsigned char*>(p);
    }
    unsigned char* base = g_na_ptr[dev];
    // k set in the reference's order and selection (src/forcem.f90:743-776)
    const double pi_r = (double)3.1415926535898f;
    const double PH_e = (double)1.6021892e-19f, PH_Na = (double)6.022045e23f, PH_eps0 = (double)8.85418782e-12f,
                 PH_A2m = (double)1.0e-10f;
    const double pipix = 2.0 * pi_r / lx, pipiy = 2.0 * pi_r / ly, pipiz = 2.0 * pi_r / lz;
    const double alf4i = -1.0 / (4.0 * alpha * alpha);
    const double fac = 2.0 * PH_e * PH_e * PH_Na / (PH_eps0 * PH_A2m * 1000.0 * lx * ly * lz);
    const double lmin = std::min(lx, std::min(ly, lz));
    const double rk = (double)(float)kmax;
    const int KL = (int)std::lround(rk * lx / lmin), KM = (int)std::lround(rk * ly / lmin),
              KN = (int)std::lround(rk * lz / lmin);
    const float lim = (float)(kmax * kmax) + 2.01f;
    int nk = 0, nrow = 0, nwork = 0;
    int kmmin = 0, knmin = 1;
    for (int kl = 0; kl <= KL; ++kl) {
        const double rl = pipix * (double)(float)kl;
        for (int km = kmmin; km <= KM; ++km) {
            const double rm = pipiy * (double)(float)km;
            int first = 0, cnt = 0;
            for (int kn = knmin; kn <= KN; ++kn) {
                volatile float a = (float)(kl * kl + km * km);
                volatile float b = (float)((int64_t)kn * kn * kmax * kmax) / (float)((int64_t)KN * KN);
                volatile float ksq = a + b;
                if (!(ksq < lim)) continue;
                if (nk >= kNaMaxK) return na_fail(MDG_E_UNSUPPORTED, "mdg_recip_forces_noalloc: more than MDG_NOALLOC_MAX_K k vectors");
                const double rn = pipiz * (double)(float)kn;
                const double rksq = rl * rl + rm * rm + rn * rn;
                if (cnt == 0) first = kn;
                ++cnt;
                g_na_ak[nk++] = fac * std::exp(rksq * alf4i) / rksq;
            }
            if (cnt > 0) {
                if (nrow >= kNaMaxRows) return na_fail(MDG_E_UNSUPPORTED, "mdg_recip_forces_noalloc: too many k rows");
                g_na_rows[nrow] = make_int4(kl, km, first, nk - cnt);
                g_na_nlen[nrow] = cnt;
                for (int off = 0; off < cnt; off += kChunk) {
                    if (nwork >= kNaMaxWork) return na_fail(MDG_E_UNSUPPORTED, "mdg_recip_forces_noalloc: too many work items");
                    g_na_wr[nwork] = nrow;
                    g_na_wn[nwork] = off;
                    ++nwork;
                }
                ++nrow;
            }
            knmin = -KN;
        }
        kmmin = -KM;
    }
    if (nk == 0) return na_fail(MDG_E_ARG, "mdg_recip_forces_noalloc: empty k set");
    const int sfac_smem = 64 * ((KL + 1 + KM + 1 + KN + 1) * (int)sizeof(double2) + (int)sizeof(double));
    const int tile = std::max(8, std::min(64, (96 * 1024) / ((KL + 1 + KM + 1 + KN + 1) * (int)sizeof(double2) + (int)sizeof(double))));
    const int smem1 = tile * ((KL + 1 + KM + 1 + KN + 1) * (int)sizeof(double2) + (int)sizeof(double));
    const int smem2 = kForceNT * (KM + 1 + KN + 1) * (int)sizeof(double2);
    (void)sfac_smem;
    if (smem1 > 200 * 1024 || smem2 > 200 * 1024)
        return na_fail(MDG_E_UNSUPPORTED, "mdg_recip_forces_noalloc: kmax too large for the phase tables");
    auto ck = [](cudaError_t e) { return e == cudaSuccess; };
    if (!ck(allow_max_smem(k_sfac)) ||
        !ck(allow_max_smem(k_kforce)))
        return na_fail(MDG_E_CUDA, "mdg_recip_forces_noalloc: cudaFuncSetAttribute failed");
    double2* S = reinterpret_cast<double2*>(base + kNaS);
    double2* C = reinterpret_cast<double2*>(base + kNaC);
    double2* Qw = reinterpret_cast<double2*>(base + kNaQw);
    double* Ak = reinterpret_cast<double*>(base + kNaAk);
    int4* rows = reinterpret_cast<int4*>(base + kNaRows);
    int* nlen = reinterpret_cast<int*>(base + kNaNlen);
    int* wr = reinterpret_cast<int*>(base + kNaWr);
    int* wn = reinterpret_cast<int*>(base + kNaWn);
    double* acc = reinterpret_cast<double*>(base + kNaAcc);
    int* status = reinterpret_cast<int*>(base + kNaStatus);
    // the array keeps the previous call's contents: clear what the sums start from
    bool ok = ck(cudaMemcpyAsync(Ak, g_na_ak, sizeof(double) * nk, cudaMemcpyHostToDevice, st)) &&
              ck(cudaMemcpyAsync(rows, g_na_rows, sizeof(int4) * nrow, cudaMemcpyHostToDevice, st)) &&
              ck(cudaMemcpyAsync(nlen, g_na_nlen, sizeof(int) * nrow, cudaMemcpyHostToDevice, st)) &&
              ck(cudaMemcpyAsync(wr, g_na_wr, sizeof(int) * nwork, cudaMemcpyHostToDevice, st)) &&
              ck(cudaMemcpyAsync(wn, g_na_wn, sizeof(int) * nwork, cudaMemcpyHostToDevice, st)) &&
              ck(cudaMemsetAsync(S, 0, sizeof(double2) * nk, st)) &&
              ck(cudaMemsetAsync(Qw, 0, sizeof(double2) * nk, st)) &&
              ck(cudaMemsetAsync(acc, 0, sizeof(double) * 64, st)) &&
              ck(cudaMemsetAsync(status, 0, sizeof(int) * ST_NWORDS, st)) &&
              ck(cudaMemsetAsync(fx, 0, sizeof(double) * n, st)) && ck(cudaMemsetAsync(fy, 0, sizeof(double) * n, st)) &&
              ck(cudaMemsetAsync(fz, 0, sizeof(double) * n, st));
    if (!ok) return na_fail(MDG_E_CUDA, "mdg_recip_forces_noalloc: copy of the k tables failed");
    View v{};
    v.nmove = (int)n;
    v.ntota = (int)n;
    v.nijt = 0;
    v.x = const_cast<double*>(x);
    v.y = const_cast<double*>(y);
    v.z = const_cast<double*>(z);
    v.q = q;
    v.fx = fx;
    v.fy = fy;
    v.fz = fz;
    v.acc = acc;
    v.status = status;
    KDims d{KL, KM, KN, pipix, pipiy, pipiz};
    const int kblocks = (nwork + kSfacNT - 1) / kSfacNT;
    int splits = std::max(1, (152 * 4 + kblocks - 1) / std::max(kblocks, 1));
    splits = std::min(splits, std::max(1, (int)((n + tile - 1) / tile)));
    const int aps = (int)((n + splits - 1) / splits);
    k_sfac<<<dim3(kblocks, splits), kSfacNT, smem1, st>>>(v, d, nrow, rows, nlen, wr, wn, nwork, tile, aps, S, nk);
    k_kenergy<<<std::min((nk + 255) / 256, 256), 256, 0, st>>>(v, nk, Ak, S, Qw, C);
    k_kforce<<<(int)((n + kForceNT - 1) / kForceNT), kForceNT, smem2, st>>>(v, d, nrow, rows, nlen, C, nk);
    k_noalloc_energy<<<1, 32, 0, st>>>(acc, uewa);
    if (cudaGetLastError() != cudaSuccess) return na_fail(MDG_E_CUDA, "mdg_recip_forces_noalloc: launch failed");
    return MDG_OK;
}

}  // namespace mdg
