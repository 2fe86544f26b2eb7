// ctx.h - device-side state of one md_sim system and the launch interface of each phase.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/mdgpu.h"

namespace mdg {

// Offsets in the FP64 accumulator block (after elj[nijt], eqq[nijt]).
enum AccSlot {
    ACC_UEWA = 0,
    ACC_EWQLL,
    ACC_ULR,
    ACC_DIPZ,
    ACC_MAXD,   // max squared displacement since the last rebuild
    ACC_FWS,    // 9 values: fwsx(-1:1), fwsy(-1:1), fwsz(-1:1)
    ACC_FWS0 = ACC_FWS + 9,  // sum of all forces x,y,z (fws*(0))
    ACC_NSLOT = ACC_FWS0 + 3
};

// Thermostat and step scalars of the resident mode (device array c.d_thermo).
enum ThermoSlot {
    TH_S = 0,      // s0..s4
    TH_RS = 5,     // rs0..rs4
    TH_KP = 10,
    TH_KW,
    TH_KE,
    TH_HTOT,
    TH_SFT,
    TH_SFR,
    TH_UCONF,
    TH_TEMPNOW,
    TH_PRESS,
    TH_STEPS,
    TH_REBUILDS,
    TH_N = 24
};

// Plain view of the device arrays, passed to kernels by value.
struct View {
    int nrig, nriga, nliqa, nmove, nwall, ntota, nit, nijt, nltype, nheads;
    int bulk;   // MDG_BULK semantics in the real-space loops
    int pbcz;   // z minimum image in the neighbour list
    double lx, ly, lz, lxi, lyi, lzi, lwh;
    double rcut, rcutsq, skin, alfa, spii, facq, rskinsq, dshsq;
    // atoms
    double *x, *y, *z;         // ntota
    double *rsx, *rsy, *rsz;   // nmove
    double *cx, *cy, *cz;      // nrig (current centres of mass)
    double *ocx, *ocy, *ocz;   // nrig at the last rebuild
    double *ox, *oy, *oz;      // flexible atoms at the last rebuild (index - nriga)
    const double *q, *mii, *mi;
    const int* type;           // 0-based site type, ntota
    // type tables
    const int* nsi;            // nit
    const int* ijt;            // nit*nit, 0-based pair index, [it*nit + jt]
    const int* vdw;            // nijt
    const double *eps, *sig, *aa, *rhoi, *cc;
    // forces
    double *fx, *fy, *fz;      // nmove
    // heads and lists
    const int* head_atom;      // nheads
    int* nb;                   // nheads * maxnb: partner atoms j > i
    int* nbcnt;                // nheads
    int maxnb;
    int* wnb;                  // nheads * maxwnb: wall atoms
    int* wnbcnt;
    int maxwnb;
    const int* excl_off;       // ntota + 1
    const int* excl;
    // accumulators and status
    double* acc;               // 2*nijt + ACC_NSLOT
    int* status;               // ST_NWORDS
};

// Cell grid used by the list build.
struct Grid {
    int nc[3];
    double cs[3];
    double org[3];
    int periodic[3];
    int ncell;
};

struct KSet {
    int nk = 0;          // valid k vectors (reference order: l outer, m, n innermost)
    int nrow = 0;        // (l, m) rows
    int klmax = 0, kmmax = 0, knmax = 0;
    double pipix = 0, pipiy = 0, pipiz = 0;
    // device
    int4* row = nullptr;          // per row: l, m, n_first, k_first (n runs n_first..|n_first| or 1..)
    int* row_nlen = nullptr;      // per row: number of n
    double* ak = nullptr;         // nk
    double2* qw = nullptr;        // nk static wall structure factor
    double2* s = nullptr;         // nk moving-atom structure factor (accumulated)
    double2* c = nullptr;         // nk: Ak * conj(S_total)
    int3* kvec = nullptr;         // nk: (l, m, n)
    int* witem_row = nullptr;     // k_sfac work items: row
    int* witem_n0 = nullptr;      //                    n offset inside the row
    int nwork = 0, tile = 0, splits = 1, atoms_per_split = 0, sfac_smem = 0, force_smem = 0;
    std::vector<int4> h_row;      // host copies of row and row_nlen
    std::vector<int> h_nlen;
};

// Per-step packed atom records of the mixed-precision real-space kernels (pair_mx.cu).
struct Pk {
    uint4* P = nullptr;     // fixed-point x, y (z if periodic) | FP32 z hi; w = type | sign(z) << 31
    float4* Q = nullptr;    // rs offset, charge
    float* zlo = nullptr;   // z - z_hi when z is not periodic
    float4* F = nullptr;    // j-side force accumulator (moving atoms)
    uint4* tc = nullptr;    // reciprocal-sum records (moving atoms), or nullptr
    float* cmax = nullptr;  // scale of the reciprocal sum's pass-2 operand, cleared here for it
    double* part = nullptr; // per-block slab dipole shares of the packing kernel
    float sx = 0, sy = 0, sz = 0;  // box edge / 2^32
    int zper = 0;
    // the pair loops' parameters in FP32, rounded once on the host (a conversion from FP64 in
    // every warp of the pair kernels kept the GPU's narrow FP64 pipe busy)
    float alfa = 0, spii = 0, facq = 0, rcutsq = 0;
    const float* par = nullptr;  // per pair type: vdW kind (int bits), sig, eps, aa, rhoi, cc
};

// Measurement arrays on the device and their bin parameters (measure.cu), passed by value.
struct MeasView {
    double rdeli = 0, lwh = 0, rfrst = 0, rscnd = 0, lxh = 0, lyh = 0, cx4 = 0, cy2 = 0;
    int lmax = 0, L = 0, ntz = 0, langmax = 201, lgx = 0, lgy = 0, l2d = 0, slab = 1;
    unsigned long long *ngc = nullptr, *nefipos = nullptr, *ngang = nullptr, *ngz = nullptr;
    unsigned long long *ng2d1 = nullptr, *ng2d2 = nullptr;
    unsigned long long* cnt = nullptr;  // calls_force, calls_do, out_of_range
    double *efipos = nullptr, *tefipos = nullptr;
    double* ndip = nullptr;  // 4 x L: ndipx, ndipy, ndipz, ndipsq
    double* mu = nullptr;    // 3 x L scratch of one measure_do call
    double* ftot = nullptr;  // 9: ftotx(-1:1), ftoty(-1:1), ftotz(-1:1)
    double* pos = nullptr;   // 3 x nmove positions handed to mdg_measure_do
    const int* ang_mt = nullptr;  // molecule type (0-based) of each angle term
};

struct Meas {
    bool init = false, force_hist = false, profiles = false;
    int smem = 0;  // bytes of the per-block ngc/efipos histogram of the pair loops, 0 = global atomics
    MeasView m;
};

// Launch plan of the tensor-core reciprocal sum (recip_tc.cu).
struct TcPlan {
    bool ready = false;
    int KN = 0, NN = 0, NP = 0, KS = 0, KM = 0, NM = 0;
    int ncols1 = 0, mtiles = 0, nchunk2 = 0, chunk1 = 0, nsplit1 = 0, grid1x = 0, rtot = 0, tpc1 = 0, smem1 = 0, smem2 = 0;
    int ntile2 = 0, nparts2 = 0, cper2 = 0, grid2 = 0, nlist2 = 0, mult1 = 2, nst2 = 2;
    int G1 = 4;  // n-side pass 1: groups of 16 atoms per TMEM accumulation chain
    int4* row2 = nullptr;    // pass-2 rows, sorted by their K-step range (nchunk2 x kRC, padded)
    int* rorig2 = nullptr;   // pass-2 row -> row of the k set (-1: padding)
    float* rowsc = nullptr;  // per row of the k set: max |C| max(1, |n|) of this evaluation
    float* rsc2 = nullptr;   // the same in pass-2 order (written by the operand packing)
    int* nlen2 = nullptr;
    int4* chunk2 = nullptr;  // per pass-2 chunk: image byte offset, first K step, K steps
    int4* items2 = nullptr;  // per pass-2 CTA: atom tile, first chunk, end chunk, whole tile (1) or piece (0)
    int nitems2 = 0;
    int4* items2_k[2] = {nullptr, nullptr};  // the item tables: pieces (system alone), whole tiles (throughput)
    int nitems2_k[2] = {0, 0}, zero2_k[2] = {0, 0};
    std::vector<int> h_chunk_ks;  // K steps of each pass-2 chunk (host)
    bool throughput = false;      // planned for throughput among many systems (recip_tc_throughput)
    int mult_alone = 2;           // pass-1 CTA multiple of the plan for the system alone
    int zero2 = 0;           // first atom of the tiles split into pieces (their forces are summed atomically)
    size_t img_bytes = 0;
};

struct Ctx {
    mdg_sysdesc sysc;   // sizes only (pointers not kept)
    View v{};
    Grid grid{}, wgrid{};
    KSet ks;
    TcPlan tcp;
    Pk pk;
    uint4* d_tc_atoms = nullptr;        // fixed-point phases + charge per moving atom
    unsigned char* d_tc_img = nullptr;  // packed C(k) operand chunks
    float* d_tc_cmax = nullptr;         // scale of the packed C(k) operand
    float* d_tc_part = nullptr;         // pass-1 partial sums [split][col][row]
    float2* d_tc_cf = nullptr;          // C(k) in FP32 for the pass-2 operand
    double* d_frc = nullptr;            // 3 x nmove reciprocal forces of the tensor-core sum, merged after the join
    cudaStream_t side = nullptr;        // second stream: the reciprocal sum runs beside the real-space loops
    cudaStream_t side2 = nullptr;       // third stream: the head-wall loop beside the head-head loop
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_fork2 = nullptr, ev_join2 = nullptr, ev_list = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;  // the context's stream while a caller's stream is in use
    int device = 0;
    int precision = MDG_FP64;
    int variant = MDG_SLAB;
    uint32_t quirks = 0;
    double uself = 0, ewqWW = 0;
    double lr_tab[9][16];  // flr_l, flr_w, flr_lja, flr_ljc, flr_bua, flr_buc, flr_bur, ulr_l, ulr_w per type
    double* d_lr = nullptr;  // same table on the device [9][nit]
    // device buffers owned here
    std::vector<void*> owned;
    // list build scratch
    int *d_cell_start = nullptr, *d_cell_count = nullptr, *d_head_cell = nullptr;
    int* d_wcell_start = nullptr;
    float4* d_cpos = nullptr;     // wrapped head positions sorted by cell, w = atom index bits
    float4* d_wpos = nullptr;     // wrapped wall positions sorted by cell
    double4* d_hpos = nullptr;    // wrapped head positions in head order
    // SHAKE
    int ncons = 0, ncmax = 0, shake_seq = 0, maxit = 10;
    double tol2 = 1e-8, rptol = 0.85;
    int* d_cons = nullptr;        // ncons * 3 * 2 atom indices (0-based), -1 unused
    double* d_clen2 = nullptr;    // ncons * 3 squared lengths
    int* d_cons_n = nullptr;      // ncons constraints per molecule
    double *d_xold = nullptr, *d_yold = nullptr, *d_zold = nullptr;  // ntota - nliqa
    double* d_kps = nullptr;      // nit
    double* d_ft_in = nullptr;    // 3 x (nmove - nriga) forces handed to SHAKE
    int* d_sweeps = nullptr;      // [0] sweeps, [1] done
    int* d_seq_flags = nullptr;   // moving/moved of the sequential SHAKE
    float* d_mlpw = nullptr;      // SHAKE-seeding network parameters
    float* d_shake_rec = nullptr; // ncons x 12 recorded features / multipliers
    bool shake_model = false, shake_record = false;
    int pair_blocks = 0;          // blocks of the real-space loops (0: by head count); autotuned
    int pred_parts = 0;           // blocks (dipole shares) of the last packing predictor launch
    int pack_parts = 0;           // blocks of the last packing kernel launch, and its forced rebuild
    bool pack_force = false;
    Meas meas;                    // measurement histograms (measure.cu)
    std::vector<int64_t> h_moltypen, h_nt, h_ns, h_itype;  // molecule types and site types (cfgio.cu)
    int64_t widom_cap = 0;        // Widom insertion scratch (widom.cu)
    double *d_widom_pos = nullptr, *d_widom_rot = nullptr, *d_widom_res = nullptr;
    int* d_widom_n = nullptr;
    float* d_widom_akf = nullptr;   // Ak in FP32 (mixed form)
    float2* d_widom_qsf = nullptr;  // S + S_wall in FP32 (mixed form)
    float4* d_widom_rsf = nullptr;  // rs offsets and charges in FP32 (mixed form)
    bool widom_attr = false;
    std::vector<int> h_ang_mt;    // molecule type of each angle term
    int64_t nfreed = 0;
    // angles
    int nang_terms = 0;
    int* d_ang = nullptr;         // per term i, j, k (0-based), type slot
    double *d_ang_kt = nullptr, *d_ang_th = nullptr;
    std::vector<double> h_qs_wall;  // wall charges (for the static structure factor)
    double *d_ft = nullptr, *d_fc = nullptr, *d_tq = nullptr;  // force_sum outputs
    bool alloc_failed = false;
    int batch_stage = 0;          // captures of a phase-ordered replica batch: 1 up to the list, 2 after the loops
    bool debug_sync = false;
    // resident mode
    bool resident = false;
    mdg_rigid body{};
    double *d_xd = nullptr, *d_c = nullptr, *d_q = nullptr, *d_w = nullptr, *d_a = nullptr;
    double *d_thermo = nullptr, *d_isum = nullptr;
    unsigned* d_done = nullptr;   // block counters of the fused integrator kernels
    std::vector<std::pair<void*, size_t>> snap_regions;
    char* d_snap = nullptr;
    cudaGraphExec_t graph_exec = nullptr;   // resident step
    cudaGraphExec_t force_exec = nullptr;   // force evaluation of the drop-in path
    int graph_steps = 0;
    int64_t kernels_per_step = 0;
    // host staging (pinned)
    double* h_acc = nullptr;
    int* h_status = nullptr;
    double* h_small = nullptr;  // pinned: SHAKE's per-type kinetic sums (nit) + its sweep words (1)
    std::string err;
};

// ---- phase launchers (each .cu file) -------------------------------------------------
// nnlist.cu
int nnlist_setup(Ctx& c, const double* x0, const double* y0, const double* z0);
void nnlist_trigger(Ctx& c, bool force);
void nnlist_build(Ctx& c);
// The list build of several systems as five launches in all (replica batches); descriptors and
// block tables on the device, rewritten from the systems' current views by the setup.
struct LsBatch {
    void* d_buf = nullptr;
    size_t cap = 0;
    void* reps = nullptr;
    int* first[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    int nblk[5] = {0, 0, 0, 0, 0};
    int nrep = 0;
};
int ls_batch_setup(LsBatch& lb, const std::vector<Ctx*>& cs, std::string& err);
void ls_batch_launch(const LsBatch& lb, cudaStream_t st);
void ls_batch_free(LsBatch& lb);
// pair.cu
void pair_forces_fp64(Ctx& c);
void wall_forces_fp64(Ctx& c);
void surf_partition(Ctx& c);
void lr_tail(Ctx& c);
// pair_mx.cu
void pack_setup(Ctx& c);
// per-evaluation records of the real-space loops and the reciprocal sum; clears the FP64 forces
// and sums the slab dipole M_z
// reset_status: also clear the list overflow words; the energy sums are always cleared.
// defer_close: the dipole and the rebuild decision are left to pack_close_launch (next, on the
// stream that builds the list)
void pack_mixed(Ctx& c, bool force_rebuild, bool reset_status = false, bool defer_close = false);
void pack_close_launch(Ctx& c);
void pairs_mixed(Ctx& c, bool merge);  // head-head pairs into F (then merged into the FP64 forces)
void walls_mixed(Ctx& c, bool concurrent = false);  // head-wall pairs into F (concurrent: beside the other branches)
// F (+ frc, + the slab dipole term) into the FP64 forces, F cleared
void merge_mixed(Ctx& c, const double* frc, bool dipole);
// The head-head and head-wall loops of several systems (each in the concurrent form: walls, no
// surface atoms) as one launch each per z treatment; descriptors and item tables on the device.
struct RsBatch {
    struct Group {
        void* reps = nullptr;     // device: one view + packed records per system
        int* first_p = nullptr;   // device: first head-head item of each system, nrep + 1
        int* first_w = nullptr;   // device: first head-wall item of each system, nrep + 1
        int nrep = 0, items_p = 0, items_w = 0;
        size_t smem_p = 0, smem_w = 0;
    };
    Group g[2];                   // z not periodic / periodic in the real-space loops
    void* d_buf = nullptr;
    size_t cap = 0;
    int blocks_p = 152 * 8, blocks_w = 152 * 8;  // measured best on 64 slab replicas (152 to 1216 tried)
};
// (Re)writes the descriptors from the systems' current views (after any list regrowth).
int rs_batch_setup(RsBatch& rb, const std::vector<Ctx*>& cs, std::string& err);
void rs_batch_launch(const RsBatch& rb, cudaStream_t s_pair, cudaStream_t s_wall);
void rs_batch_free(RsBatch& rb);
// recip.cu
int recip_setup(Ctx& c, int64_t kmax, const double* x0, const double* y0, const double* z0);
void recip_fp64(Ctx& c);
int recip_forces_noalloc(const double* x, const double* y, const double* z, const double* q, int64_t n,
                         double lx, double ly, double lz, double alpha, int64_t kmax, double* fx, double* fy,
                         double* fz, double* uewa, cudaStream_t st);
const char* recip_noalloc_error();
void recip_energy_launch(Ctx& c);
// recip_tc.cu
int recip_tc_setup(Ctx& c);
int tc_plan_pass1(Ctx& c, int tpc, int mult);
// on: the fewest CTAs per pass (pass 1 in chunks of about 1024 atoms, pass 2 whole tiles), for a
// system stepped among many in one graph; off: back to the plan for the system alone.  Drops the
// context's captured graphs.
int recip_tc_throughput(Ctx& c, bool on);
void recip_tc(Ctx& c);
int umma_selftest(int n, int k, const float* a, const float* b, float* d, std::string& err);
// mlp.cu
int mlp_nw();
int mlp_forward_host(const float* w, const float* X, int64_t n, float* Y, std::string& err);
int mlp_grad_host(const float* w, const float* X, const float* Y, int64_t n, float* grad, float* loss, std::string& err);
int mlp_train_host(const float* X, const float* Y, int64_t n, int epochs, int batch, float lr, uint64_t seed,
                   float* w_out, float* loss_out, std::string& err);
// epilogue.cu
void dipole_correction(Ctx& c);
void angle_forces(Ctx& c);
void force_sum(Ctx& c, double* d_ft, double* d_fc, double* d_tq);
void merge_force_sum(Ctx& c, const double* frc);  // mixed form without bend angles: merge + force_sum
// measure.cu
int measure_init(Ctx& c, const mdg_measure_params* p, mdg_measure_dims* d);
void measure_zero(Ctx& c);
void measure_force_real(Ctx& c);   // after the real-space loops
void measure_force_fouri(Ctx& c);  // after force_fouri's slab term
void measure_force_intra(Ctx& c);  // after force_intra
void measure_force_sum(Ctx& c);    // after force_sum
void measure_do_launch(Ctx& c, const double* x, const double* y, const double* z);
int measure_get(Ctx& c, mdg_measure_out* o);
// mdgpu.cu
int resident_alloc(Ctx& c);
// widom.cu
int widom(Ctx& c, const mdg_widom_params* p, double* seed, double* pave, int64_t* inave, int64_t* done);
// shake.cu
int shake_setup(Ctx& c, const mdg_sysdesc* s);
void shake_launch(Ctx& c, const double* d_ft, bool kps_clear = false);  // kps_clear: kps already zeroed
// integrate.cu
// Arrays of one drop-in call moved by one kernel through the GPU's mapping of pinned host memory
// (hostio.cu); 8-byte words.
struct IoBatch {
    static constexpr int kMax = 24;
    const unsigned long long* src[kMax];
    unsigned long long* dst[kMax];
    long n[kMax];
    int nseg = 0;
    long nmax = 0;
};
// Queues the move of nwords 8-byte words host -> device (h2d) or back: into the batch when the
// host side is pinned, else as a cudaMemcpyAsync on the context's stream.
cudaError_t io_add(Ctx& c, IoBatch& b, void* dst, const void* src, long nwords, bool h2d);
void io_flush(Ctx& c, IoBatch& b);  // launches the batch's copy kernel and empties it
cudaError_t pin_host_range(void* p, size_t bytes);  // cudaHostRegister + the registry of io_add
cudaError_t unpin_host_range(void* p);

// clear_acc / clear_kps: also zero the energy sums of the force call next / the surface atoms'
// kinetic sums of the SHAKE call after it
// pack: also write the mixed form's per-atom records, the slab dipole and the list rebuild
// decision for the force call next (in place of its packing kernel; no surface atoms)
void predict_launch(Ctx& c, bool clear_acc = false, bool clear_kps = false, bool pack = false);
// after a packing predictor: its packing close (dipole, rebuild decision) and the thermostat predictor
void step_close_launch(Ctx& c);
// merge: also the mixed form's final merge + force_sum, left out of the force phases before it
void correct_launch(Ctx& c, bool merge = false);

int set_err(Ctx* c, int code, const std::string& msg);
void* dalloc(Ctx& c, size_t bytes);

}  // namespace mdg

namespace mdg {
// Captured graphs hold kernel arguments by value: drop them when a pointer or a launch shape
// they captured changes (list capacity, tuning, stream, measurement switches, a new state).
inline void drop_graphs(Ctx& c) {
    if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
    if (c.force_exec) cudaGraphExecDestroy(c.force_exec);
    c.graph_exec = nullptr;
    c.force_exec = nullptr;
}
}  // namespace mdg

// The opaque context of the C ABI is the device state itself.
struct mdg_ctx : mdg::Ctx {};

#define MDG_CUDA(call)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return ::mdg::set_err(&c, MDG_E_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)
