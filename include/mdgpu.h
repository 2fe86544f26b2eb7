/*
 * mdgpu.h - C ABI of the GB300 force / neighbour-list / SHAKE library for md_sim.
 *
 * The reference reaches its hot path through three argument-less Fortran calls that talk
 * through module globals:
 *   call force_get     src/main.f90:42,62      (definition src/forcem.f90:93-129)
 *   call nnlist_make   src/forcem.f90:250      (definition src/nnlist.f90:92-165)
 *   call move_shake    src/move.f90:376        (definition src/move.f90:408-529)
 * and prepares them once in force_init (src/forcem.f90:54-81, which calls nnlist_init
 * src/nnlist.f90:14-90) and move_shake_init (src/move.f90:385-406).
 *
 * This header replaces those calls with plain C entry points.  Every pointer is a host
 * pointer to a contiguous array exactly as the Fortran modules hold it (real*8 -> double,
 * integer*8 -> int64_t), so an ISO_C_BINDING interface can pass the module arrays straight
 * through.  Atom and type indices inside the arrays stay 1-based, as in the reference.
 * Errors are returned as negative codes (the reference calls `stop`); mdg_last_error()
 * gives the message.  A context owns all device memory; calls on one context are
 * synchronous on return and must come from one host thread at a time.
 */
#ifndef MDGPU_H
#define MDGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MDG_SMX 3 /* max sites / constraints / angles per molecule, src/global.f90:7 */

/* return codes */
#define MDG_OK 0
#define MDG_E_ARG (-1)           /* bad argument or inconsistent system description */
#define MDG_E_CUDA (-2)          /* CUDA runtime failure or no device */
#define MDG_E_LIST_OVERFLOW (-3) /* neighbour list capacity exceeded, src/nnlist.f90:136-139,157-160 */
#define MDG_E_SHAKE_MAXIT (-4)   /* 'shake(): Too many constraint iterations!', src/move.f90:526 */
#define MDG_E_SHAKE_RPTOL (-5)   /* 'Constraint failure', src/move.f90:487-496 */
#define MDG_E_NAN (-6)           /* non-finite force or energy */
#define MDG_E_UNSUPPORTED (-7)   /* feature outside this library (e.g. Couette-pulled walls) */

/* force-field variants */
#define MDG_SLAB 0 /* src/forcem.f90: z not periodic in real space, wall LR tail, EW3DC dipole term */
#define MDG_BULK 1 /* src/forcem_back.f90: z minimum image in pair/angle loops, no LR tail, no EW3DC */

/* arithmetic of the force phases */
#define MDG_FP64 0  /* every phase in FP64 (reproduces the reference) */
#define MDG_MIXED 1 /* FP32 pairs with compensated sums, tensor-core reciprocal sum, FP64 state */

/* quirk switches (mdg_params.quirks); default 0 reproduces the reference */
#define MDG_QUIRK_CLEAN_SHAKE_DONE 1u /* SHAKE stops when no molecule moved (global test) instead of
                                         the reference's last-molecule test, src/move.f90:458 */

/*
 * System description: the sysdef/config module tables the hot path reads
 * (src/sysdef.f90:9-59 after sysdef_init :356-457).  Arrays are borrowed for the duration of
 * mdg_create only.
 */
typedef struct mdg_sysdesc {
    /* counts, src/sysdef.f90:16-25 */
    int64_t ntype;                                          /* molecule types */
    int64_t nrig, nriga, nliqa, nsurf, nmove, nwall, ntota; /* molecules / atom ranges */
    int64_t ngogo;                                          /* atoms in the k-space sum (= nmove) */
    int64_t nit, nijt;                                      /* site types, site-type pairs */
    int64_t nltype;                                         /* last liquid molecule type */
    int64_t ncons, nang;                                    /* constrained molecules, angle molecules */
    /* per molecule type, length ntype */
    const int64_t* moltypen; /* 0 rigmol, 1 atmol, 2 surfmol, 3 crystal */
    const int64_t* nt;       /* molecules of the type */
    const int64_t* ns;       /* sites per molecule */
    const int64_t* nst;      /* site types per molecule type */
    const int64_t* nconst;   /* constraints per molecule */
    const int64_t* nangt;    /* angles per molecule */
    const int64_t* nss_wall; /* nss(ntype,:): sites per crystal site type, max(2,nst(ntype))
                                entries (missing ones 0) */
    /* per site type, length nit */
    const int64_t* nsi; /* sites handled by a head atom of this type (0: not a head) */
    /* per site-type pair */
    const int64_t* ijtype; /* nit x nit, column-major, 1-based pair id */
    const int64_t* vdwnum; /* nijt: 0 none, 1 Lennard-Jones, 2 Buckingham */
    const double* eps;     /* nijt, 4*epsilon */
    const double* sig;     /* nijt, sigma**6 */
    const double* aa;      /* nijt, Buckingham A */
    const double* rhoi;    /* nijt, Buckingham 1/rho */
    const double* cc;      /* nijt, Buckingham C */
    /* per atom, length ntota */
    const int64_t* itype; /* 1-based site type */
    const double* qs;     /* charge in e */
    const double* mi;     /* mass, internal units (src/sysdef.f90:378-379) */
    const double* mii;    /* inverse mass, 0 for frozen sites */
    /* constraints and angles */
    const int64_t* ictype;  /* ncons: molecule type of each constrained molecule */
    const int64_t* constra; /* MDG_SMX x ncons, column-major, 1-based atoms */
    const int64_t* constrb; /* MDG_SMX x ncons */
    const double* length;   /* ntype x MDG_SMX, column-major: constraint lengths */
    const int64_t* iatype;  /* nang */
    const int64_t* ang1;    /* MDG_SMX x nang */
    const int64_t* ang2;
    const int64_t* ang3;
    const double* kt;    /* ntype x MDG_SMX: bend force constants */
    const double* theta; /* ntype x MDG_SMX: equilibrium angles, radians */
    /* geometry, src/config.f90:13 and src/sysdef.f90:46 */
    double lx, ly, lz;
    double cx, cy, cz, lw; /* crystal cell and wall-to-wall slab width */
    double dt;             /* time step, fs */
} mdg_sysdesc;

typedef struct mdg_params {
    double rcut;   /* real-space cutoff, A */
    double skin;   /* Verlet skin, A */
    double alpha;  /* Ewald alpha, 1/A; <= 0 selects 3.09/rcut as src/forcem.f90:59 */
    int64_t kmax;  /* reciprocal cutoff index */
    double dshsq;  /* squared wall shift per step (Couette), 0 otherwise, src/nnlist.f90:28 */
    int32_t variant;    /* MDG_SLAB or MDG_BULK */
    int32_t pbc_z_list; /* 1: the neighbour list also applies the z minimum image (bulk boxes);
                           the reference never does, src/nnlist.f90:129,150 */
    int32_t precision;  /* MDG_FP64 or MDG_MIXED */
    uint32_t quirks;    /* MDG_QUIRK_* bits */
    int64_t list_capacity;  /* max head-head pairs kept; 0 = sized automatically */
    int64_t wlist_capacity; /* max head-wall pairs kept; 0 = sized automatically */
    int32_t shake_maxit;    /* SHAKE sweep limit; 0 selects 10, src/move.f90:398 */
    double shake_tol2;      /* relative tolerance; 0 selects 1e-8, src/move.f90:399 */
    double shake_rptol;     /* failure ratio; 0 selects 0.85, src/move.f90:400 */
} mdg_params;

/*
 * Energies and statistics of one force evaluation (the scalars force_sum leaves,
 * src/forcem.f90:969-1124).  elj/eqq are caller arrays of length nijt, or NULL.
 * fws*[0..2] hold the reference's fws*(-1:1).
 */
typedef struct mdg_energies {
    double* elj;
    double* eqq;
    double uewa, urf, ulr, uself, uconf, uavex, press, vir;
    double ewqLL, ewqWL, ewqWW;
    double fwsx[3], fwsy[3], fwsz[3];
} mdg_energies;

typedef struct mdg_ctx mdg_ctx;

/* Replaces force_init (src/forcem.f90:54-81) with nnlist_init (src/nnlist.f90:14-90) and
 * move_shake_init (src/move.f90:385-406): uploads the tables and the frozen wall sites, builds
 * the k-vector set, Ak, the static wall structure factors, the self energy, the wall
 * long-range tail tables and the first neighbour list.  x0/y0/z0: ntota; cx0..: nrig. */
int mdg_create(const mdg_sysdesc* sys, const mdg_params* prm, const double* x0, const double* y0,
               const double* z0, const double* cx0, const double* cy0, const double* cz0,
               mdg_ctx** out);

void mdg_destroy(mdg_ctx* ctx);

/* Message of the last failure on this context (or of the last failed mdg_create if ctx is NULL). */
const char* mdg_last_error(const mdg_ctx* ctx);

/* Replaces nnlist_make (src/nnlist.f90:92-165): unconditional rebuild from the given positions.
 * x0..: nmove (or ntota), cx0..: nrig.  ipack/wpack receive the list lengths (may be NULL). */
int mdg_nnlist_make(mdg_ctx* ctx, const double* x0, const double* y0, const double* z0,
                    const double* cx0, const double* cy0, const double* cz0, int64_t* ipack,
                    int64_t* wpack);

/* Copies the current neighbour lists out as 1-based (i, j) pairs, in no particular order.
 * Arrays may be NULL; at most cap / wcap pairs are written.  Returns MDG_OK. */
int mdg_get_lists(mdg_ctx* ctx, int64_t* li, int64_t* lj, int64_t cap, int64_t* wi, int64_t* wj,
                  int64_t wcap, int64_t* ipack, int64_t* wpack);

/* The context's k set (force_fouri_init's selection, src/forcem.f90:743-776): kl, km, kn of each
 * valid k vector in the reference's order and its Ak, for the first min(cap, nk) entries (any
 * pointer may be NULL).  Returns nk, or a negative error code.  Mirrors the oracle's table of the
 * same name, so that tests can compare the two k sets. */
int64_t mdg_kvectors(mdg_ctx* ctx, int32_t* kl, int32_t* km, int32_t* kn, double* ak, int64_t cap);

/* Replaces force_get (src/forcem.f90:93-129) with force_real, force_fouri, force_intra and the
 * serial force_sum (src/forcem_3d.f90:1031-1058), including the rebuild trigger
 * (src/forcem.f90:245-250).
 *   x0,y0,z0   in  ntota site positions (walls are read at create and ignored here)
 *   cx0..      in  nrig centres of mass
 *   rsx,rsy,rsz in/out nmove site offsets; on return rsx(1:3) hold the last rigid molecule's
 *                  sites relative to its centre, as force_sum leaves them (src/forcem.f90:1006)
 *   ftx,fty,ftz out nmove-nriga forces on the flexible atoms (Fortran ftx(nriga+1:nmove))
 *   fcx..,tx..  out nrig centre-of-mass forces and torques
 *   fx,fy,fz    out optional (NULL to skip): nmove site forces before the rigid-body reduction
 *   e           out energies and wall statistics (NULL to skip) */
int mdg_force_get(mdg_ctx* ctx, const double* x0, const double* y0, const double* z0,
                  const double* cx0, const double* cy0, const double* cz0, double* rsx,
                  double* rsy, double* rsz, double* ftx, double* fty, double* ftz, double* fcx,
                  double* fcy, double* fcz, double* tx, double* ty, double* tz, double* fx,
                  double* fy, double* fz, mdg_energies* e);

/* Replaces move_shake (src/move.f90:408-529): Verlet step of the surface atoms plus SHAKE.
 *   x0,y0,z0      in/out ntota positions (atoms nliqa+1..nmove are updated)
 *   xold,yold,zold in/out ntota-nliqa previous positions (Fortran xold(nliqa+1:ntota))
 *   ftx,fty,ftz   in  nmove-nriga forces (Fortran ftx(nriga+1:nmove))
 *   kps           out nit per-type kinetic sums (may be NULL)
 *   tkps          out SHAKE temperature (may be NULL)
 *   sweeps        out SHAKE sweeps executed (may be NULL) */
int mdg_shake(mdg_ctx* ctx, double* x0, double* y0, double* z0, double* xold, double* yold,
              double* zold, const double* ftx, const double* fty, const double* ftz, double* kps,
              double* tkps, int32_t* sweeps);

/* Transfers of the two calls above.  Arrays in pinned host memory are read and written by the
 * GPU in place (one gather and one scatter kernel per call, over NVLink-C2C on a Grace-Blackwell
 * node); other arrays are copied through the driver's staging buffers, with the same results but
 * a few microseconds more per array.  mdg_pin_host pins an existing host array (for example a
 * Fortran module array, once after allocation); mdg_unpin_host releases it before it is freed.
 * No counterpart in the reference (its arrays never leave the host). */
int mdg_pin_host(void* p, int64_t bytes);
int mdg_unpin_host(void* p);

/* ---------------------------------------------------------------------------------------------
 * Resident mode: the whole MD step on the device.  The integrator that the reference keeps in
 * Fortran (move_predict / move_correct, src/move.f90:48-383) runs as device kernels around the
 * same force and SHAKE phases, so that many steps run without host traffic.
 * ------------------------------------------------------------------------------------------- */

/* Integrator state (src/config.f90:20-51 and the thermostat of src/config.f90:17), in time-step
 * units as after config_init (src/config.f90:76-90).  Host arrays of the caller. */
typedef struct mdg_state {
    double *x0, *y0, *z0;          /* ntota positions */
    double *xd[4], *yd[4], *zd[4]; /* ntota: x1..x4 etc. (atoms nriga+1..nliqa are integrated) */
    double *cx[5], *cy[5], *cz[5]; /* nrig: cx0..cx4 */
    double *q[4][5];               /* nrig: q[c][k] = q(c+1)k, i.e. q10..q14, q20..q24, ... */
    double *wx[5], *wy[5], *wz[5]; /* nrig: body angular velocity and its derivatives */
    double *xold, *yold, *zold;    /* ntota - nliqa */
    double *rsx, *rsy, *rsz;       /* nmove site offsets */
    double s[5], rs[5];            /* thermostat s0..s4, rs0..rs4 */
} mdg_state;

/* Rigid-water body and ensemble (src/sysdef.f90:443-452, src/main.f90:123-128). */
typedef struct mdg_rigid {
    double xbody[3], ybody[3], zbody[3]; /* site coordinates in the principal-axis frame */
    double mw;                           /* water mass, internal units */
    double inxx, inyy, inzz;             /* principal moments of inertia */
    double temper;                       /* K; -1 selects NVE (src/move.f90:173) */
} mdg_rigid;

/* Scalars of the last step of mdg_run (the values prntout reports, src/main.f90:320-335). */
typedef struct mdg_report {
    double kp, kw, ke, htot, tempnow, uconf, tkps, press;
    int64_t steps, rebuilds;
    int32_t last_sweeps;
} mdg_report;

/* Uploads the full integrator state; the positions of frozen atoms are taken from mdg_create. */
int mdg_set_state(mdg_ctx* ctx, const mdg_rigid* body, const mdg_state* st);

/* Downloads the integrator state (for config_output / measure_do). */
int mdg_get_state(mdg_ctx* ctx, mdg_state* st);

/* Runs nsteps of move_predict -> force_get -> move_correct (-> move_shake when there are surface
 * atoms), src/main.f90:58-68, entirely on the device.  rep may be NULL. */
int mdg_run(mdg_ctx* ctx, int64_t nsteps, mdg_report* rep);

/* Stream-ordered variant of mdg_run: queues nsteps on the context's stream and returns without
 * waiting or checking.  mdg_check waits for the queued work and reports list overflow, SHAKE
 * failures and non-finite energies of everything queued since the previous check (a list
 * overflow is reported, not repaired: rerun the steps with mdg_run). */
int mdg_run_async(mdg_ctx* ctx, int64_t nsteps);
int mdg_check(mdg_ctx* ctx, mdg_report* rep);

/* ---------------------------------------------------------------------------------------------
 * Host integrator for drop-in callers.  The reference keeps move_predict / move_correct
 * (src/move.f90:48-383) in Fortran around its force call; a caller that replaces only force_get
 * (and move_shake) with this library keeps them too.  These calls are that integrator on host
 * arrays for callers written in C or C++: the molecules split into ranges over the host threads
 * (OpenMP; MDG_HOST_THREADS, read at mdg_host_gear_create, else all cores the process may use,
 * one thread below 2,048 molecules), kinetic sums in molecule order on one thread, so results do
 * not depend on the thread count; no device memory, the reference's arithmetic order.  A drop-in
 * step is
 *     mdg_host_predict -> mdg_force_get (x0.., cx[0].., rsx..) -> mdg_host_correct
 *     (-> mdg_shake when there are surface atoms)
 * and reproduces the resident step of mdg_run to rounding.
 * ------------------------------------------------------------------------------------------- */
typedef struct mdg_host_gear mdg_host_gear;
/* sys: the description given to mdg_create (counts and masses are copied); body: the rigid water. */
int mdg_host_gear_create(const mdg_sysdesc* sys, const mdg_rigid* body, mdg_host_gear** out);
void mdg_host_gear_destroy(mdg_host_gear* g);
/* move_predict (src/move.f90:48-217) on st in place: flexible atoms nriga+1..nliqa, centres,
 * quaternions (normalised), body angular velocities, rotation matrices (kept in g), water site
 * positions and H offsets rsx(ix+2:ix+3), the thermostat predictor; kinetic energies, htot. */
int mdg_host_predict(mdg_host_gear* g, mdg_state* st);
/* move_correct (src/move.f90:220-383) with the outputs of the mdg_force_get call on the predicted
 * positions: ft* (nmove - nriga), fc* and t* (nrig), and that call's uconf. */
int mdg_host_correct(mdg_host_gear* g, mdg_state* st, const double* ftx, const double* fty, const double* ftz,
                     const double* fcx, const double* fcy, const double* fcz, const double* tx, const double* ty,
                     const double* tz, double uconf);
/* kp, kw, ke, htot (last predict), tempnow, uconf (last correct); the other fields are untouched. */
int mdg_host_report(const mdg_host_gear* g, mdg_report* rep);

/* ---------------------------------------------------------------------------------------------
 * The reference's input files read on the host, for callers written in C or C++: sysdef_input /
 * sysdef_init (src/sysdef.f90:83-340, :356-457) on the .fld and .top files and config_input /
 * config_init (src/config.f90:174-242, :55-95, config_quatsite :303-329) on the .cfg file (whose
 * first record also gives the box).  dt: the time step in fs (the .inp value).  The handle owns
 * the description's tables, the rigid-water body (temper -1: set it from the .inp for NVT) and the
 * state, ready for mdg_create (positions: the state's x0/y0/z0 and cx[0]..) and mdg_set_state or
 * the drop-in loop; molnames serves mdg_write_cfg / mdg_read_cfg.  Errors (file, format, the
 * reference's sysdef_input checks) return MDG_E_ARG with the message in mdg_last_error(NULL).
 * ------------------------------------------------------------------------------------------- */
typedef struct mdg_sysdef mdg_sysdef;
int mdg_sysdef_load(const char* fld_path, const char* top_path, const char* cfg_path, double dt, mdg_sysdef** out);
const mdg_sysdesc* mdg_sysdef_desc(const mdg_sysdef* sd);
const mdg_rigid* mdg_sysdef_rigid(const mdg_sysdef* sd);
mdg_state* mdg_sysdef_state(mdg_sysdef* sd);
const char* const* mdg_sysdef_molnames(const mdg_sysdef* sd);
void mdg_sysdef_free(mdg_sysdef* sd);

/* Kernel launches of one resident-mode step (counted in the captured step graph; 0 before the
 * first mdg_run / mdg_run_async). */
int64_t mdg_kernels_per_step(const mdg_ctx* ctx);

/* Puts all work of the context on the caller's CUDA stream (a cudaStream_t; NULL restores the
 * context's own stream), so that callers can order and time it with their own events. */
int mdg_set_stream(mdg_ctx* ctx, void* stream);

/* Phase timing: runs the force phases `reps` times on the current state (positions unchanged,
 * list rebuilt every repetition) and writes the mean device time in ms of each phase:
 * [0] list rebuild, [1] head-head pairs, [2] head-wall pairs, [3] reciprocal sum,
 * [4] other force terms and force_sum, [5] integrator (resident mode, else 0), [6] SHAKE. */
#define MDG_NPHASE 7
int mdg_phase_times(mdg_ctx* ctx, int reps, double* ms);

/* ---------------------------------------------------------------------------------------------
 * Autotuner (no reference counterpart): times whole force evaluations of the context's current
 * configuration for candidate launch parameters (real-space grid size; structure-factor row
 * tiles per CTA and atom splits) and keeps the fastest.  reps evaluations per candidate.
 * ------------------------------------------------------------------------------------------- */
typedef struct mdg_tuning {
    int32_t pair_blocks;      /* real-space blocks (0: one warp per head) */
    int32_t tc_rows_per_cta;  /* structure-factor (l, m) rows per CTA (mixed precision) */
    int32_t tc_atom_splits;   /* structure-factor atom chunks */
    float ms_before, ms_after;
} mdg_tuning;
int mdg_autotune(mdg_ctx* ctx, int32_t reps, mdg_tuning* out);

/* ---------------------------------------------------------------------------------------------
 * Replica batches (no reference counterpart; the reference runs one system per MPI job).
 * Independent contexts in resident mode, stepped together by one CUDA graph launch, so that many
 * small systems share the GPU: by default their real-space loops run as one kernel over all of
 * them (mdg_batch_set_mode below).
 * ------------------------------------------------------------------------------------------- */
typedef struct mdg_batch mdg_batch;
/* ctxs: n contexts on one device, each after mdg_set_state; they stay owned by the caller and
 * must outlive the batch. */
int mdg_batch_create(mdg_ctx* const* ctxs, int n, mdg_batch** out);
void mdg_batch_destroy(mdg_batch* b);
const char* mdg_batch_last_error(const mdg_batch* b);
int mdg_batch_set_stream(mdg_batch* b, void* stream);
/* nsteps batch steps (every replica one MD step each), checked every 64 steps; a replica whose
 * neighbour list overflows redoes its chunk alone with larger lists.  reps: n reports or NULL. */
int mdg_batch_run(mdg_batch* b, int64_t nsteps, mdg_report* reps);
/* nsteps graph launches on the batch stream, no checks (for timing; then mdg_check per context) */
int mdg_batch_run_async(mdg_batch* b, int64_t nsteps);
/* Replicas in a batch share the GPU: while a batch exists, the tensor-core reciprocal passes of its
 * mixed-precision replicas are planned for throughput (the fewest CTAs: pass 1 in chunks of about
 * 1024 atoms, pass 2 whole atom tiles) instead of spreading each replica over every SM;
 * mdg_batch_destroy restores each replica's own plan.
 * Graph form of the batch (the next run builds it):
 *   MDG_BATCH_PHASES (default)  phase order: the head-head and head-wall loops of all replicas in
 *       the mixed form with walls and no surface atoms run as one persistent kernel each over all
 *       their heads (pair_blocks / wall_blocks blocks; 0 = 1216), between the replicas' own list
 *       builds and their merge, corrector and SHAKE; other replicas step as in their own graphs;
 *   MDG_BATCH_GRAPHS  every replica's own step graph as a parallel child graph. */
#define MDG_BATCH_GRAPHS 0
#define MDG_BATCH_PHASES 1
int mdg_batch_set_mode(mdg_batch* b, int mode, int pair_blocks, int wall_blocks);
/* replicas whose real-space loops ran in the batch's kernels at the last graph build */
int mdg_batch_phased(const mdg_batch* b);

/* ---------------------------------------------------------------------------------------------
 * Configuration files and checkpoints of the resident state.
 * mdg_write_cfg writes the state in the reference's configuration format (config_output,
 * src/config.f90:244-301, records of write_rigmol/atmol/surfmol/crystal/thermostat :484-590):
 * derivatives back to 1 fs units, Fortran E15.8 fields, or with full_precision != 0 the same
 * layout with 17 significant digits (list-directed input reads both).  molnames: ntype molecule
 * names as in the .fld file.  Crystal sites are written with their site-type code (1 or 2).
 * mdg_read_cfg reads such a file (config_input :174-242, then config_init :55-95 and
 * move_shake_init, src/move.f90:394-396) and installs it as the resident state (mdg_set_state);
 * names, kinds and counts must match the context; wall positions stay those of mdg_create.
 * mdg_checkpoint_save / _load write and read the resident state in binary (every integrator,
 * SHAKE and thermostat array and the step counters), so that a run continues from it as from the
 * state it saved; the neighbour list is rebuilt at the first step after a load.
 * ------------------------------------------------------------------------------------------- */
int mdg_write_cfg(mdg_ctx* ctx, const char* path, const char* const* molnames, int full_precision);
int mdg_read_cfg(mdg_ctx* ctx, const char* path, const char* const* molnames, const mdg_rigid* body);
int mdg_checkpoint_save(mdg_ctx* ctx, const char* path);
int mdg_checkpoint_load(mdg_ctx* ctx, const char* path);

/* ---------------------------------------------------------------------------------------------
 * Learned SHAKE seed.  A small network (9 -> 64 -> 64 -> 3, SiLU) maps rotation-invariant features
 * of a 3-constraint molecule's unconstrained and previous bond vectors to the multipliers that
 * SHAKE accumulates for it; the prediction is applied as one SHAKE-type correction before the
 * sweeps, which then iterate to the unchanged tolerance.  Parameters are a float blob of
 * mdg_mlp_nw() values (weights used rounded to BF16, FP32 accumulation).
 * ------------------------------------------------------------------------------------------- */
int mdg_mlp_nw(void);
/* Seeds every later SHAKE step of the context with the network w (n = mdg_mlp_nw()); n = 0 stops. */
int mdg_shake_set_model(mdg_ctx* ctx, const float* w, int64_t n);
/* enable != 0: each SHAKE step records per constrained molecule 16 floats: 9 features, the 3
 * accumulated multipliers (scaled by the summed inverse masses of each constraint), the sweeps
 * it took, 3 zeros; mdg_shake_samples copies the last step's ncons x 16. */
int mdg_shake_record(mdg_ctx* ctx, int enable);
int mdg_shake_samples(mdg_ctx* ctx, float* out);
/* Network training and evaluation on the GPU (host arrays in and out): x is n x 9, y is n x 3.
 * mdg_mlp_train runs Adam (cosine learning-rate decay) from a seeded start and returns the blob
 * (with the input/output normalisation it computed) and the mean loss of each epoch. */
int mdg_mlp_forward(const float* w, const float* x, int64_t n, float* y);
int mdg_mlp_grad(const float* w, const float* x, const float* y, int64_t n, float* grad, float* loss);
int mdg_mlp_train(const float* x, const float* y, int64_t n, int epochs, int batch, float lr, uint64_t seed,
                  float* w_out, float* loss_out);

/* ---------------------------------------------------------------------------------------------
 * Measurement histograms.  The reference's force loops fill histograms as a side output, and
 * measure_do (src/measure.f90:270-454) adds z-profiles after every production step:
 *   ngc(nijt, 0:lmax)      site-wall pair distances, src/forcem.f90:493-495; the bulk variant
 *                          also counts the moving pairs, src/forcem_back.f90:348-349,380-382
 *   efipos(2, 0:lmax)      z force on Li/Cl-type ions (site types 3, 4) by their z bin: pair terms
 *                          src/forcem.f90:347-354,388-395, wall terms :486-489, and the whole fz of
 *                          the liquid ions after force_fouri :930-934 (slab variant only)
 *   tefipos, nefipos       final ftz of the liquid ions and their count by z bin, :1094-1098
 *   ngang(nit-2, 0:201)    bend-angle cosines by molecule type, :617-625
 *   ngz(nit-2, 0:lmax)     site z-profile; ndipx/y/z/sq(0:lmax) water dipole profile; ng2d1/2 the
 *                          near-wall 2-D maps; ftotx/y/z(-1:1) summed wall forces (measure_do)
 * measure_init (src/measure.f90:66-176) sizes the arrays from rdel and the slab width lw:
 * lmax = int(lw/rdel + 0.5) + 1.  The arrays stay on the device and accumulate until
 * mdg_measure_zero (measure_zero, :178-262).  The reference indexes without bounds checks; here a
 * sample whose bin falls outside its array is dropped and counted in out_of_range.
 * ------------------------------------------------------------------------------------------- */
typedef struct mdg_measure_params {
    double rdel;         /* bin width, A (tot.inp "rdel") */
    int32_t force_hist;  /* 1: every force evaluation adds to ngc, efipos, tefipos/nefipos, ngang */
    int32_t profiles;    /* 1: every resident step (mdg_run) ends with measure_do */
    int32_t l2d;         /* 1: measure_do also fills the near-wall 2-D maps (tot.inp "l2d") */
    int32_t pad;
    double rfrst, rscnd; /* wall distance bounds of the first and second layer of the 2-D maps */
} mdg_measure_params;

typedef struct mdg_measure_dims {
    int64_t lmax;            /* bins 0..lmax of ngc, efipos, tefipos, nefipos, ngz, ndip* */
    int64_t nijt;            /* rows of ngc */
    int64_t ntz;             /* rows of ngz, ngang, ng2d* (nit - 2) */
    int64_t langmax;         /* bins 0..langmax of ngang (201) */
    int64_t lgxmax, lgymax;  /* ng2d* bins 0..lgxmax by 0..lgymax */
} mdg_measure_dims;

/* Caller arrays, column-major as the Fortran module holds them (first index fastest); any may
 * be NULL.  The scalars are filled in always. */
typedef struct mdg_measure_out {
    int64_t* ngc;      /* nijt x (lmax+1) */
    double* efipos;    /* 2 x (lmax+1) */
    double* tefipos;   /* 2 x (lmax+1) */
    int64_t* nefipos;  /* 2 x (lmax+1) */
    int64_t* ngang;    /* ntz x (langmax+1) */
    int64_t* ngz;      /* ntz x (lmax+1) */
    double* ndipx;     /* lmax+1 each */
    double* ndipy;
    double* ndipz;
    double* ndipsq;
    int64_t* ng2d1;    /* ntz x (lgxmax+1) x (lgymax+1) */
    int64_t* ng2d2;
    double ftot[3][3]; /* ftotx, ftoty, ftotz (-1:1) */
    int64_t calls_force;   /* force evaluations accumulated */
    int64_t calls_do;      /* measure_do calls accumulated */
    int64_t out_of_range;  /* samples dropped because their bin was outside the array */
} mdg_measure_out;

/* measure_init: allocates and zeroes the arrays; dims may be NULL. */
int mdg_measure_init(mdg_ctx* ctx, const mdg_measure_params* prm, mdg_measure_dims* dims);
/* Switches the force-side histograms and the per-step profiles on or off without clearing. */
int mdg_measure_enable(mdg_ctx* ctx, int force_hist, int profiles);
int mdg_measure_zero(mdg_ctx* ctx);
/* measure_do on positions x0, y0, z0 (nmove moving atoms; NULL: the context's resident state)
 * with the wall forces of the last force evaluation. */
int mdg_measure_do(mdg_ctx* ctx, const double* x0, const double* y0, const double* z0);
int mdg_measure_get(mdg_ctx* ctx, mdg_measure_out* out);

/* ---------------------------------------------------------------------------------------------
 * Widom test-particle insertion of a water molecule (chempot, src/forcem.f90:1226-1507, set up by
 * measure_init src/measure.f90:155-175).  Each insertion puts an O at a random point of the band
 * lwmin < wall distance < lwmax (bin il of lchmax over the band), then tries 20 random
 * orientations (1 when il <= ilmid) of the rigid 3-site probe (q -0.8476 / 0.4238, O-H 1 A,
 * H-O-H from cos = -1/3) and adds exp(-u / RT) of each to pave(il), with u = real-space energy
 * (vdW and Ewald erfc of the probe against every non-H-type site within rcut of the O) + the
 * reciprocal term 0.5 Ak Re(sum_s q_s e^{ik.r_s} conj(S(k))) with S(k) of the last force
 * evaluation + the wall long-range tail of the O.  inave(il) counts the tries.  Random numbers
 * come from the reference's congruential generator (src/rndmod.f90:26-35), whose state *seed
 * the call advances exactly as the reference does.
 * Reference behaviour kept: an O position closer than 2.35 A to a water O (2 A to any other
 * site) ends the whole call (src/forcem.f90:1342 exits the insertion loop), and the slab dipole
 * term reads an uninitialised local (src/forcem.f90:1236,1477) and is left out.
 * MDG_WIDOM_SKIP_OVERLAP skips such a position instead (its orientations still draw their random
 * numbers, so the stream differs from the reference from that point on); MDG_WIDOM_EW3DC adds
 * the slab dipole term -crf sum_s q_s z_s with crf of the last evaluation.  Slab variant only.
 * ------------------------------------------------------------------------------------------- */
#define MDG_WIDOM_SKIP_OVERLAP 1u
#define MDG_WIDOM_EW3DC 2u
typedef struct mdg_widom_params {
    int64_t ichmax;   /* insertion positions per call */
    double lwmin;     /* band of distances from the walls, A (tot.inp "lwmin lwmax") */
    double lwmax;
    int64_t lchmax;   /* bins over the band */
    int64_t ilmid;    /* bins il > ilmid get 20 orientations, the others 1 */
    double temper;    /* K; <= 0 selects 300 (src/measure.f90:169-174) */
    uint32_t flags;   /* MDG_WIDOM_* */
    int32_t pad;
} mdg_widom_params;

/* One chempot call on the positions and S(k) of the last force evaluation.  pave (lchmax) and
 * inave (lchmax) are accumulated (+=); *seed is the generator state in and out; *done (may be
 * NULL) receives the positions tried. */
int mdg_widom(mdg_ctx* ctx, const mdg_widom_params* prm, double* seed, double* pave, int64_t* inave, int64_t* done);

/* Diagnostic: one tcgen05 BF16 matrix product D (128 x n) = A (128 x k) . B^T (n x k) on the
 * device with the shared-memory operand layout of the tensor-core reciprocal sum (host arrays,
 * row-major floats rounded to BF16).  Lets a caller check the tensor-core path on its GPU. */
int mdg_selftest_umma(int n, int k, const float* a, const float* b, float* d);

/* ---------------------------------------------------------------------------------------------
 * Allocation-free reciprocal sum.  This entry point has no counterpart in the reference: it is
 * offered to callers that must not allocate device memory while they run (a host that sized its
 * device memory once at start-up and may not grow it, or a framework whose caching allocator owns
 * all of the device memory).  It computes the reciprocal-space Ewald forces and energy
 * of force_fouri (src/forcem.f90:827-937, no static walls, no slab term) for n charges, with the
 * same kernels and results as the reciprocal phase of mdg_force_get.
 *
 *   x, y, z, q   in   device arrays of n doubles (positions in A, charges in e)
 *   fx, fy, fz   out  device arrays of n doubles, overwritten with the reciprocal forces
 *   uewa         out  device pointer to one double, the reciprocal energy (may be NULL)
 *   stream       CUDA stream (cudaStream_t) the work is queued on; NULL is the default stream
 * alpha and kmax as in mdg_params (alpha must be given).  Allocates nothing: its scratch is a static
 * device array of MDG_NOALLOC_MAX_K k vectors (about 2 MB) that every GPU loading the library keeps
 * until the process exits; larger k sets are rejected with MDG_E_UNSUPPORTED.  The first call on a
 * device also looks up that array's device address (a runtime query).  Calls share the one array:
 * calls whose GPU work overlaps (other streams, other
 * host threads' streams) race on it; host calls themselves are serialised.  The call returns once
 * the work is queued; errors of argument checking are returned, mdg_last_error(NULL) has the text.
 * ------------------------------------------------------------------------------------------- */
#define MDG_NOALLOC_MAX_K 32768
#define MDG_NOALLOC_MAX_ROWS 4096
int mdg_recip_forces_noalloc(const double* x, const double* y, const double* z, const double* q, int64_t n,
                             double lx, double ly, double lz, double alpha, int64_t kmax, double* fx,
                             double* fy, double* fz, double* uewa, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MDGPU_H */
