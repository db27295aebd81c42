/*
 * heatflow_gb300 — C ABI of the GB300 (sm_103a) time-stepping hot path of HeatFlow.
 *
 * The reference (ExeQuantCode/HeatFlow, Fortran 2018) has no plugin API: its hot path is a
 * set of module procedures sharing module-global state.  Each entry point below replaces one of
 * them; the citation after each declaration is the reference interface it stands in for
 * (paths relative to the reference project root).
 *
 * Conventions
 *  - Cell index I = ix + nx*(iy + ny*iz), 0-based, x fastest.  This is the reference's
 *    1-based lexicographic order (src/heatflow/mod_hmatrix.f90:71-74) minus one, i.e.
 *    Fortran grid(ix,iy,iz) == C [iz][iy][ix].
 *  - All arithmetic on the reference path is IEEE binary64; indices are int64
 *    (src/heatflow/mod_constants.f90:8-9).
 *  - Arrays passed in and out are caller-owned HOST buffers unless the name says _device.
 *    Device state is owned by the context.  Calls on one context are serialised by the
 *    caller; separate contexts are independent.
 *  - Every call returns an int status (HF_OK or an HF_E* code).  The reference prints
 *    "fatal error: NAN in ... vector" and executes `stop 1` (src/heatflow/mod_evolve.f90:70-73,
 *    82-89, 102-105, 124-127, 153-158); the matching HF_ENAN_* codes let the host do the same.
 *  - A context may hold several independent grids ("instances", hf_create_batch); state
 *    arrays of a batch are the instances' arrays concatenated in instance order.
 */
#ifndef HEATFLOW_GB300_H
#define HEATFLOW_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HF_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------------------------ */
enum {
  HF_OK = 0,
  HF_EARG = 1,        /* invalid argument or a grid the reference cannot represent */
  HF_ECUDA = 2,       /* CUDA runtime error (message via hf_last_error) */
  HF_ENOMEM = 3,      /* device allocation failed */
  HF_ESTATE = 4,      /* call order error (e.g. step before set_state) */
  HF_EDEVICE = 5,     /* a device-side check failed (see hf_last_error) */
  HF_ENAN_B = 10,     /* mod_evolve.f90:70-73   "fatal error: NAN in B vector" */
  HF_ENAN_Q = 11,     /* mod_evolve.f90:82-85   "fatal error: NAN in Q vector" */
  HF_ENAN_QDENS = 12, /* mod_evolve.f90:86-89   "fatal error: NAN in Qdens vector" */
  HF_ENAN_SCAT = 13,  /* mod_evolve.f90:102-105 "fatal error: NAN in S_CAT vector" */
  HF_ENAN_S = 14,     /* mod_evolve.f90:124-127 "fatal error: NAN in S vector" */
  HF_ENAN_X = 15      /* mod_evolve.f90:153-158 "fatal error: NAN in x tempurature vector" */
};

/* ---- solver options ---------------------------------------------------------------------- */
enum { HF_PREC_FP64 = 0, HF_PREC_MIXED = 1 };
/* HF_STOP_RECURSIVE: the reference's linbcg itol=1 rule, err = ||r_k||/||b|| on the
 * recursively updated residual, exit when err <= tol (mod_Sparse.f90:418-425).
 * HF_STOP_TRUE: exit when the true residual ||b - H x||/||b|| <= tol (FP64). */
enum { HF_STOP_RECURSIVE = 0, HF_STOP_TRUE = 1 };
/* Heat density normalisation.  HF_QDENS_HEATED_VOLUME is the reference: every cell's Q is
 * divided by the total volume of all heated cells (mod_heating.f90:164-167).
 * HF_QDENS_CELL_VOLUME divides each cell by its own volume (per-cell source amplitudes). */
enum { HF_QDENS_HEATED_VOLUME = 0, HF_QDENS_CELL_VOLUME = 1 };

typedef struct hf_problem {
  int64_t nx, ny, nz;            /* read_system, mod_inputs.f90:611 */
  double lx, ly, lz;             /* box lengths; cell length = L/n, mod_inputs.f90:619-622 */
  /* per-cell properties, length nx*ny*nz, x fastest (heatblock, mod_constructions.f90:25-31) */
  const double* kappa;           /* W/m/K */
  const double* rho;             /* kg/m^3 */
  const double* heat_capacity;   /* J/kg/K */
  const double* tau;             /* s, unscaled; the library applies tau/dt^2 (mod_setup.f90:62) */
  const double* em;              /* emissivity; NULL means 0 everywhere */
  const int64_t* iheater;        /* heater case per cell (mod_heating.f90:59-117); NULL = none */
  const double* power;           /* optional per-cell POWER replacing power_in; NULL = power_in */
  double power_in;               /* W (param.in power_in) */
  double freq;                   /* Hz (param.in freq) */
  double time_step;              /* s (param.in time_step) */
  int64_t heated_steps;          /* param.in heattime (heater case 2) */
  int32_t icattaneo;             /* 1: Cattaneo term on */
  int32_t isteady;               /* 1: steady state (alpha = 0, S = -Qdens - B) */
  int32_t periodic[3];           /* Periodicx/y/z */
  int32_t cg_face[6];            /* Neumann "CG" faces: -x,+x,-y,+y,-z,+z (CG_x_m, CG_x_p, ...) */
  double kappa_bound[6];         /* kappaBoundx1, Nx, y1, Ny, z1, Nz */
  double t_bath_face[6];         /* T_Bathx1, x2, y1, y2, z1, z2 */
  double t_bath;                 /* T_Bath (radiative loss reference temperature) */
  double t_bath_cg;              /* T_BathCG */
  double br;                     /* BR, boundary resistance factor */
  int32_t qdens_mode;            /* HF_QDENS_* */
  int32_t reserved;
} hf_problem;

typedef struct hf_solver_opts {
  int32_t precision;    /* HF_PREC_FP64 or HF_PREC_MIXED */
  int32_t criterion;    /* HF_STOP_RECURSIVE or HF_STOP_TRUE */
  double tol;           /* relative residual target (reference: 1e-32 recursive) */
  int64_t itmax;        /* max FP64 PCG iterations per step (reference: 50000) */
  double inner_tol;     /* mixed: relative reduction asked of each FP32 inner solve */
  int32_t inner_itmax;  /* mixed: max FP32 CG iterations per inner solve */
  int32_t max_refine;   /* mixed: max FP64 refinement sweeps per step */
  int32_t check_every;  /* iterations launched between host convergence polls */
  int32_t use_graph;    /* hf_run's step loop: 0 = kernels launched and polled by the host;
                           1 = the whole loop as one CUDA graph (a WHILE node around a step whose
                           solve is one persistent cooperative kernel: no host round trip);
                           2 = a CUDA graph per step with conditional WHILE/SWITCH nodes;
                           3 = as 1, but one graph launch per step (kernels visible to profilers,
                           which do not see kernels inside conditional nodes) */
  int32_t task_depth;   /* z-planes per task of the step kernels (0: 32, or 16/8/4 when the
                           grids would give fewer than 912 tasks; otherwise 4..1024) */
} hf_solver_opts;

typedef struct hf_stats {
  int64_t steps;             /* steps completed */
  int64_t iterations;        /* FP64 PCG iterations, summed over steps and instances */
  int64_t inner_iterations;  /* FP32 CG iterations (mixed), summed */
  int64_t refinements;       /* FP64 residual/refinement sweeps, summed */
  int64_t last_iter;         /* iterations of the last step (reference `iter`), max over instances */
  double last_err;           /* last step's exit criterion value, max over instances */
  double last_true_relres;   /* ||b - H x||/||b|| of the last step in FP64, max over instances */
  int64_t unconverged;       /* instance-steps that hit itmax / max_refine (the reference continues) */
  int64_t failed_step;       /* itime of the step that raised an HF_ENAN_* code, else -1 */
  int32_t status;
  int32_t failed_instance;
  int64_t kernel_launches;   /* kernels this call launched on the device */
} hf_stats;

typedef struct hf_ctx hf_ctx;

/* ---- library ---------------------------------------------------------------------------- */
int hf_abi_version(void);
const char* hf_strerror(int code);
/* Message of the last HF_ECUDA / HF_EDEVICE / HF_EARG raised on this thread. */
const char* hf_last_error(void);
/* Reference defaults: FP64, recursive criterion, tol 1e-32, itmax 50000
 * (mod_evolve.f90:142-144). */
void hf_default_opts(hf_solver_opts* opts);

/* ---- set-up ----------------------------------------------------------------------------- */
/* Replaces set_global_variables + sparse_Hmatrix (mod_setup.f90:34-83, 89-152): scales tau,
 * forms rho*c, assembles the 7-point H operator on the device (hmatrixfunc,
 * mod_hmatrix.f90:62-391) and the boundary vector (boundary, mod_boundary.f90:24-152). */
int hf_create(const hf_problem* prob, const hf_solver_opts* opts, hf_ctx** out);
/* Several independent grids of uneven sizes advanced together (one launch per kernel). */
int hf_create_batch(const hf_problem* probs, int64_t count, const hf_solver_opts* opts,
                    hf_ctx** out);
int hf_destroy(hf_ctx* ctx);
int hf_set_opts(hf_ctx* ctx, const hf_solver_opts* opts);
/* Number of instances and total cells; cells of one instance. */
int hf_get_sizes(const hf_ctx* ctx, int64_t* instances, int64_t* total_cells);
int64_t hf_instance_cells(const hf_ctx* ctx, int64_t instance);
/* Bind the context to a CUDA stream (cudaStream_t passed as void*; NULL = its own stream). */
int hf_set_stream(hf_ctx* ctx, void* stream);

/* ---- state (Temp_p = T^n, Temp_pp = T^(n-1); globe_data, mod_global.f90:10) ------------- */
/* Replaces initial_evolve (mod_init_evolve.f90:34-51).  A state written from the host (this call,
 * hf_set_state_device, hf_state_device_ready) drops the products H T^n, H T^(n-1) the library keeps
 * from its own steps, so the next two steps form their first residual with the stencil sweep. */
int hf_set_state(hf_ctx* ctx, const double* temp_p, const double* temp_pp);
int hf_get_state(hf_ctx* ctx, double* temp_p, double* temp_pp);
/* Device-resident state for zero-copy callers (torch): the context's own buffers. */
int hf_state_device(hf_ctx* ctx, double** temp_p_device, double** temp_pp_device);
/* Mark device state (written through hf_state_device) as set. */
int hf_state_device_ready(hf_ctx* ctx);

/* ---- time stepping ---------------------------------------------------------------------- */
/* Replaces simulate(itime) (mod_evolve.f90:45-177): RHS, initial guess, linear solve, state
 * rotation.  stats may be NULL. */
int hf_step(hf_ctx* ctx, int64_t itime, hf_stats* stats);
/* The time loop of heatflow.f90:67-90 without the I/O: steps itime0 .. itime0+nsteps-1. */
int hf_run(hf_ctx* ctx, int64_t itime0, int64_t nsteps, hf_stats* stats);

/* ---- parity probes (each replaces one reference routine) -------------------------------- */
/* Geometric SoA operator: y_I = diag_I x_I + sum over axes of c_a[I] x[E_a(I)] +
 * c_a[W_a(I)] x[W_a(I)], where E_a/W_a are the +/- neighbours with periodic wrap and
 * c_a[I] is the face to the + neighbour (0 where the reference stores no entry). */
int hf_get_operator(hf_ctx* ctx, double* diag, double* cx, double* cy, double* cz);
/* RHS pieces for step itime from the current state: boundary(B) (mod_boundary.f90:24),
 * heater(itime,Q,Qdens) (mod_heating.f90:27), S_catS (mod_cattaneo.f90:23), S and the
 * initial guess x0 (mod_evolve.f90:112-141).  Any pointer may be NULL. */
int hf_get_rhs(hf_ctx* ctx, int64_t itime, double* B, double* Q, double* Qdens, double* s_cat,
               double* S, double* x0);
/* y = H x with the device operator (atimes/SRSax, mod_Sparse.f90:293-315, 436-450). */
int hf_apply_operator(hf_ctx* ctx, const double* x, double* y);
/* Solve H x = b in place (x: initial guess in, solution out) with the context's options
 * (linbcg, mod_Sparse.f90:372-434).  Single-instance contexts only. */
int hf_solve(hf_ctx* ctx, const double* b, double* x, hf_stats* stats);
/* COO assembly in the reference's storage order (sparse_Hmatrix, mod_setup.f90:89-152):
 * capacity `len` slots, irow=-2/jcol=-1 in unused slots, 1-based indices.  cap must be
 * >= the reference capacity returned in *len; *count receives the entries written. */
int hf_assemble_coo(hf_ctx* ctx, int64_t instance, int64_t cap, int64_t* irow, int64_t* jcol,
                    double* val, int64_t* len, int64_t* count);

/* ---- device-resident state and the discrete adjoint ------------------------------------------
 * No reference counterpart: HeatFlow computes no gradients.  Single-grid contexts; every pointer
 * is a device buffer of nx*ny*nz doubles in cell order.  With the forward step
 * H x_k = S_k = a x_(k-1) + c x_(k-2) - Qdens_k - B (a = -rho c/dt - 2 tau' rho c, c = tau' rho c),
 * the adjoint runs k = K..1:  H lambda_k = dJ/dx_k + a lambda_(k+1) + c lambda_(k+2)  (H = H^T). */
int hf_set_state_device(hf_ctx* ctx, const double* temp_p, const double* temp_pp);
int hf_get_state_device(hf_ctx* ctx, double* temp_p, double* temp_pp);
/* Solve H x = b (x: initial guess in, solution out) with the context's options. */
int hf_solve_device(hf_ctx* ctx, const double* b, double* x, hf_stats* stats);
/* out = g + a*lam1 + c*lam2 (the adjoint right-hand side of one step). */
int hf_adjoint_rhs(hf_ctx* ctx, const double* g, const double* lam1, const double* lam2, double* out);
/* grad_logk += lambda^T (dS/dlog kappa - dH/dlog kappa x) over every face of every cell;
 * grad_src += lambda^T dS/dP (P: each cell's heater power at step itime); grad_src may be NULL.
 * Rejects Neumann (CG) faces and emissivity, whose terms are not differentiated. */
int hf_adjoint_accumulate(hf_ctx* ctx, const double* lam, const double* x, int64_t itime,
                          double* grad_logk, double* grad_src);

/* ---- host-buffer steps queued without host round trips (no reference counterpart) -------------
 * For callers that keep the state in host arrays, as simulate() does (Temp_p/Temp_pp): each call
 * queues one step whose inputs come from and whose result goes to pinned host memory, and returns
 * at once.  Copy engines move compact staging buffers (kernels place them into the state's role
 * buffers, whose indices live on the device; the step's last residual sweep also writes its
 * result into one, so the download needs no gather).  T^(n-1) - normally the
 * result of two calls back - is uploaded on a second stream while the previous step is still
 * solving; T^n - normally the previous call's temp_out - is uploaded chunk by chunk right behind
 * that download, so both directions of the host link run at once, and the right-hand side of
 * each chunk's cells is computed as soon as the chunk is placed.  A call whose temp_p is the
 * previous call's temp_out and whose temp_pp is the previous call's temp_p (the rotation simulate
 * performs) starts at once from the device's copy of those fields while its uploads travel; the
 * uploaded bits are compared with that copy before it can be overwritten, and if they differ
 * (an array was changed while queued) hf_host_sync runs the queue again from that call, each
 * step from its uploaded inputs as hf_set_state would place them.  Any arrays may be passed:
 * an input that is the temp_out of one of the queued calls waits for that download, in
 * whatever order the arrays rotate.  Every array
 * holds total_cells doubles (instances back to back) and must stay valid and untouched until
 * hf_host_sync returns.  Needs use_graph 1 or 3.  While steps are queued, every other call that
 * reads or changes the state returns HF_ESTATE. */
int hf_step_host_async(hf_ctx* ctx, int64_t itime, const double* temp_p, const double* temp_pp,
                       double* temp_out);
/* Wait for the queued steps; statistics over them and the first error (HF_ENAN_*, HF_EDEVICE). */
int hf_host_sync(hf_ctx* ctx, hf_stats* stats);
/* Page-lock and map an existing host array (e.g. Fortran's Temp_p) so it can be passed to
 * hf_step_host_async; wraps cudaHostRegister. */
int hf_host_register(void* ptr, size_t bytes);
int hf_host_unregister(void* ptr);

/* ---- measurement (no reference counterpart: the reference times with cpu_time only) ------- */
enum {
  HF_KERNEL_RHS = 0,         /* per-step right-hand side */
  HF_KERNEL_RESIDUAL = 1,    /* FP64 solution update + true residual sweep */
  HF_KERNEL_CG_P = 2,        /* inner CG direction update p = r + beta p */
  HF_KERNEL_CG_SPMV = 3,     /* inner CG SpMV q = A p and p.q */
  HF_KERNEL_CG_UPDATE = 4,   /* inner CG solution/residual update + r.r */
  HF_KERNEL_XUPDATE = 5,     /* FP64 solution update x += S^-1 y */
  HF_KERNEL_SOLVE = 6,       /* the persistent solve kernel: one whole solve of the next step's
                                system (the step's RHS runs before each timed launch) */
  HF_KERNEL_CG_PQ = 7,       /* the fused direction update + SpMV pass of the persistent solve's
                                FP32 inner CG, launched on its own (FP64: CG_P then CG_SPMV) */
  HF_KERNEL_RESIDUAL_INIT = 8 /* the step-start residual sweep r = S - H (x0 + TINY) */
};
/* Timeline of the latest step, from %globaltimer stamps its kernels write when they start
 * (microseconds): us[0] step begin -> RHS, us[1] RHS -> RHS finalize, us[2] finalize -> persistent
 * solve, us[3] solve start -> end of its last round, us[4] -> step end.  -1 where the step had no
 * such kernel (the per-kernel solve paths, use_graph 0 and 2, have no persistent solve).  No
 * counterpart in the reference. */
int hf_step_timeline(hf_ctx* ctx, double* us);
/* Launch one kernel `reps` times on the current state, each bracketed by CUDA events on the
 * context's stream, and return its mean duration in milliseconds.  Solver scalars are restored
 * afterwards; the temperature state is not modified.  Call after at least one step. */
int hf_time_kernel(hf_ctx* ctx, int kernel, int reps, double* ms_per_launch);
/* FP64 and FP32 FMA throughput of the current device in TFLOP/s (independent FMA chains over
 * every SM, CUDA-event timed).  On GB300 the FP64 rate bounds the FP64 kernels of a step. */
int hf_measure_fp_rates(double* fp64_tflops, double* fp32_tflops);

/* Phases of the persistent solve kernel, one per grid-wide round. */
enum {
  HF_PHASE_IDLE = 0,      /* nothing left (step finished) */
  HF_PHASE_START = 1,     /* reserved */
  HF_PHASE_RES_INIT = 2,  /* first true residual r = S - H x0 */
  HF_PHASE_CG_P = 3,      /* FP64 inner CG: p = r + beta p */
  HF_PHASE_CG_Q = 4,      /* FP64 inner CG: q = Ah p, p.q */
  HF_PHASE_CG_PQ = 5,     /* FP32 inner CG: p = r + beta p and q = Ah p in one pass */
  HF_PHASE_CG_B = 6,      /* inner CG: y += alpha p, r -= alpha q, r.r */
  HF_PHASE_XUPD = 7,      /* x += sigma S^-1 y */
  HF_PHASE_RES = 8,       /* true residual of the updated x */
  HF_PHASE_RES_INIT_HX = 9, /* first true residual from the stored H T^n and H T^(n-1) (pointwise) */
  HF_PHASE_CG_BX = 10     /* inner CG update that also forms x += sigma S^-1 y: the iteration
                             predicted to end the inner solve (true-residual criterion) */
};
/* Round profile of the context's last persistent solve (use_graph = 1, or hf_time_kernel with
 * HF_KERNEL_SOLVE).  No counterpart in the reference.  *rounds = grid-wide rounds run; for the
 * first min(rounds, cap, 512) rounds, phases[r] = the phase instance 0 ran and round_us[r] = the
 * round's length in microseconds (device %globaltimer; round 0 counts from the kernel's start). */
int hf_solve_profile(hf_ctx* ctx, int64_t cap, int64_t* rounds, int32_t* phases, double* round_us);

/* ---- index checks ------------------------------------------------------------------------------
 * No counterpart in the reference (the reference has no bounds-checked build; this stands in for a
 * memory checker, which is not available on the GPUs this library is tested on).  The library can
 * be built with -DHF_CHECKED (a separate build for tests): every global load and store of the
 * step kernels then checks its index against the extent of its array in the instance's layout
 * (4-cell vector accesses also their 16-byte alignment); a failed check is recorded on the device
 * and the access is moved inside the array, with no trap and no fault, and the next call that
 * finishes steps returns HF_EDEVICE naming the first failed check's site in hf_last_error.
 * hf_index_checks sets *enabled = 1 in the checked build (0 otherwise), copies the record
 * {failed checks, site of the first (100000 * file + line), its index, the extent} to record
 * (4 values, or NULL) and clears it.  probe != 0 (checked build only) first runs one check on an
 * index outside its range without any memory access, so a test can see a failure recorded. */
int hf_index_checks(hf_ctx* ctx, int32_t probe, int32_t* enabled, int64_t* record);

/* ---- temperature-dependent properties -------------------------------------------------------
 * The reference's TempDepProp = 1 rebuilds H after every step from unchanged properties (its
 * table lookup is commented out, mod_tempdep.f90:66-95; the rebuild is called at
 * mod_evolve.f90:172-174).  This call makes the rebuild real: after every step, each cell with a
 * table takes kappa, rho and c at its new temperature T^n -- rows (T ascending, kappa, rho, c),
 * held constant below the first and above the last row, linear in between -- and the operator,
 * the boundary vector and the solver scaling are rebuilt on the device inside the captured step.
 * Tables k = 0..ntables-1 are rows[4*offsets[k] .. 4*offsets[k+1]); cell_table holds one table
 * index (or -1: fixed properties) per cell of all instances in cell order.  ntables = 0 returns
 * to fixed properties (the ones in effect stay). */
int hf_set_property_tables(hf_ctx* ctx, int32_t ntables, const int32_t* offsets, const double* rows,
                           const int32_t* cell_table);

/* ---- sub-box snapshots overlapped with stepping --------------------------------------------
 * The reference logs a sub-box of the field after a step (data_write, mod_output.f90:57-66,
 * :92-113: Temp_pp, i.e. T^(n-1) after the state rotation, for start_i..end_i on each axis).
 * hf_subbox_async enqueues, on the context stream after the work already queued, a gather of the
 * box lo..hi (0-based, inclusive; packed x fastest, then y, then z) of instance `inst`'s field
 * `which` (0: T^n, 1: T^(n-1)) into a device staging slot, and a copy of that slot to `host` on a
 * separate copy stream; it returns at once with a ticket, so the following steps run while the
 * copy engine moves the data (with a pinned `host` buffer; a pageable one makes the calling thread
 * wait for the copy).  Four staging slots rotate; reusing a slot waits on the device for its
 * previous copy.  hf_subbox_wait blocks until the copy of `ticket` has landed in `host`. */
int hf_subbox_async(hf_ctx* ctx, int64_t inst, const int64_t* lo, const int64_t* hi, int which,
                    double* host, int64_t* ticket);
int hf_subbox_wait(hf_ctx* ctx, int64_t ticket);

/* ---- failure-path check ------------------------------------------------------------------------
 * No counterpart in the reference.  Runs the next step's persistent solve once with one block
 * that leaves without arriving at the first grid barrier and a barrier time limit of wait_ms:
 * the other blocks give up after wait_ms, record the failure and return, and *status receives the
 * code the step loop would report (HF_EDEVICE).  The temperature state and the scalars are
 * restored, so the context stays usable.  For tests of the bounded-wait path (no GPU fault). */
int hf_check_barrier_timeout(hf_ctx* ctx, int32_t wait_ms, int32_t* status, double* seconds);

/* ---- autotuner ------------------------------------------------------------------------------
 * No counterpart in the reference.  Chooses the stencil task shape (z-planes per 32 x 8 column
 * tile: 8, 16, 32 or 64) and, on the mixed path, the inner FP32 tolerance (1e-4, 1e-5, 1e-6) for this
 * context's own grids: for every candidate it restores the current state, runs one untimed step
 * and then `steps` steps from step `itime0` timed with CUDA events through the context's step loop
 * (use_graph as set), and keeps the fastest.  On return the options hold the choice and the state,
 * the scalars and the statistics are those of the call (the tuning steps leave no trace).
 * results (may be NULL): up to cap candidates with their measured time per step. */
typedef struct hf_tune_result {
  int32_t task_depth;
  int32_t chosen;        /* 1 for the candidate kept */
  double inner_tol;
  double ms_per_step;
} hf_tune_result;
int hf_autotune(hf_ctx* ctx, int64_t itime0, int32_t steps, hf_tune_result* results, int32_t cap,
                int32_t* n_results);

/* ---- allocation-free residual ---------------------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory - hosts that
 * own all device memory through a fixed arena and hand the library pre-allocated buffers, and
 * loops that may not stall on the allocator (cudaMalloc can synchronise the device): r = b - H x and
 * norms2 = {||r||^2, ||b||^2} for the geometric operator of hf_get_operator (diag and the face to
 * the + neighbour per axis, periodic wrap on the last cell of a periodic axis).  Every pointer is
 * a caller-owned device buffer (norms2: two doubles); stream is a cudaStream_t or NULL.  The call
 * allocates nothing: its reduction scratch is a static device array of 256 KiB that every device
 * loading the library holds until the process exits, which limits grids to
 * HF_NOALLOC_MAX_CELLS cells (larger grids return HF_EARG).  The first call on a device looks up
 * that array's device address (cudaGetSymbolAddress), so make it before any stream capture; so
 * does the first call after the device's context was reset (cudaDeviceReset).
 * Calls share the scratch and keep the last call's partial sums: calls whose kernels overlap on
 * the GPU race and must be serialised by the caller.  Asynchronous: results are ready when the
 * stream reaches them. */
#define HF_NOALLOC_MAX_CELLS 16777216
int hf_residual_noalloc(int64_t nx, int64_t ny, int64_t nz, const int32_t* periodic,
                        const double* diag, const double* cx, const double* cy, const double* cz,
                        const double* b, const double* x, double* r, double* norms2, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* HEATFLOW_GB300_H */
