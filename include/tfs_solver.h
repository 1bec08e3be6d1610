/*
 * tfs_solver.h -- C ABI of the GB300 (sm_103a) Krylov solver library
 * libtfs_gb300.so.
 *
 * The library replaces the sequential linear-solver module of the T-FlowS
 * flow solver (Sources/Process/Solvers_Mod.f90 with the routines included at
 * Solvers_Mod.f90:16-21).  The flow solver keeps calling
 *
 *     call Cg  (A, x, r1, prec, niter, tol, ini_res, fin_res)
 *     call Bicg(A, x, r1, prec, niter, tol, ini_res, fin_res)
 *     call Cgs (A, x, r1, prec, niter, tol, ini_res, fin_res)
 *
 * through an ISO_C_BINDING module that expands `A` (type Matrix_Type,
 * Matrix_Mod.f90:36-49) into its compressed-row arrays.  Everything below uses
 * plain pointers and sizes:
 *
 *   n       number of cells = rows      (A % pnt_grid % n_cells)
 *   nnz     stored entries = row(n+1)-1 (the reference allocates nnz+1)
 *   row1    A % row(1:n+1), 1-based, int32
 *   col1    A % col(1:nnz), 1-based column numbers, ascending within a row
 *   dia1    A % dia(1:n),   1-based position of the diagonal in each row
 *   val     A % val(1:nnz), float64
 *   x       x(1:n), the interior part of x(-NB:N); in/out
 *   r1      on entry b(1:n); on return the final recursive residual (F3)
 *   prec    0 none, 1 diagonal, 2 diagonal incomplete Cholesky (DIC)
 *   niter   in: iteration limit; out: iterations done, or limit+1 if the
 *           solve did not converge (Fortran DO-loop exit value)
 *   tol     ABSOLUTE tolerance on ||r||_2 (the reference does not scale it)
 *   ini_res out: ||b - A x0||_2 (left untouched when ||b|| < tol)
 *   fin_res out: last ||r||_2 (||b||_2 on the ||b|| < tol exit, where the
 *           reference returns an uninitialised local)
 *
 * All calls return an int status (TFS_OK = 0).  A non-finite residual is
 * reported as TFS_ERR_NONFINITE with fin_res = NaN and niter = limit+1; the
 * contents of x and r1 are then unspecified (the reference carries the NaN
 * through every remaining iteration; this library stops at the first one).
 *
 * Threading: a handle is used by one host thread at a time; every handle owns
 * one CUDA stream.  Different handles may be used concurrently.
 */
#ifndef TFS_SOLVER_H
#define TFS_SOLVER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define TFS_OK             0
#define TFS_ERR_ARG        1  /* null pointer, bad size, unknown method/prec  */
#define TFS_ERR_MATRIX     2  /* malformed CSR: range, unsorted row, no diag   */
#define TFS_ERR_CUDA       3  /* CUDA runtime failure (no device, OOM, ...)    */
#define TFS_ERR_NONFINITE  4  /* breakdown: NaN/Inf residual, rho or (p,q)     */
#define TFS_ERR_TOPOLOGY   5  /* arrays do not match the registered topology   */
#define TFS_ERR_TIMEOUT    6  /* a bounded device-side wait expired            */
#define TFS_ERR_BUDGET     7  /* request refused by the device-memory budget   */

/* ---- methods (the three Solvers_Mod routines) and preconditioners ----- */
#define TFS_CG    0   /* Cg.f90:2   */
#define TFS_BICG  1   /* Bicg.f90:2 */
#define TFS_CGS   2   /* Cgs.f90:2  */

#define TFS_PREC_NONE 0   /* Prec_Form.f90:45-49 / Prec_Solve.f90:71-74 */
#define TFS_PREC_DIAG 1   /* Prec_Form.f90:24-27 / Prec_Solve.f90:35-38 */
#define TFS_PREC_DIC  2   /* Prec_Form.f90:32-40 / Prec_Solve.f90:43-67 */

/* ---- arithmetic of the Krylov iterations ------------------------------ */
#define TFS_FP64  0   /* every operation in binary64, per-row arithmetic of the reference */
#define TFS_MIXED 1   /* binary32 matrix and vectors inside the iteration; binary64
                         true residual b-Ax, alpha/beta reductions and solution */

typedef struct tfs_handle tfs_handle;

/* Statistics of the last solve on a handle (device-measured). */
typedef struct tfs_stats {
    int32_t  iterations;        /* Krylov iterations executed                   */
    int32_t  true_residuals;    /* binary64 b-Ax evaluations (TFS_MIXED)        */
    int32_t  n_levels;          /* DIC level-schedule depth of the topology     */
    int32_t  status;            /* status of the last solve                     */
    double   solve_ms;          /* device time of the last solve (CUDA events)  */
    double   spmv_ns_total;     /* summed duration of the SpMV launches          */
    int64_t  spmv_launches;     /* number of SpMV launches timed                 */
    double   sweep_ns_total;    /* summed duration of DIC sweep launches         */
    int64_t  sweep_launches;
    int64_t  kernel_launches;   /* kernels launched by the last solve            */
    int64_t  device_bytes;      /* device memory held by the handle             */
    int32_t  spmv_kernel;       /* SpMV kernel of the CG iterations: 0 direct,
                                   1 software-pipelined                        */
    int32_t  sell_width;        /* uniform SELL-32 slice width, 0 if per slice  */
    int32_t  dic_kernel;        /* DIC application last launched: 0 level
                                   kernels, 1 one-block (TFS_OPT_DIC_BLOCK)    */
    int32_t  pad;
} tfs_stats;

/* ---- topology ----------------------------------------------------------- */

/* Register a CSR topology (row1/col1/dia1, 1-based) and build its device
 * layout: 0-based sliced-ELL storage, the DIC level schedule (computed on the
 * device) and the Krylov work vectors.  The topology of T-FlowS is built once
 * at start-up (Main.f90:141-142, Matrix_Mod/Topology.f90:2-127) and only the
 * values change between solves, so a handle is built once per mesh.
 * Replaces: the device-side counterpart of Matrix_Mod_Topology's output. */
int tfs_topology_register(int32_t n, int32_t nnz, const int32_t *row1,
                          const int32_t *col1, const int32_t *dia1,
                          tfs_handle **out);

/* Free every device and host resource of a handle. */
int tfs_release(tfs_handle *h);

/* Arithmetic of the Krylov iterations for later solves on h: TFS_FP64 or
 * TFS_MIXED.  Replaces nothing in the reference (it has binary64 only). */
int tfs_set_precision(tfs_handle *h, int mode);

/* Precision (TFS_FP64 or TFS_MIXED) of the handles that the library keeps
 * for tfs_cg/tfs_bicg/tfs_cgs and tfs_solve(h = NULL): those already built
 * and those built later.  A Fortran caller selects mixed precision for its
 * drop-in Cg/Bicg/Cgs calls with this one call.  Replaces nothing in the
 * reference. */
int tfs_set_default_precision(int mode);

/* ---- options of a handle ------------------------------------------------
 * Alternatives the library was measured with, kept selectable for profiling
 * and for the tests that check them against each other.  The defaults are the
 * fastest measured on GB300.  Except TFS_OPT_FUSE_L0 (another summation
 * order of rho in DIC-CG), every alternative gives bitwise the same results.
 * Setting an option drops the handle's captured graphs; the layout options
 * (TFS_OPT_LAYOUT, TFS_OPT_SELL_UNIFORM) also drop its device layout, which
 * the next solve rebuilds.  No option is read from the environment. */
#define TFS_OPT_LAUNCH        1  /* 0 one CUDA graph per solve (default); 1 eager
                                    launches from a host loop (kernel tracing)   */
#define TFS_OPT_LAYOUT        2  /* 0 RCM row order unless DIC (default); 1 DIC
                                    level order for every preconditioner        */
#define TFS_OPT_BICG          3  /* 0 BiCG on the CG kernels (default: its iterates
                                    equal CG's bit for bit); 1 both sequences   */
#define TFS_OPT_SELL_UNIFORM  4  /* 1 one SELL slice width when it costs <= 5%
                                    padding (default); 0 per-slice widths       */
#define TFS_OPT_SPMV          5  /* 1 software-pipelined SpMV where the width
                                    allows (default); 0 the direct kernel       */
#define TFS_OPT_SPMV_GRID     6  /* 0 8 blocks per SM, grid-stride (default);
                                    1 one block per 256-row chunk               */
#define TFS_OPT_LEVEL_TPB     7  /* threads per block of the DIC level kernels:
                                    128, 256 (default), 512 or 1024             */
#define TFS_OPT_TAIL_PF       8  /* 1 prefetching one-block tail (default); 0 the
                                    level loop                                  */
#define TFS_OPT_FUSE_L0       9  /* DIC-CG level 0 swept inside its neighbouring
                                    kernels: 2 both arithmetics (default), 1
                                    binary32 only, 0 off                        */
#define TFS_OPT_PDL          10  /* 1 programmatic dependent launch between the
                                    level kernels (default); 0 plain launches   */
#define TFS_OPT_PDL_VEC      11  /* 1 PDL-chained CG vector kernels (default); 0 */
#define TFS_OPT_FWD_PRE      12  /* 1 forward level kernels load b and D before
                                    their dependency wait (default); 0          */
#define TFS_OPT_BWD_PRE      13  /* 1 backward level kernels compute their start
                                    values before the wait (default); 0         */
#define TFS_OPT_DIC_BLOCK    14  /* 1 each DIC sweep (and Prec_Form) in one
                                    thread block, the vector in shared memory
                                    and groups of levels staged there ahead,
                                    where the vector and two slots of the
                                    widest level fit (deep schedules of narrow
                                    levels; default); 0 the level kernels       */
#define TFS_OPT_L2_WINDOW    15  /* 1 the column indices in an L2 persisting
                                    access window of the solve kernels (a
                                    limit of the calling process's context;
                                    default); 0 none                           */

/* One DIC application (the tfs_time_prec workload: factor from val, r = 1)
 * with its level launches stamped on the device: for slot k (launch order)
 * start_us[k] = when the launch's blocks passed their dependency wait
 * (earliest) and end_us[k] = when they had finished (latest), in
 * microseconds after the first stamp; kind[k] = the level of a forward
 * launch, -1 - level of a backward one, 1 << 20 for the one-block tail.
 * Level-kernel schedule only (TFS_ERR_ARG when the one-block DIC runs).
 * Allocates the stamp buffer itself (a profiling call).  Replaces nothing
 * in the reference. */
int tfs_profile_prec(tfs_handle *h, const double *val, int mode, int max_slots, double *start_us,
                     double *end_us, int32_t *kind, int32_t *n_slots);

/* Set / read one option of a handle.  TFS_ERR_ARG for an unknown option or
 * value.  Replaces nothing in the reference. */
int tfs_set_option(tfs_handle *h, int option, int value);
int tfs_get_option(const tfs_handle *h, int option, int *value);

/* Diagnostics of the one-block DIC's bounded waits: with wait_ns > 0 (at
 * most 1e9), the solves of this handle that follow run the one-block DIC
 * with its copy lane staging nothing and every wait limited to wait_ns, so
 * its first wait runs out: the kernel raises its abort flag, no thread
 * waits or reads a slot again, and the solve returns TFS_ERR_TIMEOUT with
 * the GPU unaffected.  wait_ns = 0 restores the normal limit (0.5 s).
 * Replaces nothing in the reference. */
int tfs_diag_dic_timeout(tfs_handle *h, long long wait_ns);

/* ---- solves ------------------------------------------------------------- */

/* One preconditioned Krylov solve with host arrays (val, x, r1 host memory).
 * method: TFS_CG / TFS_BICG / TFS_CGS.  h may be NULL: the library then
 * keeps one handle per (row1, col1, n, nnz) and builds it on first use.
 * Replaces: Cg.f90:2-4, Bicg.f90:2-4, Cgs.f90:2-4 (same argument meaning). */
int tfs_solve(int method, tfs_handle *h, int32_t n, int32_t nnz,
              const int32_t *row1, const int32_t *col1, const int32_t *dia1,
              const double *val, double *x, double *r1, int32_t prec,
              int32_t *niter, double tol, double *ini_res, double *fin_res);

/* The three Fortran-shaped entry points the ISO_C_BINDING shim binds.
 * Replace Cg.f90:2-4, Bicg.f90:2-4 and Cgs.f90:2-4 respectively. */
int tfs_cg(int32_t n, int32_t nnz, const int32_t *row1, const int32_t *col1,
           const int32_t *dia1, const double *val, double *x, double *r1,
           int32_t prec, int32_t *niter, double tol, double *ini_res,
           double *fin_res);
int tfs_bicg(int32_t n, int32_t nnz, const int32_t *row1, const int32_t *col1,
             const int32_t *dia1, const double *val, double *x, double *r1,
             int32_t prec, int32_t *niter, double tol, double *ini_res,
             double *fin_res);
int tfs_cgs(int32_t n, int32_t nnz, const int32_t *row1, const int32_t *col1,
            const int32_t *dia1, const double *val, double *x, double *r1,
            int32_t prec, int32_t *niter, double tol, double *ini_res,
            double *fin_res);

/* The same solve on device-resident arrays (natural cell order, 0-based
 * C arrays of length nnz / n).  Used by callers that assemble on the GPU.
 * Replaces: Cg.f90:2-4, Bicg.f90:2-4, Cgs.f90:2-4. */
int tfs_solve_device(int method, tfs_handle *h, const double *d_val,
                     double *d_x, double *d_r1, int32_t prec, int32_t *niter,
                     double tol, double *ini_res, double *fin_res);

/* ---- single routines (host arrays), for callers and parity checks ------ */

/* q = A p (the product loop of Cg.f90:128-134, per-row arithmetic kept). */
int tfs_spmv(tfs_handle *h, const double *val, const double *p, double *q);

/* r1 <- r1 - A x.  Replaces Residual.f90:2-40 (n_proc = 0). */
int tfs_residual(tfs_handle *h, const double *val, const double *x, double *r1);

/* d(i) = D % val(D % dia(i)) after Prec_Form.  Replaces Prec_Form.f90:2-51. */
int tfs_prec_form(tfs_handle *h, const double *val, int32_t prec, double *d);

/* x = M^-1 b for the preconditioner formed from val.
 * Replaces Prec_Form.f90:2-51 followed by Prec_Solve.f90:2-78. */
int tfs_prec_solve(tfs_handle *h, const double *val, int32_t prec,
                   const double *b, double *x);

/* ---- introspection ------------------------------------------------------ */
int tfs_get_stats(const tfs_handle *h, tfs_stats *out);

/* Level of every row (0-based levels, natural row order) of the DIC
 * dependency analysis done on the device at registration. */
int tfs_get_levels(tfs_handle *h, int32_t *levels);

/* Device time of one SpMV launch averaged over `reps` back-to-back launches
 * on the handle's stream (CUDA events), with values val (host, nnz), in the
 * given arithmetic (TFS_FP64 or TFS_MIXED). */
int tfs_time_spmv(tfs_handle *h, const double *val, int mode, int reps,
                  double *ms_per_launch);

/* Device time of one DIC preconditioner application (forward sweep,
 * diagonal scaling, backward sweep; replaces Prec_Solve.f90:46-67 with prec
 * = 2) averaged over `reps` back-to-back applications (CUDA events), with the
 * factor formed from val (host, nnz), in the given arithmetic. */
int tfs_time_prec(tfs_handle *h, const double *val, int mode, int reps,
                  double *ms_per_application);

/* Launch shapes picked for one handle by tfs_autotune, with the timings
 * they were picked from (0 where a candidate was not timed). */
typedef struct tfs_tuning {
    int32_t level_tpb;        /* threads per block of the DIC level kernels  */
    int32_t spmv_chunks;      /* 1: one 256-row chunk per SpMV block,
                                 0: 8 blocks per SM, grid-stride            */
    double  prec_ms[4];       /* DIC application, level_tpb 128/256/512/1024 */
    double  spmv_ms[2];       /* direct SpMV kernel, spmv_chunks 0 / 1       */
    int32_t spmv_kernel;      /* SpMV kernel kept: 0 direct, 1 software-
                                 pipelined                                  */
    int32_t pad;
    double  spmv_pipe_ms[2];  /* software-pipelined SpMV, spmv_chunks 0 / 1
                                 (0: matrix not of uniform slice width)     */
} tfs_tuning;

/* Time the candidate launch shapes of the single-solve kernels on this
 * handle's own system (values val, host, nnz) in the given arithmetic and
 * keep the fastest: the SpMV kernel and grid always, the DIC level-kernel block size
 * when prec == 2 (this builds the level layout if the handle has none).
 * Graphs built earlier for the handle are dropped and rebuilt on the next
 * solve.  Results do not depend on the shapes (per-row arithmetic and
 * reductions are shape-independent except for the order of the block
 * partial sums).  No reference counterpart: the reference has no launch
 * shapes. */
int tfs_autotune(tfs_handle *h, const double *val, int mode, int prec, int reps,
                 tfs_tuning *out);

/* Human-readable text for a status code. */
const char *tfs_status_string(int status);

/* Text of the last error recorded by this thread (CUDA error names etc.). */
const char *tfs_last_error(void);

/* ---- batches of independent systems -------------------------------------
 * Many registered topologies solved together by one persistent kernel: each
 * system is solved start to finish by one thread-block cluster, clusters take
 * systems longest first from a device queue, and a system's result does not
 * depend on what else is in the batch (bitwise).  CG or BiCG with no or
 * diagonal preconditioning (the pressure and transport solves of
 * Compute_Pressure_Fractional.f90:203 / Compute_Scalar.f90:619), in
 * TFS_FP64 or TFS_MIXED.  Per-system arrays are indexed like `handles`.
 * Replaces: a loop of Cg.f90:2-4 / Bicg.f90:2-4 calls, one per system. */
typedef struct tfs_batch tfs_batch;

int tfs_batch_create(int n_sys, tfs_handle *const *handles, tfs_batch **out);
int tfs_batch_release(tfs_batch *b);

/* Cluster size (1..16, power of two) and threads per CTA (128, 256, 512). */
int tfs_batch_configure(tfs_batch *b, int cluster_size, int threads_per_cta);

/* Device arrays (natural order) per system; niter/tol per system in,
 * niter_out/ini_res/fin_res/status per system out (ini_res untouched on the
 * ||b|| < tol exit).  Returns the first non-OK system status, or TFS_OK. */
int tfs_batch_solve_device(tfs_batch *b, int method, int prec, int mode,
                           const double *const *d_val, double *const *d_x,
                           double *const *d_r1, const int32_t *niter,
                           const double *tol, int32_t *niter_out,
                           double *ini_res, double *fin_res, int32_t *status);

/* The same with host arrays (copied through each handle's staging buffers). */
int tfs_batch_solve(tfs_batch *b, int method, int prec, int mode,
                    const double *const *val, double *const *x,
                    double *const *r1, const int32_t *niter, const double *tol,
                    int32_t *niter_out, double *ini_res, double *fin_res,
                    int32_t *status);

/* Device time (CUDA events) of the last batch solve, gather included. */
int tfs_batch_last_ms(const tfs_batch *b, double *ms);

/* n copies dst[k] <- src[k] (bytes[k]) ordered on the batch's stream, e.g.
 * to reset every system's x and r1 before a solve. */
int tfs_batch_copy(tfs_batch *b, int n, void *const *dst, const void *const *src,
                   const size_t *bytes);

/* ---- device and timing helpers ------------------------------------------
 * For callers without a CUDA runtime of their own (the benchmark harness, a
 * Fortran driver).  None of these replaces a reference interface. */

/* Make `device` current for the calling host thread (handles created later
 * live on it). */
int tfs_use_device(int device);

/* Device memory (cudaMalloc / cudaFree) and page-locked host memory
 * (cudaMallocHost / cudaFreeHost). */
int tfs_device_alloc(size_t bytes, void **ptr);
int tfs_device_free(void *ptr);
int tfs_host_alloc(size_t bytes, void **ptr);
int tfs_host_free(void *ptr);

/* Copy `bytes` between any two of host/device memory, ordered on the
 * handle's stream (asynchronous for device and page-locked memory). */
int tfs_copy(tfs_handle *h, void *dst, const void *src, size_t bytes);

/* Synchronous copy in any direction on the current device (no handle). */
int tfs_memcpy(void *dst, const void *src, size_t bytes);

/* Wait for all work queued on the handle's stream. */
int tfs_sync(tfs_handle *h);

/* CUDA events on the handle's stream around a region of calls:
 * tfs_timer_stop waits for the region and returns its device time. */
int tfs_timer_start(tfs_handle *h);
int tfs_timer_stop(tfs_handle *h, double *ms);

/* ---- serving: solves that arrive over time --------------------------------
 * A request loop for the solves a flow solver (or many of them) issues over
 * time: pressure and transport systems of different sizes.  A worker thread
 * admits each request as soon as its system is idle and a slot is free, so
 * requests that arrive while others run start at once and their work
 * overlaps on the GPU (each solve is one graph launch on its system's
 * stream).  Matrix layouts, preconditioners and Krylov vectors stay resident
 * between requests; systems are admitted against a device-memory budget and
 * idle ones are evicted, least recently used first, when a new one does not
 * fit (an evicted system is rebuilt on its next request).  A result does not
 * depend on what else was running.  Replaces: the sequence of Cg.f90 /
 * Bicg.f90 / Cgs.f90 calls of one or more Process runs. */
typedef struct tfs_server tfs_server;

typedef struct tfs_result {
    int64_t ticket;
    int32_t niter, status;          /* as the solve entry points return them  */
    double  ini_res, fin_res;
    double  queued_ms, run_ms, latency_ms;  /* submit->start, start->done, submit->done */
    /* The GPU's global nanosecond timer when the solve's first kernel began
     * and when its iterations had ended (the store of x and r1 began): two
     * requests whose intervals intersect ran on the device at once. */
    int64_t device_begin_ns, device_end_ns;
} tfs_result;

typedef struct tfs_server_stats {
    int64_t submitted, completed, refused, evictions, registrations;
    int64_t resident_bytes, resident_systems, running, queued;
    int64_t peak_running;           /* most solves launched and unfinished at once */
} tfs_server_stats;

int tfs_server_create(int device, int64_t hbm_budget_bytes, int max_inflight,
                      tfs_server **out);
/* Waits for running solves, then frees every resident system. */
int tfs_server_destroy(tfs_server *s);
/* Register a topology (1-based CSR, copied); device state is built lazily. */
int tfs_server_add_system(tfs_server *s, int32_t n, int32_t nnz, const int32_t *row1,
                          const int32_t *col1, const int32_t *dia1, int64_t *sys_id);
/* Queue one solve on device arrays (natural order; valid until done).
 * b is read from d_b (NULL: from d_r1, the in/out convention of Cg.f90);
 * r1 is written to d_r1; x starts from zero when x0_zero, else from d_x.
 * mode: TFS_FP64 or TFS_MIXED.  Returns at once with a ticket. */
int tfs_server_submit(tfs_server *s, int64_t sys_id, int method, int prec, int mode,
                      const double *d_val, const double *d_b, double *d_x, double *d_r1,
                      int x0_zero, int32_t niter, double tol, int64_t *ticket);
/* As tfs_server_submit with the Fortran call's host arrays: val (nnz), x
 * (n, the start value unless x0_zero) and r1 (n: b on entry, the final
 * residual on return), all in host memory (page-locked for overlap).  The
 * copies in and out run on the system's stream as part of the request, as
 * the drop-in tfs_cg/tfs_bicg/tfs_cgs do per call; the arrays must stay
 * valid until the ticket is waited for.  Replaces: Cg.f90:2-4 called from
 * several threads at once, served concurrently. */
int tfs_server_submit_host(tfs_server *s, int64_t sys_id, int method, int prec, int mode,
                           const double *val, double *x, double *r1, int x0_zero, int32_t niter,
                           double tol, int64_t *ticket);
/* Wait up to timeout_s for a ticket; TFS_ERR_TIMEOUT if still running.  A
 * ticket is returned once. */
int tfs_server_wait(tfs_server *s, int64_t ticket, double timeout_s, tfs_result *out);
int tfs_server_get_stats(tfs_server *s, tfs_server_stats *out);

/* ---- no-allocation entry point -------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory at the time of the call: code handed a fixed device arena by its
 * host framework, work issued while another thread captures a CUDA graph
 * (cudaMalloc is not allowed then), or a coupling loop that must never block
 * in the allocator.
 *
 * r1 <- r1 - A x with the per-row arithmetic of Residual.f90:22-27, and
 * *d_norm = ||r1||_2, for a 1-based CSR matrix (row1/col1/val as in
 * Matrix_Type) whose arrays, like x, r1 and the norm, already live in device
 * memory.  Nothing is allocated: the only scratch is a static device array
 * holding one partial sum per 256 rows, sized for TFS_NOALLOC_MAX_ROWS rows;
 * every GPU that loads the library keeps it (about 128 KB) until the process
 * exits.  Larger n is rejected with TFS_ERR_ARG.  The call is asynchronous on
 * `stream` (a cudaStream_t; NULL = the default stream).  The first call in a
 * CUDA context looks up the scratch array's device address
 * (cudaGetSymbolAddress) and caches it for that context; a call under another
 * context of the same device (after cudaDeviceReset, after the primary
 * context was released and retained again, or in a context the caller
 * created) looks it up again.  Make a context's first call before any stream
 * capture.  Calls share the scratch array, so calls that overlap on the GPU
 * (different streams or threads) race: serialise them. */
#define TFS_NOALLOC_MAX_ROWS 4194304
int tfs_residual_norm_noalloc(int32_t n, const int32_t *d_row1,
                              const int32_t *d_col1, const double *d_val,
                              const double *d_x, double *d_r1, double *d_norm,
                              void *stream);

/* ---- device-side assembly through the face -> entry map ---------------- */

/* Attach the mesh faces to a handle: faces_c (2*n_faces, 1-based cells c1,
 * c2; c2 <= 0 marks a boundary face) and pos1 (2*n_faces, the 1-based CSR
 * positions of the entries (c1,c2) and (c2,c1) of an interior face) as
 * tfs_topology_build returns them.  Checked against the registered topology;
 * builds on the device, once per mesh, every cell's faces in ascending face
 * order.  Replaces: the face loops' use of Matrix_Type%pos and %dia
 * (Matrix_Mod.f90:44-46, filled by Topology.f90:106-121). */
int tfs_faces_register(tfs_handle *h, int32_t n_faces, const int32_t *faces_c,
                       const int32_t *pos1);

/* Assemble matrix values on the device from per-face coefficients, as the
 * reference's face loops do (NewUVW.f90:366-384 followed by the cell loop
 * NewUVW.f90:500-505; Compute_Pressure_Simple.f90:100-113 is the case
 * off12 = off21 = dia12 = dia21 = A12 on a zeroed matrix):
 *   interior face s:  val(pos(1,s)) -= off12(s); val(dia(c1)) += dia12(s);
 *                     val(pos(2,s)) -= off21(s); val(dia(c2)) += dia21(s)
 *   boundary face s:  val(dia(c1)) += dia12(s), skipped when dia12(s) == 0
 *                     (a boundary type that adds nothing)
 *   then every cell:  val(dia(c)) += cell(c)          (d_cell may be NULL)
 * Every diagonal receives its additions in face order, so the values are
 * bitwise those of the sequential loops.  d_val (nnz, CSR order) holds the
 * starting values (normally zero) and receives the result; all arrays are
 * device pointers (off21, dia21 of boundary faces are not read).  Runs on the
 * handle's stream, before any solve issued after it; no synchronisation. */
int tfs_assemble_faces_device(tfs_handle *h, const double *d_off12, const double *d_off21,
                              const double *d_dia12, const double *d_dia21,
                              const double *d_cell, double *d_val);

/* ---- host-side mesh utilities ------------------------------------------ */

/* Count of stored entries of the face-connectivity matrix (one per cell plus
 * two per interior face).  faces_c: 2*n_faces 1-based cell numbers (c1, c2);
 * c2 <= 0 marks a boundary face.  Replaces Topology.f90:33-47. */
int32_t tfs_topology_count(int32_t n_cells, int32_t n_faces,
                           const int32_t *faces_c);

/* Build row/col/dia/mir/pos exactly as Matrix_Mod_Topology does (rows
 * sorted, 1-based).  col and mir have nnz entries, pos 2*n_faces (0 for
 * boundary faces).  Replaces Matrix_Mod/Topology.f90:2-127. */
int tfs_topology_build(int32_t n_cells, int32_t n_faces, const int32_t *faces_c,
                       int32_t *row1, int32_t *col1, int32_t *dia1,
                       int32_t *mir1, int32_t *pos1);

/* Matrix_Mod_Topology on the device: the same row/col/dia/mir/pos as
 * tfs_topology_build, bit for bit, from device-resident faces_c (2*n_faces,
 * 1-based; c2 <= 0 marks a boundary face).  d_col1 and d_mir1 must hold
 * n_cells + 2*n_faces entries (an upper bound of nnz); d_row1 n_cells+1,
 * d_dia1 n_cells, d_pos1 2*n_faces (0 for boundary faces).  *nnz_out
 * receives nnz.  Faces must join distinct pairs of distinct cells (checked:
 * cell numbers in range and c1 != c2; TFS_ERR_TOPOLOGY otherwise).  Runs on
 * the current device's default stream and returns when done.
 * Replaces Matrix_Mod/Topology.f90:2-127 for meshes held on the GPU. */
int tfs_topology_build_device(int32_t n_cells, int32_t n_faces, const int32_t *d_faces_c,
                              int32_t *d_row1, int32_t *d_col1, int32_t *d_dia1,
                              int32_t *d_mir1, int32_t *d_pos1, int32_t *nnz_out);

#ifdef __cplusplus
}
#endif
#endif /* TFS_SOLVER_H */
