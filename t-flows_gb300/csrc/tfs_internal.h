// tfs_internal.h -- device layout and per-handle state of libtfs_gb300.
//
// Layout in HBM (one handle = one registered topology):
//   internal row order   rows sorted by DIC level (level 0 first), natural
//                        order inside a level, each level padded with empty
//                        rows to a multiple of 32, the total padded to a
//                        multiple of TFS_TPB.  perm[internal] = natural row
//                        (or -1 for a padding row), iperm[natural] = internal.
//   SELL-32 matrix       slice s = internal rows 32s..32s+31, entries stored
//                        column-major: entry j of the row in lane t sits at
//                        slice_off[s] + 32*j + t.  Entries keep the reference's
//                        ascending column order, so j < dpos are the lower
//                        triangle, j == dpos the diagonal, j > dpos the upper.
//                        col[] holds internal column numbers.
//   rowinfo[i]           len | dpos << 16 (len == 0 marks a padding row).
//   vectors              binary64 (and binary32 for TFS_MIXED), n_int long,
//                        in internal order; padding rows stay exactly zero.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <map>
#include <vector>

#include "../../include/tfs_solver.h"

#define TFS_TPB 256           // threads per block = rows per chunk
#define TFS_LAYOUT_RCM 0      // rows in reverse Cuthill-McKee order
#define TFS_LAYOUT_LEVELS 1   // rows by DIC level, RCM order inside a level
#define TFS_SWEEP_TPB 1024    // threads per block = rows per tile of the level sweeps
#define TFS_TAIL_ROWS 1024    // levels after the last one above this size form the tail
#define TFS_NPART 4           // values reduced at once, at most
#define TFS_SPMV_DIRECT 0     // CG SpMV kernels: per-row dependent chain (any SELL-32 matrix)
#define TFS_SPMV_PIPE 1       //   software-pipelined, uniform slice width

// Device-resident state of one solve.  Written by k_init from DevParams and
// then only by the last block of each reducing kernel.
struct DevState {
    double tol;
    int niter_max;
    int prec;
    double bnrm2, ini_res, error, fin_res;
    double rho, rho_old, alpha, beta;
    int iter, done, niter_out, status;
    int early, loops, loop_limit, true_res;
    unsigned int counter;
    unsigned int pad0;
    unsigned long long t_spmv0, t_sweep0;
    unsigned long long spmv_ns, spmv_n, sweep_ns, sweep_n;
    // TFS_MIXED bookkeeping
    double r_true;       // norm of the last binary64 true residual
    double delta;        // reliable-update threshold
    int need_true;       // the next true-residual step must run
    int pad1;
    // beta (above) = rho / rho_old of the coming p update (Cg.f90:114-119)
    // and its binary32 rounding, computed once by the thread that finalises
    // rho instead of by every thread
    float beta32;
    float alpha32;       // (float) alpha, published with alpha
    // global timer (ns) at the start of the solve's first kernel and at the
    // start of its epilogue
    unsigned long long t_begin, t_end;
    // tfs_profile_prec only (else null): per sweep launch ("slot") and block,
    // the global timer after the block's dependency wait and at its end
    unsigned long long *stamps;
    int stamp_stride;      // entries per slot (2 per block)
    int pad3;
    // tfs_diag_dic_timeout: > 0, the one-block DIC's waits give up after
    // this many ns and its copy lane stages nothing (its first wait runs
    // out); 0, the normal limit
    unsigned long long dicb_wait_ns;
};

// Per-call arguments, written by the host before every graph launch.
struct DevParams {
    double tol;
    int niter_max;
    int x0_zero;             // 1: start from x0 = 0 instead of reading x
    const double *val_csr;   // natural CSR order, nnz
    const double *b;         // natural order, n (r1 on entry)
    double *x;               // natural order, n (in/out)
    double *r_out;           // natural order, n (r1 on return)
    unsigned long long dicb_wait_ns;   // DevState::dicb_wait_ns of the call
};

struct SellDev {
    int n_int;
    int n_chunks;
    const uint32_t *rowinfo;
    const int *slice_off;
    const int *col;
    int width;    // > 0: every slice has this width (slice s starts at 32*width*s)
};

// Work vectors (binary64).
struct Vec64 {
    double *x, *r, *r2, *p, *p2, *q, *q2, *u1, *u2, *v2, *w, *d, *y, *y2, *z, *z2;
};
// Work vectors (binary32) of the mixed-precision inner iteration.
struct Vec32 {
    float *r, *r2, *p, *p2, *q, *q2, *u1, *u2, *v2, *w, *d, *y, *y2, *z, *z2;
    float *e;   // solution correction since the last binary64 true residual
};

struct FaceMap;   // tfs_assemble.cu

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    int prologue_kernels = 0, body_kernels = 0, epilogue_kernels = 0;
};

struct tfs_handle {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr, stream2 = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, tev0 = nullptr, tev1 = nullptr, ev_done = nullptr;
    const struct GraphEntry *last_graph = nullptr;
    int32_t n = 0, nnz = 0;
    int n_int = 0, n_chunks = 0, n_slices = 0, nnz_pad = 0, n_levels = 0;
    int sell_width = 0;                // uniform slice width (0: per-slice widths)
    int spmv_kind = 0;                 // TFS_SPMV_DIRECT / _PIPE: kernel of the CG SpMV
    int grid = 0;                      // blocks of the vector kernels (grid-stride)
    int grid_spmv = 0;                 // blocks of the SpMV-type kernels
    int grid_vec4 = 0;                 // blocks of the 16-byte binary32 vector kernels
    int vec4 = 1;                      // 1: binary32 CG vector kernels with 16-byte loads
    // Options (tfs_set_option; every default is the measured fastest).
    int use_pdl = 1;                   // TFS_OPT_PDL: programmatic dependent launch between level kernels
    int pdl_vec = 1;                   // TFS_OPT_PDL_VEC: CG vector kernels PDL-chained
    int fwd_pre = 1;                   // TFS_OPT_FWD_PRE: forward level kernels load b and D before the wait
    int bwd_pre = 1;                   // TFS_OPT_BWD_PRE: backward level kernels after a tail compute start values before the wait
    int tail_pf = 1;                   // TFS_OPT_TAIL_PF: prefetching tail (k_sweep_tail1)
    int fuse_l0 = 2;                   // TFS_OPT_FUSE_L0: DIC-CG level 0 inside the neighbouring kernels (1: binary32 only, 2: both)
    int level_tpb = TFS_TPB;           // TFS_OPT_LEVEL_TPB: threads per block of the level kernels
                                       // (128/256/512/1024 measured 147.7/146.4/147.4/150.1 us per DIC application)
    int sell_uniform = 1;              // TFS_OPT_SELL_UNIFORM: one slice width when it costs <= 5% padding
    int spmv_pref = 1;                 // TFS_OPT_SPMV: 1 software-pipelined where possible, 0 direct
    int spmv_chunks = 0;               // TFS_OPT_SPMV_GRID: 1 one block per 256-row chunk
    int eager = 0;                     // TFS_OPT_LAUNCH: 1 launch kernels from a host loop, no CUDA graph
    int bicg_literal = 0;              // TFS_OPT_BICG: 1 BiCG runs its shadow sequence explicitly
    int dic_block = 1;                 // TFS_OPT_DIC_BLOCK: 1 one-block DIC where the vector and two slots of the widest level fit
    unsigned long long dicb_diag_ns = 0;   // tfs_diag_dic_timeout
    int l2_window = 1;                 // TFS_OPT_L2_WINDOW: 1 the column indices persisting in L2
    int dicb_used = 0;                 // the last DIC application launched was the one-block kernel
    // One-block DIC per arithmetic: shared memory (0: does not fit), ring
    // slot capacity (rows and SELL entries), number of level groups and the
    // offset of the group table in d_lvl_begin's allocation.
    struct DicbPlan {
        int bytes = 0, rm = 0, ents = 0, n_groups = 0, group_off = 0;
    } dicb64, dicb32;
    std::vector<int> lvl_tab;          // host copy of d_lvl_begin's allocation (levels, then both group tables)
    bool profiling = false;            // tfs_profile_prec: number the sweep launches
    int stamp_next = 0;                // next slot number while profiling
    std::vector<int> stamp_kind;       // per slot: level (forward), -1 - level (backward), 1 << 20 tail
    int pf_tail_level = 0;             // first level of the prefetching tail
    bool pf_ok = false;                // the prefetching tail can run
    int precision = TFS_FP64;
    std::vector<int> lvl_begin;        // internal row offset of every level (+end)
    std::vector<int32_t> levels_nat;   // level per natural row
    uint64_t fingerprint = 0;
    std::vector<int> row0, col0, dia0;  // the topology, 0-based (host copy)
    std::vector<int> rcm_pos;          // RCM position of every natural row
    int layout = -1;                   // TFS_LAYOUT_* built, -1 none yet
    int layout_pref = TFS_LAYOUT_RCM;  // TFS_OPT_LAYOUT = 1 forces level order
    int64_t fixed_bytes = 0;           // device bytes independent of the layout
    // device arrays
    int *perm = nullptr, *iperm = nullptr, *slice_off = nullptr, *col = nullptr, *vmap = nullptr;
    uint32_t *rowinfo = nullptr;
    double *val = nullptr;
    float *val32 = nullptr;
    double *stage_val = nullptr, *stage_b = nullptr, *stage_x = nullptr;
    double *part = nullptr;
    int *d_lvl_begin = nullptr;
    int tail_level = 0;                // first level of the one-block tail
    DevState *st = nullptr;
    DevParams *params = nullptr;
    void *vec_pool = nullptr, *vec32_pool = nullptr;
    Vec64 v{};
    Vec32 f{};
    // pinned host mirror of params and state
    DevParams *h_params = nullptr;
    DevState *h_state = nullptr;
    std::map<int, GraphEntry> graphs;  // key: method | prec << 4 | precision << 8
    tfs_stats stats{};
    int64_t device_bytes = 0;
    FaceMap *faces = nullptr;          // tfs_faces_register
};

// tfs_engine.cu
int tfs_engine_error(cudaError_t e, const char *what);
void tfs_set_error_text(const char *msg);
// Enqueue a whole solve on h->stream (ends with h->ev_done), then read its
// outputs once h->ev_done has completed.
int tfs_solve_launch(int method, tfs_handle *h, const double *val, double *x, double *r1,
                     int32_t prec, int32_t niter, double tol, bool device_ptrs,
                     const double *b_in = nullptr, int x0_zero = 0);
int tfs_solve_collect(tfs_handle *h, int32_t *niter, double *ini_res, double *fin_res);
// Device bytes a topology will hold once its layout is built (estimate).
int64_t tfs_estimate_bytes(int32_t n, int32_t nnz);
// tfs_assemble.cu
void tfs_faces_free(tfs_handle *h);
