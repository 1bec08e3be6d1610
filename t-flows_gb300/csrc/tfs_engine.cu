// tfs_engine.cu -- handles, device layout, CUDA-graph solve loop and the
// C ABI of libtfs_gb300.so (declared in include/tfs_solver.h).
//
// One solve is one CUDA graph launch:
//   prologue  k_init, k_gather_val, k_load (||b||), DIC form by levels,
//             k_residual (r = b - A x, ||r0||)
//   WHILE     conditional node; its body is one Krylov iteration and the
//             body's last kernel sets the condition from the convergence test
//   epilogue  k_store (x and r1 back to natural order)
// The graph of each (method, prec, arithmetic) is built once per handle and
// reused; per-call arguments go through a small DevParams block copied in
// before the launch.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "tfs_internal.h"
#include "tfs_kernels.cuh"
#include "tfs_mixed.cuh"
#include "tfs_spmv.cuh"
#include "tfs_dic_block.cuh"

using namespace tfs;

// ------------------------------------------------------------ errors

static thread_local std::string g_err;

void tfs_set_error_text(const char *msg) { g_err = msg ? msg : ""; }

int tfs_engine_error(cudaError_t e, const char *what)
{
    char buf[512];
    snprintf(buf, sizeof buf, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    g_err = buf;
    return TFS_ERR_CUDA;
}

#define CK(call)                                                        \
    do {                                                                \
        cudaError_t _e = (call);                                        \
        if (_e != cudaSuccess) return tfs_engine_error(_e, #call);      \
    } while (0)

#define CKL(what)                                                       \
    do {                                                                \
        cudaError_t _e = cudaGetLastError();                            \
        if (_e != cudaSuccess) return tfs_engine_error(_e, what);       \
    } while (0)

extern "C" const char *tfs_last_error(void) { return g_err.c_str(); }

extern "C" const char *tfs_status_string(int s)
{
    switch (s) {
    case TFS_OK: return "ok";
    case TFS_ERR_ARG: return "invalid argument";
    case TFS_ERR_MATRIX: return "malformed matrix";
    case TFS_ERR_CUDA: return "CUDA error";
    case TFS_ERR_NONFINITE: return "non-finite residual (breakdown)";
    case TFS_ERR_TOPOLOGY: return "arrays do not match the registered topology";
    case TFS_ERR_TIMEOUT: return "device-side iteration guard expired";
    case TFS_ERR_BUDGET: return "device memory budget exceeded";
    default: return "unknown status";
    }
}

// ------------------------------------------------------------ helpers

static SellDev sell_of(const tfs_handle *h)
{
    SellDev A;
    A.n_int = h->n_int;
    A.n_chunks = h->n_chunks;
    A.rowinfo = h->rowinfo;
    A.slice_off = h->slice_off;
    A.col = h->col;
    A.width = h->sell_width;
    return A;
}

// Kernel launch with programmatic dependent launch allowed (PDL) when pdl.
template <typename... KArgs, typename... Args>
static cudaError_t launch_ex(bool pdl, void (*kernel)(KArgs...), int grid, int block, cudaStream_t s,
                             Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, ((KArgs)args)...);
}

// launch_ex with dynamic shared memory.
template <typename... KArgs, typename... Args>
static cudaError_t launch_ex_smem(bool pdl, void (*kernel)(KArgs...), int grid, int block, int smem,
                                  cudaStream_t s, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = (size_t)smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, ((KArgs)args)...);
}

// One kernel per large level (PDL-chained), then the tail levels in one
// block; MODE 1 runs the tail first and the levels in descending order.
template <typename T, int NR, int MODE>
static int launch_levels(tfs_handle *h, cudaStream_t s, const T *val, T *d, const T *b1, const T *b2,
                         T *o1, T *o2, const T *y1, const T *y2, int *count, bool with_tail = true,
                         int tail_at = -1, int lvl_from = 0, bool prey = false)
{
    SellDev A = sell_of(h);
    const int L = h->n_levels, tail = tail_at >= 0 ? tail_at : h->tail_level;
    const bool pdl = h->use_pdl != 0;
    int first = 1;
    auto tail_launch = [&]() -> cudaError_t {
        if (tail >= L || !with_tail) return cudaSuccess;
        (*count)++;
        cudaError_t e = launch_ex(pdl, k_sweep_tail<T, NR, MODE>, 1, TFS_SWEEP_TPB, s, A, val, d, b1, b2, o1, o2,
                                  y1, y2, (const int *)h->d_lvl_begin, tail, L, h->st, first);
        first = 0;
        return e;
    };
    if (MODE == 1) {
        cudaError_t e = tail_launch();
        if (e != cudaSuccess) return tfs_engine_error(e, "tail launch");
    }
    for (int q = 0; q < tail; q++) {
        const int l = MODE == 1 ? tail - 1 - q : q;
        if (l < lvl_from) continue;
        const int r0 = h->lvl_begin[l], r1 = h->lvl_begin[l + 1];
        const int bs = h->level_tpb;
        const int nb = (r1 - r0 + bs - 1) / bs;
        cudaError_t e;
        if (h->profiling && MODE != 2) {
            h->stamp_kind.push_back(MODE == 0 ? l : -1 - l);
            first = (first & 1) | (h->stamp_next++ << 1);
        }
        if ((MODE == 1 || MODE == 0) && prey) {
            // Backward levels after a tail that releases them only past its
            // own wait: start values computed before the dependency wait;
            // forward levels: right-hand side and D loaded before it.
            if (bs == 1024)
                e = launch_ex(pdl, k_sweep_level<T, NR, MODE, 1024, true>, nb, bs, s, A, val, d, b1, b2, o1, o2, y1, y2, r0, r1, h->st, first);
            else if (bs == 512)
                e = launch_ex(pdl, k_sweep_level<T, NR, MODE, 512, true>, nb, bs, s, A, val, d, b1, b2, o1, o2, y1, y2, r0, r1, h->st, first);
            else if (bs == 128)
                e = launch_ex(pdl, k_sweep_level<T, NR, MODE, 128, true>, nb, bs, s, A, val, d, b1, b2, o1, o2, y1, y2, r0, r1, h->st, first);
            else
                e = launch_ex(pdl, k_sweep_level<T, NR, MODE, 256, true>, nb, bs, s, A, val, d, b1, b2, o1, o2, y1, y2, r0, r1, h->st, first);
        } else if (bs == 1024)
            e = launch_ex(pdl, k_sweep_level<T, NR, MODE, 1024>, nb, bs, s, A, val, d, b1, b2, o1, o2, y1, y2, r0, r1, h->st, first);
        else if (bs == 512)
            e = launch_ex(pdl, k_sweep_level<T, NR, MODE, 512>, nb, bs, s, A, val, d, b1, b2, o1, o2, y1, y2, r0, r1, h->st, first);
        else if (bs == 128)
            e = launch_ex(pdl, k_sweep_level<T, NR, MODE, 128>, nb, bs, s, A, val, d, b1, b2, o1, o2, y1, y2, r0, r1, h->st, first);
        else
            e = launch_ex(pdl, k_sweep_level<T, NR, MODE, 256>, nb, bs, s, A, val, d, b1, b2, o1, o2, y1, y2, r0, r1, h->st, first);
        if (e != cudaSuccess) return tfs_engine_error(e, "level launch");
        first = 0;   // (and slot 0: stamps are recorded only while profiling)
        (*count)++;
    }
    if (MODE != 1) {
        cudaError_t e = tail_launch();
        if (e != cudaSuccess) return tfs_engine_error(e, "tail launch");
    }
    return TFS_OK;
}

template <typename T>
static int dalloc(tfs_handle *h, T **p, size_t count)
{
    size_t bytes = count * sizeof(T);
    if (bytes == 0) bytes = sizeof(T);
    CK(cudaMalloc((void **)p, bytes));
    h->device_bytes += (int64_t)bytes;
    return TFS_OK;
}

// The SpMV kernel of the CG iterations: the software-pipelined kernel for
// uniform-width matrices (width <= 8), else the direct kernel; both give
// bitwise the same results (TFS_OPT_SPMV = 0 forces the direct one).
static void spmv_kind_setup(tfs_handle *h)
{
    h->spmv_kind = (h->sell_width > 0 && h->sell_width <= 8 && h->spmv_pref != 0) ? TFS_SPMV_PIPE
                                                                                : TFS_SPMV_DIRECT;
}

template <typename VT, bool MIXED>
static void launch_spmv_pipe(const tfs_handle *h, cudaStream_t s, const VT *val, const VT *p, VT *q, bool pdl)
{
    const SellDev A = sell_of(h);
    const int G = h->grid_spmv;
    switch (h->sell_width) {
    case 1: launch_ex(pdl, k_spmv_pq_pipe<VT, MIXED, 1>, G, TFS_TPB, s, A, val, p, q, h->st, h->part); break;
    case 2: launch_ex(pdl, k_spmv_pq_pipe<VT, MIXED, 2>, G, TFS_TPB, s, A, val, p, q, h->st, h->part); break;
    case 3: launch_ex(pdl, k_spmv_pq_pipe<VT, MIXED, 3>, G, TFS_TPB, s, A, val, p, q, h->st, h->part); break;
    case 4: launch_ex(pdl, k_spmv_pq_pipe<VT, MIXED, 4>, G, TFS_TPB, s, A, val, p, q, h->st, h->part); break;
    case 5: launch_ex(pdl, k_spmv_pq_pipe<VT, MIXED, 5>, G, TFS_TPB, s, A, val, p, q, h->st, h->part); break;
    case 6: launch_ex(pdl, k_spmv_pq_pipe<VT, MIXED, 6>, G, TFS_TPB, s, A, val, p, q, h->st, h->part); break;
    case 7: launch_ex(pdl, k_spmv_pq_pipe<VT, MIXED, 7>, G, TFS_TPB, s, A, val, p, q, h->st, h->part); break;
    default: launch_ex(pdl, k_spmv_pq_pipe<VT, MIXED, 8>, G, TFS_TPB, s, A, val, p, q, h->st, h->part); break;
    }
}

// q = A p, (p, q) and alpha of a CG iteration on stream s, binary32 (mixed)
// or binary64, with the handle's SpMV kernel over grid_spmv (virtual)
// blocks.
static void launch_spmv_pq(tfs_handle *h, cudaStream_t s, bool mixed, bool pdl = false)
{
    const SellDev A = sell_of(h);
    const int VG = h->grid_spmv;
    if (h->spmv_kind == TFS_SPMV_PIPE) {
        if (mixed) launch_spmv_pipe<float, true>(h, s, h->val32, h->f.p, h->f.q, pdl);
        else launch_spmv_pipe<double, false>(h, s, h->val, h->v.p, h->v.q, pdl);
    } else if (mixed) {
        k_mx_spmv_pq<<<VG, TFS_TPB, 0, s>>>(A, h->val32, h->f.p, h->f.q, h->st, h->part);
    } else {
        k_spmv_pq<<<VG, TFS_TPB, 0, s>>>(A, h->val, h->v.p, h->v.q, h->st, h->part);
    }
}

static uint64_t fingerprint(int32_t n, int32_t nnz, const int32_t *row1, const int32_t *col1,
                            const int32_t *dia1)
{
    uint64_t f = 1469598103934665603ull;
    auto mix = [&](uint64_t v) { f = (f ^ v) * 1099511628211ull; };
    mix((uint64_t)n);
    mix((uint64_t)nnz);
    for (int k = 0; k < 64; k++) {
        int64_t i = (int64_t)n * k / 64, j = (int64_t)nnz * k / 64;
        mix((uint64_t)row1[i]);
        mix((uint64_t)col1[j]);
        mix((uint64_t)dia1[i]);
    }
    mix((uint64_t)row1[n]);
    return f;
}

// Checks the Matrix_Type invariants the kernels rely on.
static int validate_csr(int32_t n, int32_t nnz, const int32_t *row1, const int32_t *col1,
                        const int32_t *dia1)
{
    if (n <= 0 || nnz < n || !row1 || !col1 || !dia1) {
        tfs_set_error_text("n must be positive, nnz >= n, arrays non-null");
        return TFS_ERR_ARG;
    }
    if (row1[0] != 1 || row1[n] - 1 != nnz) {
        tfs_set_error_text("row(1) must be 1 and row(n+1)-1 must equal nnz");
        return TFS_ERR_MATRIX;
    }
    for (int32_t i = 0; i < n; i++) {
        int32_t a = row1[i], b = row1[i + 1];
        if (b <= a || b - a > 65535) {
            tfs_set_error_text("every row needs 1..65535 entries (the diagonal at least)");
            return TFS_ERR_MATRIX;
        }
        for (int32_t p = a; p < b; p++) {
            int32_t c = col1[p - 1];
            if (c < 1 || c > n || (p > a && c <= col1[p - 2])) {
                tfs_set_error_text("column numbers must lie in 1..n and ascend within a row");
                return TFS_ERR_MATRIX;
            }
        }
        int32_t d = dia1[i];
        if (d < a || d >= b || col1[d - 1] != i + 1) {
            tfs_set_error_text("dia(i) must point at column i inside row i");
            return TFS_ERR_MATRIX;
        }
    }
    return TFS_OK;
}

// ------------------------------------------------------- registration

// Dependency lists of the level analysis: for row i every k < i that the
// forward sweep reads (a_ik != 0) and, when the pattern is not structurally
// symmetric, every k < i whose row reads i in the backward sweep (a_ki != 0),
// so that descending levels are a valid backward schedule too.
static void dependency_lists(int n, const std::vector<int> &row0, const std::vector<int> &col0,
                             const std::vector<int> &dia0, std::vector<int> &lrow,
                             std::vector<int> &lcol)
{
    auto has = [&](int r, int c) {
        int lo = row0[r], hi = row0[r + 1] - 1;
        while (lo <= hi) {
            int mid = lo + (hi - lo) / 2;
            if (col0[mid] == c) return true;
            if (col0[mid] < c) lo = mid + 1; else hi = mid - 1;
        }
        return false;
    };
    bool sym = true;
    for (int i = 0; i < n && sym; i++)
        for (int j = row0[i]; j < row0[i + 1]; j++)
            if (col0[j] != i && !has(col0[j], i)) { sym = false; break; }
    lrow.assign(n + 1, 0);
    if (sym) {
        for (int i = 0; i < n; i++) lrow[i + 1] = lrow[i] + (dia0[i] - row0[i]);
        lcol.resize(lrow[n]);
        for (int i = 0; i < n; i++)
            for (int j = row0[i]; j < dia0[i]; j++) lcol[lrow[i] + (j - row0[i])] = col0[j];
        return;
    }
    std::vector<std::vector<int>> dep(n);
    for (int i = 0; i < n; i++)
        for (int j = row0[i]; j < row0[i + 1]; j++) {
            int k = col0[j];
            if (k < i) dep[i].push_back(k);
            else if (k > i) dep[k].push_back(i);
        }
    for (int i = 0; i < n; i++) {
        std::sort(dep[i].begin(), dep[i].end());
        dep[i].erase(std::unique(dep[i].begin(), dep[i].end()), dep[i].end());
        lrow[i + 1] = lrow[i] + (int)dep[i].size();
    }
    lcol.resize(lrow[n]);
    for (int i = 0; i < n; i++) std::copy(dep[i].begin(), dep[i].end(), lcol.begin() + lrow[i]);
}

static int compute_levels(tfs_handle *h, const std::vector<int> &lrow, const std::vector<int> &lcol,
                          std::vector<int32_t> &level)
{
    const int n = h->n;
    const size_t ndep = lcol.size();
    int *d_row = nullptr, *d_col = nullptr, *d_lvl = nullptr, *d_chg = nullptr;
    int rc = TFS_OK;
    const int PASSES = 8;
    auto cleanup = [&]() {
        cudaFree(d_row); cudaFree(d_col); cudaFree(d_lvl); cudaFree(d_chg);
    };
#define CKC(call)                                                       \
    do {                                                                \
        cudaError_t _e = (call);                                        \
        if (_e != cudaSuccess) { rc = tfs_engine_error(_e, #call); cleanup(); return rc; } \
    } while (0)
    CKC(cudaMalloc(&d_row, sizeof(int) * (n + 1)));
    CKC(cudaMalloc(&d_col, sizeof(int) * (ndep ? ndep : 1)));
    CKC(cudaMalloc(&d_lvl, sizeof(int) * n));
    CKC(cudaMalloc(&d_chg, sizeof(int) * PASSES));
    CKC(cudaMemcpyAsync(d_row, lrow.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, h->stream));
    if (ndep) CKC(cudaMemcpyAsync(d_col, lcol.data(), sizeof(int) * ndep, cudaMemcpyHostToDevice, h->stream));
    CKC(cudaMemsetAsync(d_lvl, 0, sizeof(int) * n, h->stream));
    int grid = (n + 255) / 256;
    if (grid > h->sm_count * 8) grid = h->sm_count * 8;
    // The longest dependency chain bounds the passes: at most n + 1.
    for (int64_t done_passes = 0; done_passes <= (int64_t)n + PASSES; done_passes += PASSES) {
        CKC(cudaMemsetAsync(d_chg, 0, sizeof(int) * PASSES, h->stream));
        for (int p = 0; p < PASSES; p++)
            k_level_pass<<<grid, 256, 0, h->stream>>>(n, d_row, d_col, d_lvl, d_chg + p);
        CKC(cudaGetLastError());
        int chg[PASSES];
        CKC(cudaMemcpyAsync(chg, d_chg, sizeof chg, cudaMemcpyDeviceToHost, h->stream));
        CKC(cudaStreamSynchronize(h->stream));
        if (chg[PASSES - 1] == 0) break;
    }
    level.resize(n);
    CKC(cudaMemcpyAsync(level.data(), d_lvl, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
    CKC(cudaStreamSynchronize(h->stream));
#undef CKC
    cleanup();
    return TFS_OK;
}

// Reverse Cuthill-McKee order of the (structurally symmetrised) pattern: BFS
// from a pseudo-peripheral row of each connected component, neighbours by
// increasing degree, the whole order reversed.  rcm_pos[row] = position.
// Keeping rows that are close in the mesh close in memory lets the 32 lanes
// of a warp gather from shared 32-byte sectors: with the random cell numbers
// of the workloads this cuts the gathered sectors per SpMV about 2.4x inside
// a DIC level and about 8x without levels (measured on the 64^3 system).
static void rcm_order(int n, const std::vector<int> &row0, const std::vector<int> &col0,
                      std::vector<int> &rcm_pos)
{
    std::vector<int> deg(n);
    for (int i = 0; i < n; i++) deg[i] = row0[i + 1] - row0[i];
    std::vector<int> order;
    order.reserve(n);
    std::vector<char> seen(n, 0);
    std::vector<int> nb;
    auto bfs = [&](int start, std::vector<int> &out, std::vector<int> *depth) {
        size_t head = out.size();
        out.push_back(start);
        seen[start] = 1;
        if (depth) (*depth)[start] = 0;
        while (head < out.size()) {
            int u = out[head++];
            nb.clear();
            for (int j = row0[u]; j < row0[u + 1]; j++) {
                int v = col0[j];
                if (!seen[v]) { seen[v] = 1; nb.push_back(v); }
            }
            std::sort(nb.begin(), nb.end(), [&](int a, int c) { return deg[a] != deg[c] ? deg[a] < deg[c] : a < c; });
            for (int v : nb) {
                if (depth) (*depth)[v] = (*depth)[u] + 1;
                out.push_back(v);
            }
        }
    };
    std::vector<int> comp, depth(n, 0);
    for (int s0 = 0; s0 < n; s0++) {
        if (seen[s0]) continue;
        // Pseudo-peripheral start: two BFS sweeps from s0.
        comp.clear();
        bfs(s0, comp, &depth);
        int far = comp.back();
        for (int v : comp) seen[v] = 0;
        comp.clear();
        bfs(far, comp, &depth);
        int far2 = comp.back();
        for (int v : comp) seen[v] = 0;
        size_t before = order.size();
        bfs(far2, order, nullptr);
        std::reverse(order.begin() + (long)before, order.end());
    }
    rcm_pos.assign(n, 0);
    for (int k = 0; k < n; k++) rcm_pos[order[k]] = k;
}

static void free_layout(tfs_handle *h)
{
    for (auto &kv : h->graphs) {
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
    }
    h->graphs.clear();
    void *ptrs[] = {h->perm, h->iperm, h->rowinfo, h->slice_off, h->col, h->vmap, h->val, h->val32,
                    h->d_lvl_begin, h->vec_pool, h->vec32_pool, h->part};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    h->perm = h->iperm = h->slice_off = h->col = h->vmap = nullptr;
    h->rowinfo = nullptr;
    h->val = nullptr;
    h->val32 = nullptr;
    h->d_lvl_begin = nullptr;
    h->vec_pool = h->vec32_pool = nullptr;
    h->part = nullptr;
    h->device_bytes = h->fixed_bytes;
    h->layout = -1;
}

// Device layout in one of two row orders: TFS_LAYOUT_RCM (reverse
// Cuthill-McKee) for solves without DIC, TFS_LAYOUT_LEVELS (DIC level, then
// RCM position inside a level) which every preconditioner can use.
static int build_layout(tfs_handle *h, int kind)
{
    const int n = h->n;
    const std::vector<int> &row0 = h->row0, &col0 = h->col0, &dia0 = h->dia0;
    CK(cudaStreamSynchronize(h->stream));
    free_layout(h);
    int rc;
    int nl = 1;
    std::vector<int32_t> level(n, 0);
    if (kind == TFS_LAYOUT_LEVELS) {
        std::vector<int> lrow, lcol;
        dependency_lists(n, row0, col0, dia0, lrow, lcol);
        if ((rc = compute_levels(h, lrow, lcol, level))) return rc;
        nl = 0;
        for (int i = 0; i < n; i++) {
            if (level[i] < 0 || level[i] >= n) { tfs_set_error_text("level analysis failed"); return TFS_ERR_CUDA; }
            if (level[i] + 1 > nl) nl = level[i] + 1;
        }
        h->levels_nat.assign(level.begin(), level.end());
    }
    // Rows by (level, RCM position); each level padded to a multiple of 32.
    std::vector<int> byrcm(n);
    for (int i = 0; i < n; i++) byrcm[h->rcm_pos[i]] = i;
    std::vector<int> cnt(nl, 0);
    for (int i = 0; i < n; i++) cnt[level[i]]++;
    h->lvl_begin.assign(nl + 1, 0);
    for (int l = 0; l < nl; l++) h->lvl_begin[l + 1] = h->lvl_begin[l] + ((cnt[l] + 31) & ~31);
    const int quad = 4 * TFS_TPB;
    int64_t n_int64 = ((int64_t)h->lvl_begin[nl] + quad - 1) / quad * quad;
    if (n_int64 > INT32_MAX / 2) { tfs_set_error_text("matrix too large"); return TFS_ERR_ARG; }
    const int n_int = (int)n_int64;
    std::vector<int> perm(n_int, -1), iperm(n), fillp(nl);
    for (int l = 0; l < nl; l++) fillp[l] = h->lvl_begin[l];
    for (int k = 0; k < n; k++) {
        int i = byrcm[k];
        int p = fillp[level[i]]++;
        perm[p] = i;
        iperm[i] = p;
    }
    // SELL-32 slices.
    const int n_slices = n_int / 32;
    std::vector<uint32_t> rowinfo(n_int, 0u);
    std::vector<int> slice_off(n_slices + 1, 0);
    for (int p = 0; p < n_int; p++) {
        int o = perm[p];
        if (o >= 0) rowinfo[p] = (uint32_t)(row0[o + 1] - row0[o]) | ((uint32_t)(dia0[o] - row0[o]) << 16);
    }
    int64_t off = 0;
    int wmax = 0;
    for (int s = 0; s < n_slices; s++) {
        int w = 0;
        for (int t = 0; t < 32; t++) {
            int len = (int)(rowinfo[32 * s + t] & 0xffffu);
            if (len > w) w = len;
        }
        if (w > wmax) wmax = w;
        slice_off[s] = (int)off;
        off += 32 * (int64_t)w;
        if (off > INT32_MAX) { tfs_set_error_text("padded matrix exceeds 2^31 entries"); return TFS_ERR_ARG; }
    }
    slice_off[n_slices] = (int)off;
    // One width for every slice (the slice offset computed instead of
    // loaded) when rows have at most 8 entries and it costs at most 5% more
    // slots: the 7-entry rows of a hex mesh.  Measured equal to per-slice
    // widths on the 128^3 system (binary32 SpMV 39.3 against 39.5 us);
    // TFS_OPT_SELL_UNIFORM = 0 keeps per-slice widths.
    h->sell_width = 0;
    {
        const int64_t uni = 32 * (int64_t)wmax * n_slices;
        if (h->sell_uniform && wmax > 0 && wmax <= 8 && uni <= off + off / 20 && uni <= INT32_MAX) {
            h->sell_width = wmax;
            for (int s = 0; s <= n_slices; s++) slice_off[s] = 32 * wmax * s;
            off = uni;
        }
    }
    const int nnz_pad = (int)off;
    std::vector<int> colx((size_t)nnz_pad, 0), vmap((size_t)nnz_pad, -1);
    for (int p = 0; p < n_int; p++) {
        int o = perm[p];
        if (o < 0) continue;
        int base = slice_off[p >> 5] + (p & 31);
        for (int j = 0; j < row0[o + 1] - row0[o]; j++) {
            colx[(size_t)base + 32 * (size_t)j] = iperm[col0[row0[o] + j]];
            vmap[(size_t)base + 32 * (size_t)j] = row0[o] + j;
        }
    }
    h->n_int = n_int;
    h->n_chunks = n_int / TFS_TPB;
    h->n_slices = n_slices;
    h->nnz_pad = nnz_pad;
    h->n_levels = nl;
    int g = h->sm_count * 8;
    h->grid = h->n_chunks < g ? h->n_chunks : g;
    if (h->grid < 1) h->grid = 1;
    // SpMV-type kernels: 8 blocks per SM, grid-stride over the 256-row
    // chunks (measured faster than one chunk per block on the 128^3
    // system: 42.5 us against 72.9 us); TFS_OPT_SPMV_GRID = 1 selects the
    // latter (the autotuner times both).
    h->grid_spmv = h->spmv_chunks ? h->n_chunks : h->grid;
    // Binary32 CG vector kernels: 16-byte loads, grid-stride over the same
    // grid as the other vector kernels.
    h->vec4 = 1;
    h->grid_vec4 = h->grid < h->n_int / (4 * TFS_TPB) ? h->grid : h->n_int / (4 * TFS_TPB);
    if (h->grid_vec4 < 1) h->grid_vec4 = 1;

    if ((rc = dalloc(h, &h->perm, n_int)) || (rc = dalloc(h, &h->iperm, n)) ||
        (rc = dalloc(h, &h->rowinfo, n_int)) || (rc = dalloc(h, &h->slice_off, n_slices + 1)) ||
        (rc = dalloc(h, &h->col, nnz_pad)) || (rc = dalloc(h, &h->vmap, nnz_pad)) ||
        (rc = dalloc(h, &h->val, nnz_pad)) || (rc = dalloc(h, &h->val32, nnz_pad)) ||
        (rc = dalloc(h, &h->part, TFS_NPART * (size_t)h->n_chunks + 64)))
        return rc;
    {
        // The tail: the levels after the last level with more than
        // TFS_TAIL_ROWS rows, swept by one block (level 0 is never part of it).
        int tail = nl;
        while (tail > 0 && h->lvl_begin[tail] - h->lvl_begin[tail - 1] <= TFS_TAIL_ROWS) tail--;
        if (tail == 0) tail = nl > 1 ? 1 : nl;
        h->tail_level = tail;
        // Prefetching tail (k_sweep_tail1): the longest suffix of levels
        // (never level 0) whose rows fit one per thread of one block, used
        // when it reaches at least as far down as the plain tail.  Spreading
        // it over a cluster (2-16 CTAs, the hardware cluster barrier between
        // levels) so that mid-sized levels join it measured no faster on the
        // 128^3 system (one block 128.8 us per DIC application; 2, 8, 16 CTAs
        // 131.8, 129.3, 126.3 us).
        int l = nl, rows = 0;
        while (l > 1 && rows + (h->lvl_begin[l] - h->lvl_begin[l - 1]) <= TFS_SWEEP_TPB) {
            rows += h->lvl_begin[l] - h->lvl_begin[l - 1];
            l--;
        }
        h->pf_tail_level = l;
        h->pf_ok = l < nl && l <= h->tail_level;
        // One-block DIC: the plan per arithmetic (tfs_dicb_plan.h); the
        // group tables follow the level table in d_lvl_begin's allocation.
        h->dicb64 = h->dicb32 = tfs_handle::DicbPlan{};
        h->lvl_tab.assign(h->lvl_begin.begin(), h->lvl_begin.end());
        if (kind == TFS_LAYOUT_LEVELS) {
            int optin = 0;
            CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
            auto keep = [&](const DicbPlanResult &r, tfs_handle::DicbPlan &P) {
                if (!r.bytes) return;
                P.bytes = r.bytes;
                P.rm = r.rm;
                P.ents = r.ents;
                P.n_groups = (int)r.groups.size() - 1;
                P.group_off = (int)h->lvl_tab.size();
                h->lvl_tab.insert(h->lvl_tab.end(), r.groups.begin(), r.groups.end());
            };
            keep(dicb_plan<double>(h->lvl_begin, slice_off, optin, TFS_DICB_SLOTS, TFS_DICB_MAX_LEVELS), h->dicb64);
            keep(dicb_plan<float>(h->lvl_begin, slice_off, optin, TFS_DICB_SLOTS, TFS_DICB_MAX_LEVELS), h->dicb32);
            // (a function attribute of the current device's context: set on
            // every layout build)
            const void *fns[] = {(const void *)k_dic_block<double, 0>, (const void *)k_dic_block<double, 2>,
                                 (const void *)k_dic_block<double, 3>, (const void *)k_dic_block<double, 4>,
                                 (const void *)k_dic_block<float, 0>, (const void *)k_dic_block<float, 3>,
                                 (const void *)k_dic_block<float, 4>};
            for (const void *f : fns) CK(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
        }
        if ((rc = dalloc(h, &h->d_lvl_begin, h->lvl_tab.size()))) return rc;
        CK(cudaMemcpyAsync(h->d_lvl_begin, h->lvl_tab.data(), sizeof(int) * h->lvl_tab.size(), cudaMemcpyHostToDevice,
                           h->stream));
    }
    spmv_kind_setup(h);
    CK(cudaMemcpyAsync(h->perm, perm.data(), sizeof(int) * n_int, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->iperm, iperm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->rowinfo, rowinfo.data(), sizeof(uint32_t) * n_int, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->slice_off, slice_off.data(), sizeof(int) * (n_slices + 1), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->col, colx.data(), sizeof(int) * (size_t)nnz_pad, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->vmap, vmap.data(), sizeof(int) * (size_t)nnz_pad, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemsetAsync(h->val, 0, sizeof(double) * (size_t)nnz_pad, h->stream));
    CK(cudaMemsetAsync(h->val32, 0, sizeof(float) * (size_t)nnz_pad, h->stream));
    CK(cudaMemsetAsync(h->part, 0, sizeof(double) * (TFS_NPART * (size_t)h->n_chunks + 64), h->stream));

    // Work vectors: 16 binary64 + 16 binary32, zero so padding rows stay zero.
    const size_t nv64 = 16, nv32 = 16;
    double *pool = nullptr;
    float *pool32 = nullptr;
    if ((rc = dalloc(h, &pool, nv64 * (size_t)n_int)) || (rc = dalloc(h, &pool32, nv32 * (size_t)n_int)))
        return rc;
    h->vec_pool = pool;
    h->vec32_pool = pool32;
    CK(cudaMemsetAsync(pool, 0, sizeof(double) * nv64 * (size_t)n_int, h->stream));
    CK(cudaMemsetAsync(pool32, 0, sizeof(float) * nv32 * (size_t)n_int, h->stream));
    double *v[16];
    for (size_t k = 0; k < nv64; k++) v[k] = pool + k * (size_t)n_int;
    h->v = Vec64{v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9], v[10], v[11], v[12], v[13], v[14], v[15]};
    float *f[16];
    for (size_t k = 0; k < nv32; k++) f[k] = pool32 + k * (size_t)n_int;
    h->f = Vec32{f[0], f[1], f[2], f[3], f[4], f[5], f[6], f[7], f[8], f[9], f[10], f[11], f[12], f[13], f[14], f[15]};
    CK(cudaStreamSynchronize(h->stream));
    h->layout = kind;
    h->stats.n_levels = h->n_levels;
    h->stats.device_bytes = h->device_bytes;
    return TFS_OK;
}

// The layout a solve with preconditioner `prec` needs: a level layout serves
// every preconditioner; DIC needs one.  Built on first use.
static int ensure_layout(tfs_handle *h, int prec)
{
    if (h->layout == TFS_LAYOUT_LEVELS) return TFS_OK;
    if (prec == 2 || h->layout_pref == TFS_LAYOUT_LEVELS) return build_layout(h, TFS_LAYOUT_LEVELS);
    if (h->layout == TFS_LAYOUT_RCM) return TFS_OK;
    return build_layout(h, TFS_LAYOUT_RCM);
}

static void free_handle(tfs_handle *h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_layout(h);
    tfs_faces_free(h);
    void *ptrs[] = {h->stage_val, h->stage_b, h->stage_x, h->st, h->params};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (h->h_params) cudaFreeHost(h->h_params);
    if (h->h_state) cudaFreeHost(h->h_state);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->tev0) cudaEventDestroy(h->tev0);
    if (h->tev1) cudaEventDestroy(h->tev1);
    if (h->ev_done) cudaEventDestroy(h->ev_done);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->stream2) cudaStreamDestroy(h->stream2);
    delete h;
}

extern "C" int tfs_topology_register(int32_t n, int32_t nnz, const int32_t *row1,
                                     const int32_t *col1, const int32_t *dia1, tfs_handle **out)
{
    if (!out) return TFS_ERR_ARG;
    *out = nullptr;
    int rc = validate_csr(n, nnz, row1, col1, dia1);
    if (rc) return rc;
    tfs_handle *h = new tfs_handle;
    h->n = n;
    h->nnz = nnz;
    h->fingerprint = fingerprint(n, nnz, row1, col1, dia1);
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) { delete h; return tfs_engine_error(e, "cudaGetDevice"); }
    e = cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->device);
    if (e != cudaSuccess) { delete h; return tfs_engine_error(e, "cudaDeviceGetAttribute"); }
#define CKH(call)                                                              \
    do {                                                                       \
        cudaError_t _e = (call);                                               \
        if (_e != cudaSuccess) { int _r = tfs_engine_error(_e, #call); free_handle(h); return _r; } \
    } while (0)
    CKH(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    CKH(cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking));
    CKH(cudaEventCreate(&h->ev0));
    CKH(cudaEventCreate(&h->ev1));
    CKH(cudaMallocHost((void **)&h->h_params, sizeof(DevParams)));
    CKH(cudaMallocHost((void **)&h->h_state, sizeof(DevState)));
#undef CKH
    h->row0.resize(n + 1);
    h->col0.resize((size_t)nnz);
    h->dia0.resize(n);
    for (int i = 0; i <= n; i++) h->row0[i] = row1[i] - 1;
    for (int j = 0; j < nnz; j++) h->col0[j] = col1[j] - 1;
    for (int i = 0; i < n; i++) h->dia0[i] = dia1[i] - 1;
    rcm_order(n, h->row0, h->col0, h->rcm_pos);
    if ((rc = dalloc(h, &h->stage_val, nnz)) || (rc = dalloc(h, &h->stage_b, n)) ||
        (rc = dalloc(h, &h->stage_x, n)) || (rc = dalloc(h, &h->st, 1)) ||
        (rc = dalloc(h, &h->params, 1))) {
        free_handle(h);
        return rc;
    }
    h->fixed_bytes = h->device_bytes;
    cudaMemsetAsync(h->st, 0, sizeof(DevState), h->stream);
    *out = h;
    return TFS_OK;
}

extern "C" int tfs_release(tfs_handle *h)
{
    if (!h) return TFS_ERR_ARG;
    free_handle(h);
    return TFS_OK;
}

extern "C" int tfs_set_precision(tfs_handle *h, int mode)
{
    if (!h || (mode != TFS_FP64 && mode != TFS_MIXED)) return TFS_ERR_ARG;
    h->precision = mode;
    return TFS_OK;
}

static void drop_graphs(tfs_handle *h)
{
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto &kv : h->graphs) {
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
    }
    h->graphs.clear();
    h->last_graph = nullptr;
}

// The field behind an option and the values it accepts.
static int *option_field(tfs_handle *h, int option, bool (**ok)(int))
{
    static bool (*const bit)(int) = [](int v) { return v == 0 || v == 1; };
    static bool (*const fuse)(int) = [](int v) { return v >= 0 && v <= 2; };
    static bool (*const tpb)(int) = [](int v) { return v == 128 || v == 256 || v == 512 || v == 1024; };
    *ok = bit;
    switch (option) {
    case TFS_OPT_LAUNCH: return &h->eager;
    case TFS_OPT_LAYOUT: return &h->layout_pref;
    case TFS_OPT_BICG: return &h->bicg_literal;
    case TFS_OPT_SELL_UNIFORM: return &h->sell_uniform;
    case TFS_OPT_SPMV: return &h->spmv_pref;
    case TFS_OPT_SPMV_GRID: return &h->spmv_chunks;
    case TFS_OPT_LEVEL_TPB: *ok = tpb; return &h->level_tpb;
    case TFS_OPT_TAIL_PF: return &h->tail_pf;
    case TFS_OPT_FUSE_L0: *ok = fuse; return &h->fuse_l0;
    case TFS_OPT_PDL: return &h->use_pdl;
    case TFS_OPT_PDL_VEC: return &h->pdl_vec;
    case TFS_OPT_FWD_PRE: return &h->fwd_pre;
    case TFS_OPT_BWD_PRE: return &h->bwd_pre;
    case TFS_OPT_DIC_BLOCK: return &h->dic_block;
    case TFS_OPT_L2_WINDOW: return &h->l2_window;
    default: return nullptr;
    }
}

extern "C" int tfs_set_option(tfs_handle *h, int option, int value)
{
    if (!h) return TFS_ERR_ARG;
    bool (*ok)(int) = nullptr;
    int *f = option_field(h, option, &ok);
    if (!f || !ok(value)) {
        tfs_set_error_text("tfs_set_option: unknown option or value");
        return TFS_ERR_ARG;
    }
    CK(cudaSetDevice(h->device));
    drop_graphs(h);
    *f = value;
    if (option == TFS_OPT_LAYOUT || option == TFS_OPT_SELL_UNIFORM) {
        free_layout(h);
    } else if (h->layout >= 0) {
        // launch shapes derived from options at layout time
        h->grid_spmv = h->spmv_chunks ? h->n_chunks : h->grid;
        spmv_kind_setup(h);
    }
    return TFS_OK;
}

extern "C" int tfs_diag_dic_timeout(tfs_handle *h, long long wait_ns)
{
    if (!h || wait_ns < 0 || wait_ns > 1000000000LL) {
        tfs_set_error_text("tfs_diag_dic_timeout: null handle or wait_ns outside [0, 1e9]");
        return TFS_ERR_ARG;
    }
    h->dicb_diag_ns = (unsigned long long)wait_ns;
    return TFS_OK;
}

extern "C" int tfs_get_option(const tfs_handle *h, int option, int *value)
{
    if (!h || !value) return TFS_ERR_ARG;
    bool (*ok)(int) = nullptr;
    int *f = option_field(const_cast<tfs_handle *>(h), option, &ok);
    if (!f) return TFS_ERR_ARG;
    *value = *f;
    return TFS_OK;
}

// ------------------------------------------------------ graph capture

// Whether the one-block DIC runs for arithmetic T (1) or not (0:
// TFS_OPT_DIC_BLOCK = 0, or the vector and two slots of the widest level do
// not fit); *bytes its dynamic shared memory.
template <typename T>
static int dic_block_kind(const tfs_handle *h, int *bytes = nullptr)
{
    if (!h->dic_block || h->layout != TFS_LAYOUT_LEVELS) return 0;
    const tfs_handle::DicbPlan &P = sizeof(T) == 8 ? h->dicb64 : h->dicb32;
    if (!P.bytes) return 0;
    if (bytes) *bytes = P.bytes;
    return 1;
}

// One-block DIC application z1 = M^-1 b1 (MODE 0) or recurrence (MODE 2).
// Its bulk copies want 16-byte aligned sources: every array it stages is a
// cudaMalloc base or one offset by a multiple of 32 elements, checked here
// anyway -- cudaErrorMisalignedAddress, with nothing launched, sends the
// caller to the level kernels.  A launch error stays pending for the
// caller's check.
template <typename T, int MODE>
static cudaError_t launch_dic_one_block(tfs_handle *h, cudaStream_t s, int bytes, const T *val, T *d,
                                        const T *b1, T *z1)
{
    const tfs_handle::DicbPlan &P = sizeof(T) == 8 ? h->dicb64 : h->dicb32;
    const SellDev A = sell_of(h);
    const uintptr_t chk = (uintptr_t)val | (uintptr_t)d | (uintptr_t)b1 | (uintptr_t)z1 | (uintptr_t)A.rowinfo |
                          (uintptr_t)A.col;
    if (chk & 15u) return cudaErrorMisalignedAddress;
    const DicbSlot L = dicb_slot<T>(P.rm, P.ents);
    const int *groups = h->d_lvl_begin + P.group_off;
    if (MODE == 0 && dicb_split<T>(h->n_levels)) {
        // forward sweep, the scaling on every SM, backward sweep
        const bool pdl = h->use_pdl != 0;
        const int rows = h->lvl_begin[h->n_levels];
        launch_ex_smem(false, k_dic_block<T, 3>, 1, TFS_DICB_TPB, bytes, s, A, val, d, b1, z1,
                       (const int *)h->d_lvl_begin, h->n_levels, groups, P.n_groups, L, TFS_DICB_SLOTS, h->st);
        launch_ex(pdl, k_dic_scale<T>, std::min(h->grid, (rows + 255) / 256), 256, s, (const uint32_t *)A.rowinfo,
                  (const T *)d, z1, rows, (const DevState *)h->st);
        launch_ex_smem(pdl, k_dic_block<T, 4>, 1, TFS_DICB_TPB, bytes, s, A, val, d, b1, z1,
                       (const int *)h->d_lvl_begin, h->n_levels, groups, P.n_groups, L, TFS_DICB_SLOTS, h->st);
        return cudaPeekAtLastError();
    }
    k_dic_block<T, MODE><<<1, TFS_DICB_TPB, bytes, s>>>(A, val, d, b1, z1, h->d_lvl_begin, h->n_levels, groups,
                                                        P.n_groups, L, TFS_DICB_SLOTS, h->st);
    return cudaPeekAtLastError();
}

// DIC recurrence (Prec_Form.f90:32-40): one launch per large level, the tail
// in one block, or the one-block kernel.  Returns the number of kernels
// launched.
static int launch_dic_form(tfs_handle *h, cudaStream_t s)
{
    int bytes = 0;
    if (dic_block_kind<double>(h, &bytes) &&
        launch_dic_one_block<double, 2>(h, s, bytes, h->val, h->v.d, nullptr, nullptr) != cudaErrorMisalignedAddress)
        return 1;
    int cnt = 0;
    if (launch_levels<double, 1, 2>(h, s, h->val, h->v.d, nullptr, nullptr, nullptr, nullptr, nullptr,
                                    nullptr, &cnt))
        return cnt;
    return cnt;
}

static int tfs_mixed_prologue(tfs_handle *h, cudaStream_t s, int method, int prec, cudaGraphConditionalHandle cond);
static int dic_l0_rows(const tfs_handle *h, int method, int prec);
static int tfs_mixed_body(tfs_handle *h, cudaStream_t s, int method, int prec, cudaGraphConditionalHandle cond, int *count);
static void tfs_mixed_fill32(tfs_handle *h, const double *src, float *dst);
static void tfs_mixed_spmv_only(tfs_handle *h, cudaStream_t s);

static int launch_prologue(tfs_handle *h, cudaStream_t s, int method, int prec,
                           cudaGraphConditionalHandle cond, int *count)
{
    SellDev A = sell_of(h);
    const int G = h->grid, T = TFS_TPB;
    int gv = (h->nnz_pad + T - 1) / T;
    if (gv > h->sm_count * 16) gv = h->sm_count * 16;
    k_init<<<1, 1, 0, s>>>(h->st, h->params, prec);
    k_gather_val<<<gv, T, 0, s>>>(h->vmap, h->params, h->val,
                                  h->precision == TFS_MIXED ? h->val32 : nullptr, h->nnz_pad);
    k_load<<<G, T, 0, s>>>(A, h->val, h->perm, h->params, h->v, h->st, h->part, prec);
    *count = 3;
    if (prec == 2) *count += launch_dic_form(h, s);
    if (h->precision == TFS_MIXED) {
        tfs_mixed_prologue(h, s, method, prec, cond);
        *count += 2;
    } else {
        if (method == TFS_CG) k_residual<0><<<G, T, 0, s>>>(A, h->val, h->v, h->st, h->part, prec, cond,
                                                            dic_l0_rows(h, method, prec));
        else if (method == TFS_BICG) k_residual<1><<<G, T, 0, s>>>(A, h->val, h->v, h->st, h->part, prec, cond);
        else k_residual<2><<<G, T, 0, s>>>(A, h->val, h->v, h->st, h->part, prec, cond);
        *count += 1;
    }
    CKL("prologue launch");
    return TFS_OK;
}

// The tail of the per-level schedule: the prefetching tail (k_sweep_tail1)
// for one right-hand side on uniform-width matrices when it was set up, else
// the single-block level loop (k_sweep_tail2).
static bool pf_tail(const tfs_handle *h, int nr)
{
    return nr == 1 && h->tail_pf && h->pf_ok && h->sell_width > 0 && h->sell_width <= 8;
}

static int sweep_tail_at(const tfs_handle *h, int nr)
{
    return pf_tail(h, nr) ? h->pf_tail_level : h->tail_level;
}

template <typename T>
static int launch_sweeps(tfs_handle *h, cudaStream_t s, int nr, const T *b1, const T *b2,
                         T *y1, T *y2, T *z1, T *z2, int *count, bool fuse_l0 = false)
{
    SellDev A = sell_of(h);
    const int T_ = TFS_TPB;
    const T *val;
    T *d;
    if constexpr (sizeof(T) == 8) { val = (const T *)h->val; d = (T *)h->v.d; }
    else { val = (const T *)h->val32; d = (T *)h->f.d; }
    if (nr == 1 && !fuse_l0) {
        int bytes = 0;
        if (dic_block_kind<T>(h, &bytes)) {
            cudaError_t e = launch_dic_one_block<T, 0>(h, s, bytes, val, d, b1, z1);
            if (e == cudaSuccess) {
                h->dicb_used = 1;
                *count += dicb_split<T>(h->n_levels) ? 3 : 1;
                return TFS_OK;
            }
            if (e != cudaErrorMisalignedAddress) return tfs_engine_error(cudaGetLastError(), "one-block DIC launch");
        }
    }
    // Forward levels, both tails in one block, backward levels.
    h->dicb_used = 0;
    int rc;
    const int tail_at = sweep_tail_at(h, nr);
    const bool tails = tail_at < h->n_levels;
    auto tail2 = [&](auto kernel) -> int {
        if (!tails) return TFS_OK;
        cudaError_t e;
        int slot = 0;
        if (h->profiling) {
            h->stamp_kind.push_back(1 << 20);
            slot = h->stamp_next++;
        }
        if (pf_tail(h, nr))
            e = launch_ex(h->use_pdl != 0, k_sweep_tail1<T>, 1, TFS_SWEEP_TPB, s, A, val, (const T *)d, b1,
                          y1, z1, (const int *)h->d_lvl_begin, tail_at, h->n_levels, h->st, slot);
        else
            e = launch_ex(h->use_pdl != 0, kernel, 1, TFS_SWEEP_TPB, s, A, val, d, b1, b2, y1, y2, z1,
                          z2, (const int *)h->d_lvl_begin, tail_at, h->n_levels, h->st, slot);
        (*count)++;
        return e == cudaSuccess ? TFS_OK : tfs_engine_error(e, "tail launch");
    };
    if (nr == 1) {
        // fuse_l0 (CG): the forward sweep of level 0 is done by the update /
        // true-residual kernels, and the backward sweep of level 0 by
        // k_sweep0_rho together with rho.
        const int from = fuse_l0 ? 1 : 0;
        if ((rc = launch_levels<T, 1, 0>(h, s, val, d, b1, b2, y1, y2, nullptr, nullptr, count, false, tail_at, from,
                                         h->fwd_pre != 0))) return rc;
        if ((rc = tail2(k_sweep_tail2<T, 1>))) return rc;
        if ((rc = launch_levels<T, 1, 1>(h, s, val, d, nullptr, nullptr, z1, z2, y1, y2, count, false, tail_at, from,
                                         tails && h->bwd_pre))) return rc;
        if (fuse_l0) {
            const int l0 = h->lvl_begin[1];
            cudaError_t e = launch_ex(h->use_pdl != 0, k_sweep0_rho<T>, (l0 + T_ - 1) / T_, T_, s, A, val,
                                      (const T *)d, b1, z1, (const T *)y1, l0, h->n_int, h->st, h->part);
            (*count)++;
            if (e != cudaSuccess) return tfs_engine_error(e, "level-0 sweep launch");
        }
    } else {
        if ((rc = launch_levels<T, 2, 0>(h, s, val, d, b1, b2, y1, y2, nullptr, nullptr, count, false, tail_at))) return rc;
        if ((rc = tail2(k_sweep_tail2<T, 2>))) return rc;
        if ((rc = launch_levels<T, 2, 1>(h, s, val, d, nullptr, nullptr, z1, z2, y1, y2, count, false, tail_at, 0,
                                         tails && h->bwd_pre))) return rc;
    }
    return TFS_OK;
}

// ------------------------------------------------ mixed-precision graphs

// Rows of DIC level 0 whose forward sweep the CG kernels take over
// (k_mx_true, k_mx_cg_update4, k_residual, k_cg_update: y = r D) and whose
// backward sweep runs with rho in k_sweep0_rho, or 0 when the plain level
// schedule runs.  Level 0 must be one of the per-level kernels (not part of
// a tail).  fuse_l0 = 2 (default) fuses both arithmetics, 1 the binary32
// iteration only (the binary64 fused body first measured slower, 5.98
// against 6.11 solves/s; since its level-0 rows compute their start values
// before the dependency wait it is faster, 7.01 against 6.97).
static int dic_l0_rows(const tfs_handle *h, int method, int prec)
{
    if (method != TFS_CG || prec != 2 || !h->fuse_l0) return 0;
    if (h->precision == TFS_MIXED ? dic_block_kind<float>(h) : dic_block_kind<double>(h)) return 0;
    if (h->precision == TFS_MIXED && !h->vec4) return 0;
    if (h->precision != TFS_MIXED && h->fuse_l0 != 2) return 0;
    const int tail_at = sweep_tail_at(h, 1);
    if (tail_at < 1 || h->lvl_begin.size() < 2) return 0;
    return h->lvl_begin[1];
}

// After the binary64 preconditioner is formed: d32 = (float) d, then the
// binary64 initial residual (k_mx_true<INIT>).
static int tfs_mixed_prologue(tfs_handle *h, cudaStream_t s, int method, int prec,
                              cudaGraphConditionalHandle cond)
{
    SellDev A = sell_of(h);
    const int G = h->grid, T = TFS_TPB;
    k_mx_cast<<<G, T, 0, s>>>(h->n_int, h->v.d, h->f.d);
    if (method == TFS_CG) k_mx_true<0, true><<<G, T, 0, s>>>(A, h->val, h->v, h->f, h->st, h->part, prec, cond,
                                                             dic_l0_rows(h, method, prec));
    else if (method == TFS_BICG) k_mx_true<1, true><<<G, T, 0, s>>>(A, h->val, h->v, h->f, h->st, h->part, prec, cond);
    else k_mx_true<2, true><<<G, T, 0, s>>>(A, h->val, h->v, h->f, h->st, h->part, prec, cond);
    CKL("mixed prologue");
    return TFS_OK;
}

static int tfs_mixed_body(tfs_handle *h, cudaStream_t s, int method, int prec,
                          cudaGraphConditionalHandle cond, int *count)
{
    SellDev A = sell_of(h);
    const int G = h->grid, GS = h->grid_spmv, T = TFS_TPB, nc = h->n_chunks;
    Vec64 &V = h->v;
    Vec32 &F = h->f;
    const float *v32 = h->val32;
    int rc;
    *count = 0;
    if (method == TFS_CG) {
        const int n4 = h->n_int / 4, G4 = h->grid_vec4;
        if (!h->vec4 && prec == 2) {
            if ((rc = launch_sweeps<float>(h, s, 1, F.r, nullptr, F.y, nullptr, F.z, nullptr, count))) return rc;
            k_mx_dot_rho<0><<<G, T, 0, s>>>(nc, F, h->st, h->part);
            k_mx_cg_p<true><<<G, T, 0, s>>>(nc, F, h->st);
            launch_spmv_pq(h, s, true);
            k_mx_cg_update<false><<<G, T, 0, s>>>(nc, V, F, h->st, h->part);
            k_mx_fold<<<G, T, 0, s>>>(nc, V, F, h->st);
            k_mx_true<0, false><<<G, T, 0, s>>>(A, h->val, V, F, h->st, h->part, prec, cond);
            *count += 6;
        } else if (!h->vec4) {
            k_mx_cg_p<true><<<G, T, 0, s>>>(nc, F, h->st);
            launch_spmv_pq(h, s, true);
            k_mx_cg_update<true><<<G, T, 0, s>>>(nc, V, F, h->st, h->part);
            k_mx_fold<<<G, T, 0, s>>>(nc, V, F, h->st);
            k_mx_true<0, false><<<G, T, 0, s>>>(A, h->val, V, F, h->st, h->part, prec, cond);
            *count += 5;
        } else if (prec == 2 && dic_l0_rows(h, method, prec) > 0) {
            const int l0 = dic_l0_rows(h, method, prec);
            // The vector kernels after the sweeps are PDL-chained as well
            // (each waits for its predecessor before it reads anything).
            const bool pv = h->use_pdl && h->pdl_vec;
            if ((rc = launch_sweeps<float>(h, s, 1, F.r, nullptr, F.y, nullptr, F.z, nullptr, count, true))) return rc;
            launch_ex(pv, k_mx_cg_p4, G4, T, s, n4, F, (const DevState *)h->st);
            launch_spmv_pq(h, s, true, pv);
            launch_ex(pv, k_mx_cg_update4<false>, G4, T, s, n4, F, h->st, h->part, l0 / 4);
            launch_ex(pv, k_mx_fold4, G4, T, s, n4, V, F, (const DevState *)h->st);
            launch_ex(pv, k_mx_true<0, false>, G, T, s, A, (const double *)h->val, V, F, h->st, h->part, prec, cond, l0);
            *count += 5;
        } else if (prec == 2) {
            // (the one-block DIC, or levels that cannot take level 0 into the
            // CG kernels) the vector kernels PDL-chained
            const bool pv = h->use_pdl && h->pdl_vec;
            if ((rc = launch_sweeps<float>(h, s, 1, F.r, nullptr, F.y, nullptr, F.z, nullptr, count))) return rc;
            launch_ex(pv, k_mx_dot_rho4, G4, T, s, n4, F, h->st, h->part);
            launch_ex(pv, k_mx_cg_p4, G4, T, s, n4, F, (const DevState *)h->st);
            launch_spmv_pq(h, s, true, pv);
            launch_ex(pv, k_mx_cg_update4<false>, G4, T, s, n4, F, h->st, h->part, 0);
            launch_ex(pv, k_mx_fold4, G4, T, s, n4, V, F, (const DevState *)h->st);
            launch_ex(pv, k_mx_true<0, false>, G, T, s, A, (const double *)h->val, V, F, h->st, h->part, prec, cond, 0);
            *count += 6;
        } else {
            // Diagonal (or no) preconditioner: the whole body PDL-chained.
            const bool pv = h->use_pdl && h->pdl_vec;
            launch_ex(pv, k_mx_cg_p4, G4, T, s, n4, F, (const DevState *)h->st);
            launch_spmv_pq(h, s, true, pv);
            launch_ex(pv, k_mx_cg_update4<true>, G4, T, s, n4, F, h->st, h->part, 0);
            launch_ex(pv, k_mx_fold4, G4, T, s, n4, V, F, (const DevState *)h->st);
            launch_ex(pv, k_mx_true<0, false>, G, T, s, A, (const double *)h->val, V, F, h->st, h->part, prec, cond, 0);
            *count += 5;
        }
    } else if (method == TFS_BICG) {
        if (prec == 2) {
            if ((rc = launch_sweeps<float>(h, s, 2, F.r, F.r2, F.y, F.y2, F.z, F.z2, count))) return rc;
            k_mx_dot_rho<1><<<G, T, 0, s>>>(nc, F, h->st, h->part);
            k_mx_bicg_p<true><<<G, T, 0, s>>>(nc, F, h->st);
            k_mx_spmv2_pq<<<GS, T, 0, s>>>(A, v32, F, h->st, h->part);
            k_mx_bicg_update<false><<<G, T, 0, s>>>(nc, V, F, h->st, h->part);
            k_mx_fold<<<G, T, 0, s>>>(nc, V, F, h->st);
            k_mx_true<1, false><<<G, T, 0, s>>>(A, h->val, V, F, h->st, h->part, prec, cond);
            *count += 6;
        } else {
            k_mx_bicg_p<true><<<G, T, 0, s>>>(nc, F, h->st);
            k_mx_spmv2_pq<<<GS, T, 0, s>>>(A, v32, F, h->st, h->part);
            k_mx_bicg_update<true><<<G, T, 0, s>>>(nc, V, F, h->st, h->part);
            k_mx_fold<<<G, T, 0, s>>>(nc, V, F, h->st);
            k_mx_true<1, false><<<G, T, 0, s>>>(A, h->val, V, F, h->st, h->part, prec, cond);
            *count += 5;
        }
    } else {
        if (prec == 2) {
            k_mx_cgs_u<false><<<G, T, 0, s>>>(nc, F, h->st);
            if ((rc = launch_sweeps<float>(h, s, 1, F.u2, nullptr, F.y, nullptr, F.p2, nullptr, count))) return rc;
            k_mx_spmv_v<<<GS, T, 0, s>>>(A, v32, F, h->st, h->part);
            k_mx_cgs_q<false><<<G, T, 0, s>>>(nc, F, h->st);
            if ((rc = launch_sweeps<float>(h, s, 1, F.w, nullptr, F.y, nullptr, F.p, nullptr, count))) return rc;
            k_mx_cgs_spmv_r<<<GS, T, 0, s>>>(A, v32, V, F, h->st, h->part);
            k_mx_fold<<<G, T, 0, s>>>(nc, V, F, h->st);
            k_mx_true<2, false><<<G, T, 0, s>>>(A, h->val, V, F, h->st, h->part, prec, cond);
            *count += 6;
        } else {
            k_mx_cgs_u<true><<<G, T, 0, s>>>(nc, F, h->st);
            k_mx_spmv_v<<<GS, T, 0, s>>>(A, v32, F, h->st, h->part);
            k_mx_cgs_q<true><<<G, T, 0, s>>>(nc, F, h->st);
            k_mx_cgs_spmv_r<<<GS, T, 0, s>>>(A, v32, V, F, h->st, h->part);
            k_mx_fold<<<G, T, 0, s>>>(nc, V, F, h->st);
            k_mx_true<2, false><<<G, T, 0, s>>>(A, h->val, V, F, h->st, h->part, prec, cond);
            *count += 6;
        }
    }
    CKL("mixed body launch");
    return TFS_OK;
}

static void tfs_mixed_fill32(tfs_handle *h, const double *src, float *dst)
{
    k_mx_cast<<<h->grid, TFS_TPB, 0, h->stream>>>(h->n_int, src, dst);
}

static void tfs_mixed_spmv_only(tfs_handle *h, cudaStream_t s)
{
    launch_spmv_pq(h, s, true);
}

static int launch_body(tfs_handle *h, cudaStream_t s, int method, int prec,
                       cudaGraphConditionalHandle cond, int *count)
{
    SellDev A = sell_of(h);
    const int G = h->grid, GS = h->grid_spmv, T = TFS_TPB, nc = h->n_chunks;
    Vec64 &V = h->v;
    int rc;
    *count = 0;
    if (method == TFS_CG) {
        if (prec == 2 && dic_l0_rows(h, method, prec) > 0) {
            const int l0 = dic_l0_rows(h, method, prec);
            const bool pv = h->use_pdl && h->pdl_vec;   // vector kernels PDL-chained
            if ((rc = launch_sweeps<double>(h, s, 1, V.r, nullptr, V.y, nullptr, V.z, nullptr, count, true))) return rc;
            launch_ex(pv, k_cg_p<true>, G, T, s, nc, V, (const DevState *)h->st);
            launch_spmv_pq(h, s, false, pv);
            launch_ex(pv, k_cg_update<false>, G, T, s, nc, V, h->st, h->part, cond, l0);
            *count += 3;
        } else if (prec == 2) {
            const bool pv = h->use_pdl && h->pdl_vec;
            if ((rc = launch_sweeps<double>(h, s, 1, V.r, nullptr, V.y, nullptr, V.z, nullptr, count))) return rc;
            launch_ex(pv, k_dot_rho<0>, G, T, s, nc, V, h->st, h->part);
            launch_ex(pv, k_cg_p<true>, G, T, s, nc, V, (const DevState *)h->st);
            launch_spmv_pq(h, s, false, pv);
            launch_ex(pv, k_cg_update<false>, G, T, s, nc, V, h->st, h->part, cond, 0);
            *count += 4;
        } else {
            const bool pv = h->use_pdl && h->pdl_vec;
            launch_ex(pv, k_cg_p<true>, G, T, s, nc, V, (const DevState *)h->st);
            launch_spmv_pq(h, s, false, pv);
            launch_ex(pv, k_cg_update<true>, G, T, s, nc, V, h->st, h->part, cond, 0);
            *count += 3;
        }
    } else if (method == TFS_BICG) {
        if (prec == 2) {
            if ((rc = launch_sweeps<double>(h, s, 2, V.r, V.r2, V.y, V.y2, V.z, V.z2, count))) return rc;
            k_dot_rho<1><<<G, T, 0, s>>>(nc, V, h->st, h->part);
            k_bicg_p<true><<<G, T, 0, s>>>(nc, V, h->st);
            k_spmv2_pq<<<GS, T, 0, s>>>(A, h->val, V, h->st, h->part);
            k_bicg_update<false><<<G, T, 0, s>>>(nc, V, h->st, h->part, cond);
            *count += 4;
        } else {
            k_bicg_p<true><<<G, T, 0, s>>>(nc, V, h->st);
            k_spmv2_pq<<<GS, T, 0, s>>>(A, h->val, V, h->st, h->part);
            k_bicg_update<true><<<G, T, 0, s>>>(nc, V, h->st, h->part, cond);
            *count += 3;
        }
    } else {
        if (prec == 2) {
            k_cgs_u<false><<<G, T, 0, s>>>(nc, V, h->st);
            if ((rc = launch_sweeps<double>(h, s, 1, V.u2, nullptr, V.y, nullptr, V.p2, nullptr, count))) return rc;
            k_spmv_v<<<GS, T, 0, s>>>(A, h->val, V, h->st, h->part);
            k_cgs_q<false><<<G, T, 0, s>>>(nc, V, h->st);
            if ((rc = launch_sweeps<double>(h, s, 1, V.w, nullptr, V.y, nullptr, V.p, nullptr, count))) return rc;
            k_cgs_spmv_r<<<GS, T, 0, s>>>(A, h->val, V, h->st, h->part, cond);
            *count += 4;
        } else {
            k_cgs_u<true><<<G, T, 0, s>>>(nc, V, h->st);
            k_spmv_v<<<GS, T, 0, s>>>(A, h->val, V, h->st, h->part);
            k_cgs_q<true><<<G, T, 0, s>>>(nc, V, h->st);
            k_cgs_spmv_r<<<GS, T, 0, s>>>(A, h->val, V, h->st, h->part, cond);
            *count += 4;
        }
    }
    CKL("body launch");
    return TFS_OK;
}

static int launch_epilogue(tfs_handle *h, int *count)
{
    int g = (h->n_int + 255) / 256;
    if (g > h->sm_count * 8) g = h->sm_count * 8;
    k_store<<<g, 256, 0, h->stream>>>(h->n_int, h->perm, h->v.x, h->v.r, h->params, h->st);
    *count = 1;
    CKL("epilogue launch");
    return TFS_OK;
}

// The L2 access window of TFS_OPT_L2_WINDOW: the column indices (read by
// the SpMV and both sweeps every iteration, 4 B per SELL slot, 59 MB at
// 128^3) marked persisting in L2, hit ratio 1 up to the persisting set-aside
// the device allows (cudaLimitPersistingL2CacheSize, a limit of this
// process's context); or none.  Measured on the 128^3 DIC-CG system (mixed /
// binary64 solves/s): none 14.23 / 6.91, column indices 14.93 / 6.98; the
// binary32 values instead 14.53 / 6.70 (binary64 values for binary64); the
// column indices and as many values as the set-aside holds (84.7 MB)
// 14.31 / 6.76; the column indices at hit ratio 0.5 or 0.75 14.32, 14.47.
static cudaAccessPolicyWindow l2_window_of(tfs_handle *h)
{
    cudaAccessPolicyWindow w = {};
    if (!h->l2_window || h->layout < 0 || !h->col) return w;
    int maxwin = 0, maxpers = 0;
    cudaDeviceGetAttribute(&maxwin, cudaDevAttrMaxAccessPolicyWindowSize, h->device);
    cudaDeviceGetAttribute(&maxpers, cudaDevAttrMaxPersistingL2CacheSize, h->device);
    if (maxwin <= 0 || maxpers <= 0) return w;
    w.base_ptr = h->col;
    w.num_bytes = std::min(sizeof(int) * (size_t)h->nnz_pad, (size_t)maxwin);
    w.hitRatio = std::min(1.0f, (float)maxpers / (float)w.num_bytes);
    w.hitProp = cudaAccessPropertyPersisting;
    w.missProp = cudaAccessPropertyStreaming;
    cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, std::min((size_t)maxpers, w.num_bytes));
    return w;
}

// The window on the handle's streams (eager launches) and on every kernel
// node of a captured graph (g, and its loop body).
static void l2_window_streams(tfs_handle *h, const cudaAccessPolicyWindow &w)
{
    cudaStreamAttrValue v = {};
    v.accessPolicyWindow = w;
    cudaStreamSetAttribute(h->stream, cudaStreamAttributeAccessPolicyWindow, &v);
    cudaStreamSetAttribute(h->stream2, cudaStreamAttributeAccessPolicyWindow, &v);
}

static void l2_window_nodes(cudaGraph_t g, const cudaAccessPolicyWindow &w)
{
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return;
    std::vector<cudaGraphNode_t> nodes(n);
    if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return;
    cudaKernelNodeAttrValue v = {};
    v.accessPolicyWindow = w;
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
            cudaGraphKernelNodeSetAttribute(nd, cudaKernelNodeAttributeAccessPolicyWindow, &v);
    }
}

static int build_graph(tfs_handle *h, int method, int prec, GraphEntry &ge)
{
    const cudaAccessPolicyWindow l2w = l2_window_of(h);
    l2_window_streams(h, l2w);
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle cond;
    cudaError_t e = cudaGraphConditionalHandleCreate(&cond, g, 1u, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return tfs_engine_error(e, "cudaGraphConditionalHandleCreate"); }
    int rc = TFS_OK;
    auto fail = [&](cudaError_t err, const char *what) {
        cudaGraph_t tmp;
        cudaStreamEndCapture(h->stream, &tmp);
        cudaStreamEndCapture(h->stream2, &tmp);
        cudaGetLastError();
        cudaGraphDestroy(g);
        return tfs_engine_error(err, what);
    };
    e = cudaStreamBeginCaptureToGraph(h->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fail(e, "begin capture");
    if ((rc = launch_prologue(h, h->stream, method, prec, cond, &ge.prologue_kernels))) { fail(cudaErrorUnknown, "prologue"); return rc; }
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    e = cudaStreamGetCaptureInfo(h->stream, &cs, nullptr, nullptr, &deps, nullptr, &ndeps);
    if (e != cudaSuccess) return fail(e, "cudaStreamGetCaptureInfo");
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t wnode;
    e = cudaGraphAddNode(&wnode, g, deps, nullptr, ndeps, &np);
    if (e != cudaSuccess) return fail(e, "cudaGraphAddNode(while)");
    cudaGraph_t body = np.conditional.phGraph_out[0];
    e = cudaStreamUpdateCaptureDependencies(h->stream, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return fail(e, "cudaStreamUpdateCaptureDependencies");
    // Body, captured on the second stream into the conditional node's graph.
    e = cudaStreamBeginCaptureToGraph(h->stream2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fail(e, "begin body capture");
    if (h->precision == TFS_MIXED) rc = tfs_mixed_body(h, h->stream2, method, prec, cond, &ge.body_kernels);
    else rc = launch_body(h, h->stream2, method, prec, cond, &ge.body_kernels);
    if (rc) { fail(cudaErrorUnknown, "body"); return rc; }
    cudaGraph_t btmp;
    e = cudaStreamEndCapture(h->stream2, &btmp);
    if (e != cudaSuccess) return fail(e, "end body capture");
    if ((rc = launch_epilogue(h, &ge.epilogue_kernels))) { fail(cudaErrorUnknown, "epilogue"); return rc; }
    cudaGraph_t gtmp;
    e = cudaStreamEndCapture(h->stream, &gtmp);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return tfs_engine_error(e, "end capture"); }
    if (l2w.num_bytes) {
        l2_window_nodes(g, l2w);
        l2_window_nodes(body, l2w);
    }
    e = cudaGraphInstantiate(&ge.exec, g, 0);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return tfs_engine_error(e, "cudaGraphInstantiate"); }
    ge.graph = g;
    return TFS_OK;
}

// The same kernels without a graph: the host drives the loop, reading the
// device's done flag after every TFS_EAGER_BATCH iterations (kernels of a
// finished solve return at once).  Selected by TFS_OPT_LAUNCH = 1, for
// kernel-level profiling and launch tracing, which cannot look inside graphs
// with conditional nodes.
#define TFS_EAGER_BATCH 8
static int run_eager(tfs_handle *h, int method, int prec, GraphEntry *ge)
{
    l2_window_streams(h, l2_window_of(h));
    cudaStream_t s = h->stream;
    int rc, cnt = 0;
    if ((rc = launch_prologue(h, s, method, prec, 0, &cnt))) return rc;
    ge->prologue_kernels = cnt;
    const int limit = (h->h_params->niter_max > 0 ? h->h_params->niter_max : 0) + 8;
    for (int it = 0; it < limit; it += TFS_EAGER_BATCH) {
        CK(cudaMemcpyAsync(h->h_state, h->st, sizeof(DevState), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (h->h_state->done) break;
        for (int b = 0; b < TFS_EAGER_BATCH; b++) {
            if (h->precision == TFS_MIXED) rc = tfs_mixed_body(h, s, method, prec, 0, &cnt);
            else rc = launch_body(h, s, method, prec, 0, &cnt);
            if (rc) return rc;
        }
        ge->body_kernels = cnt;
    }
    if ((rc = launch_epilogue(h, &cnt))) return rc;
    ge->epilogue_kernels = cnt;
    return TFS_OK;
}

static int get_graph(tfs_handle *h, int method, int prec, GraphEntry **out)
{
    if (h->eager) {
        static thread_local GraphEntry eager_entry;
        *out = &eager_entry;
        return TFS_OK;
    }
    int key = method | (prec << 4) | (h->precision << 8);
    auto it = h->graphs.find(key);
    if (it != h->graphs.end()) { *out = &it->second; return TFS_OK; }
    GraphEntry ge;
    int rc = build_graph(h, method, prec, ge);
    if (rc && h->use_pdl) {
        // A driver that cannot keep programmatic edges inside a conditional
        // body gets plain stream-ordered level launches instead.
        h->use_pdl = 0;
        rc = build_graph(h, method, prec, ge);
    }
    if (rc) return rc;
    h->graphs[key] = ge;
    *out = &h->graphs[key];
    return TFS_OK;
}

// --------------------------------------------------------------- solve

// Everything a solve puts on the handle's stream, without waiting: per-call
// parameters, host-to-device copies (host arrays), the graph, device-to-host
// copies and the state read-back, then h->ev_done.
int tfs_solve_launch(int method, tfs_handle *h, const double *val, double *x, double *r1,
                     int32_t prec, int32_t niter, double tol, bool device_ptrs,
                     const double *b_in, int x0_zero)
{
    if (!h || !val || !x || !r1) return TFS_ERR_ARG;
    if (method < TFS_CG || method > TFS_CGS || prec < 0 || prec > 2) return TFS_ERR_ARG;
    CK(cudaSetDevice(h->device));
    int rc = ensure_layout(h, prec);
    if (rc) return rc;
    // The reference's BiCG starts its shadow residual as r1 and drives it
    // with A, not A^T (Bicg.f90:91-93, 107-108, 136-144, 171-175): the shadow
    // sequence equals the primary one bit for bit, rho = (z1, r2) = (r1, z1)
    // and (p2, q1) = (p1, q1), so every iterate is exactly the CG iterate.
    // It therefore runs through the CG kernels (half the work, same bits);
    // TFS_OPT_BICG = 1 runs the two sequences explicitly.
    const int kmethod = (method == TFS_BICG && !h->bicg_literal) ? TFS_CG : method;
    GraphEntry *ge = nullptr;
    rc = get_graph(h, kmethod, prec, &ge);
    if (rc) return rc;
    h->last_graph = ge;
    cudaStream_t s = h->stream;
    DevParams &P = *h->h_params;
    P.tol = tol;
    P.niter_max = niter;
    P.x0_zero = x0_zero;
    P.val_csr = device_ptrs ? val : h->stage_val;
    P.b = device_ptrs ? (b_in ? b_in : r1) : h->stage_b;
    P.x = device_ptrs ? x : h->stage_x;
    P.r_out = device_ptrs ? r1 : h->stage_b;
    P.dicb_wait_ns = h->dicb_diag_ns;
    CK(cudaMemcpyAsync(h->params, h->h_params, sizeof(DevParams), cudaMemcpyHostToDevice, s));
    if (!device_ptrs) {
        CK(cudaMemcpyAsync(h->stage_val, val, sizeof(double) * (size_t)h->nnz, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(h->stage_b, r1, sizeof(double) * (size_t)h->n, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(h->stage_x, x, sizeof(double) * (size_t)h->n, cudaMemcpyHostToDevice, s));
    }
    CK(cudaEventRecord(h->ev0, s));
    if (h->eager) {
        if ((rc = run_eager(h, kmethod, prec, ge))) return rc;
    } else {
        CK(cudaGraphLaunch(ge->exec, s));
    }
    CK(cudaEventRecord(h->ev1, s));
    if (!device_ptrs) {
        CK(cudaMemcpyAsync(x, h->stage_x, sizeof(double) * (size_t)h->n, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(r1, h->stage_b, sizeof(double) * (size_t)h->n, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaMemcpyAsync(h->h_state, h->st, sizeof(DevState), cudaMemcpyDeviceToHost, s));
    if (!h->ev_done) CK(cudaEventCreateWithFlags(&h->ev_done, cudaEventDisableTiming));
    CK(cudaEventRecord(h->ev_done, s));
    return TFS_OK;
}

// Outputs of a launched solve once h->ev_done has completed.
int tfs_solve_collect(tfs_handle *h, int32_t *niter, double *ini_res, double *fin_res)
{
    const DevState &S = *h->h_state;
    if (S.early != 1) *ini_res = S.ini_res;
    *fin_res = S.fin_res;
    *niter = S.niter_out;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    tfs_stats &T = h->stats;
    T.iterations = S.loops;
    T.true_residuals = S.true_res;
    T.status = S.status;
    T.solve_ms = ms;
    T.spmv_ns_total = (double)S.spmv_ns;
    T.spmv_launches = (int64_t)S.spmv_n;
    T.sweep_ns_total = (double)S.sweep_ns;
    T.sweep_launches = (int64_t)S.sweep_n;
    const GraphEntry *ge = h->last_graph;
    T.kernel_launches = ge ? ge->prologue_kernels + (int64_t)S.loops * ge->body_kernels + ge->epilogue_kernels : 0;
    T.device_bytes = h->device_bytes;
    return S.status;
}

static int solve_impl(int method, tfs_handle *h, const double *val, double *x, double *r1,
                      int32_t prec, int32_t *niter, double tol, double *ini_res, double *fin_res,
                      bool device_ptrs)
{
    if (!h || !niter || !ini_res || !fin_res) return TFS_ERR_ARG;
    int rc = tfs_solve_launch(method, h, val, x, r1, prec, *niter, tol, device_ptrs);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->stream));
    return tfs_solve_collect(h, niter, ini_res, fin_res);
}

extern "C" int tfs_solve_device(int method, tfs_handle *h, const double *d_val, double *d_x,
                                double *d_r1, int32_t prec, int32_t *niter, double tol,
                                double *ini_res, double *fin_res)
{
    return solve_impl(method, h, d_val, d_x, d_r1, prec, niter, tol, ini_res, fin_res, true);
}

// Handles built on demand for tfs_solve(h = NULL) and the Fortran-shaped
// entry points, keyed by the topology arrays the caller passes.
namespace {
std::mutex g_cache_mu;
std::map<std::tuple<const int32_t *, const int32_t *, int32_t, int32_t, int>, tfs_handle *> g_cache;
int g_default_precision = TFS_FP64;
}

extern "C" int tfs_set_default_precision(int mode)
{
    if (mode != TFS_FP64 && mode != TFS_MIXED) return TFS_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_cache_mu);
    g_default_precision = mode;
    for (auto &kv : g_cache) kv.second->precision = mode;
    return TFS_OK;
}

static int cached_handle(int32_t n, int32_t nnz, const int32_t *row1, const int32_t *col1,
                         const int32_t *dia1, tfs_handle **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return tfs_engine_error(e, "cudaGetDevice");
    std::lock_guard<std::mutex> lk(g_cache_mu);
    auto key = std::make_tuple(row1, col1, n, nnz, dev);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
        if (it->second->fingerprint == fingerprint(n, nnz, row1, col1, dia1)) { *out = it->second; return TFS_OK; }
        free_handle(it->second);
        g_cache.erase(it);
    }
    tfs_handle *h = nullptr;
    int rc = tfs_topology_register(n, nnz, row1, col1, dia1, &h);
    if (rc) return rc;
    h->precision = g_default_precision;
    g_cache[key] = h;
    *out = h;
    return TFS_OK;
}

extern "C" int tfs_solve(int method, tfs_handle *h, int32_t n, int32_t nnz, const int32_t *row1,
                         const int32_t *col1, const int32_t *dia1, const double *val, double *x,
                         double *r1, int32_t prec, int32_t *niter, double tol, double *ini_res,
                         double *fin_res)
{
    if (!h) {
        int rc = cached_handle(n, nnz, row1, col1, dia1, &h);
        if (rc) return rc;
    } else if (h->n != n || h->nnz != nnz) {
        tfs_set_error_text("n/nnz differ from the registered topology");
        return TFS_ERR_TOPOLOGY;
    }
    return solve_impl(method, h, val, x, r1, prec, niter, tol, ini_res, fin_res, false);
}

extern "C" int tfs_cg(int32_t n, int32_t nnz, const int32_t *row1, const int32_t *col1,
                      const int32_t *dia1, const double *val, double *x, double *r1, int32_t prec,
                      int32_t *niter, double tol, double *ini_res, double *fin_res)
{
    return tfs_solve(TFS_CG, nullptr, n, nnz, row1, col1, dia1, val, x, r1, prec, niter, tol, ini_res, fin_res);
}
extern "C" int tfs_bicg(int32_t n, int32_t nnz, const int32_t *row1, const int32_t *col1,
                        const int32_t *dia1, const double *val, double *x, double *r1, int32_t prec,
                        int32_t *niter, double tol, double *ini_res, double *fin_res)
{
    return tfs_solve(TFS_BICG, nullptr, n, nnz, row1, col1, dia1, val, x, r1, prec, niter, tol, ini_res, fin_res);
}
extern "C" int tfs_cgs(int32_t n, int32_t nnz, const int32_t *row1, const int32_t *col1,
                       const int32_t *dia1, const double *val, double *x, double *r1, int32_t prec,
                       int32_t *niter, double tol, double *ini_res, double *fin_res)
{
    return tfs_solve(TFS_CGS, nullptr, n, nnz, row1, col1, dia1, val, x, r1, prec, niter, tol, ini_res, fin_res);
}

// ------------------------------------------------------ single routines

// Uploads val and runs the gather with a fresh DevState (tol 0, one iteration).
static int prepare_values(tfs_handle *h, const double *val, int prec = 0)
{
    int rc = ensure_layout(h, prec);
    if (rc) return rc;
    cudaStream_t s = h->stream;
    DevParams &P = *h->h_params;
    P.tol = 0.0;
    P.niter_max = 1;
    P.x0_zero = 0;
    P.val_csr = h->stage_val;
    P.b = h->stage_b;
    P.x = h->stage_x;
    P.r_out = h->stage_b;
    P.dicb_wait_ns = 0;
    CK(cudaMemcpyAsync(h->params, h->h_params, sizeof(DevParams), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->stage_val, val, sizeof(double) * (size_t)h->nnz, cudaMemcpyHostToDevice, s));
    int gv = (h->nnz_pad + 255) / 256;
    if (gv > h->sm_count * 16) gv = h->sm_count * 16;
    k_init<<<1, 1, 0, s>>>(h->st, h->params, 0);
    k_gather_val<<<gv, 256, 0, s>>>(h->vmap, h->params, h->val, h->val32, h->nnz_pad);
    CKL("gather");
    return TFS_OK;
}

static int vec_in(tfs_handle *h, const double *host, double *dst)
{
    CK(cudaMemcpyAsync(h->stage_x, host, sizeof(double) * (size_t)h->n, cudaMemcpyHostToDevice, h->stream));
    k_perm_in<<<(h->n_int + 255) / 256, 256, 0, h->stream>>>(h->n_int, h->perm, h->stage_x, dst);
    CKL("perm in");
    return TFS_OK;
}

static int vec_out(tfs_handle *h, const double *src, double *host)
{
    k_perm_out<<<(h->n_int + 255) / 256, 256, 0, h->stream>>>(h->n_int, h->perm, src, h->stage_x);
    CKL("perm out");
    CK(cudaMemcpyAsync(host, h->stage_x, sizeof(double) * (size_t)h->n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return TFS_OK;
}

static int form_prec(tfs_handle *h, int prec)
{
    SellDev A = sell_of(h);
    k_diag_form<<<(h->n_int + 255) / 256, 256, 0, h->stream>>>(A, h->val, h->v.d, prec == 1 ? 1 : 0);
    if (prec == 2) launch_dic_form(h, h->stream);
    CKL("prec form");
    return TFS_OK;
}

extern "C" int tfs_spmv(tfs_handle *h, const double *val, const double *p, double *q)
{
    if (!h || !val || !p || !q) return TFS_ERR_ARG;
    CK(cudaSetDevice(h->device));
    int rc;
    if ((rc = prepare_values(h, val)) || (rc = vec_in(h, p, h->v.p))) return rc;
    launch_spmv_pq(h, h->stream, false);
    CKL("spmv");
    return vec_out(h, h->v.q, q);
}

extern "C" int tfs_residual(tfs_handle *h, const double *val, const double *x, double *r1)
{
    if (!h || !val || !x || !r1) return TFS_ERR_ARG;
    CK(cudaSetDevice(h->device));
    int rc;
    if ((rc = prepare_values(h, val)) || (rc = vec_in(h, x, h->v.x)) || (rc = vec_in(h, r1, h->v.r))) return rc;
    k_diag_form<<<(h->n_int + 255) / 256, 256, 0, h->stream>>>(sell_of(h), h->val, h->v.d, 0);
    k_residual<0><<<h->grid, TFS_TPB, 0, h->stream>>>(sell_of(h), h->val, h->v, h->st, h->part, 0, 0);
    CKL("residual");
    return vec_out(h, h->v.r, r1);
}

extern "C" int tfs_prec_form(tfs_handle *h, const double *val, int32_t prec, double *d)
{
    if (!h || !val || !d || prec < 0 || prec > 2) return TFS_ERR_ARG;
    CK(cudaSetDevice(h->device));
    int rc;
    if ((rc = prepare_values(h, val, prec)) || (rc = form_prec(h, prec))) return rc;
    return vec_out(h, h->v.d, d);
}

extern "C" int tfs_prec_solve(tfs_handle *h, const double *val, int32_t prec, const double *b, double *x)
{
    if (!h || !val || !b || !x || prec < 0 || prec > 2) return TFS_ERR_ARG;
    CK(cudaSetDevice(h->device));
    int rc;
    if ((rc = prepare_values(h, val, prec)) || (rc = form_prec(h, prec)) || (rc = vec_in(h, b, h->v.r))) return rc;
    if (prec == 2) {
        int cnt = 0;
        if ((rc = launch_sweeps<double>(h, h->stream, 1, h->v.r, nullptr, h->v.y, nullptr, h->v.z, nullptr, &cnt))) return rc;
    } else {
        k_diag_apply<<<(h->n_int + 255) / 256, 256, 0, h->stream>>>(h->n_int, h->v.d, h->v.r, h->v.z);
        CKL("diag apply");
    }
    return vec_out(h, h->v.z, x);
}

extern "C" int tfs_get_stats(const tfs_handle *h, tfs_stats *out)
{
    if (!h || !out) return TFS_ERR_ARG;
    *out = h->stats;
    out->spmv_kernel = h->spmv_kind;
    out->sell_width = h->sell_width;
    out->dic_kernel = h->dicb_used;
    return TFS_OK;
}

extern "C" int tfs_get_levels(tfs_handle *h, int32_t *levels)
{
    if (!h || !levels) return TFS_ERR_ARG;
    CK(cudaSetDevice(h->device));
    int rc = ensure_layout(h, 2);
    if (rc) return rc;
    memcpy(levels, h->levels_nat.data(), sizeof(int32_t) * (size_t)h->n);
    return TFS_OK;
}

extern "C" int tfs_time_spmv(tfs_handle *h, const double *val, int mode, int reps, double *ms)
{
    if (!h || !val || !ms || reps < 1 || (mode != TFS_FP64 && mode != TFS_MIXED)) return TFS_ERR_ARG;
    CK(cudaSetDevice(h->device));
    int rc = prepare_values(h, val);
    if (rc) return rc;
    SellDev A = sell_of(h);
    cudaStream_t s = h->stream;
    // p = 1 on real rows so the products are finite.
    k_diag_form<<<(h->n_int + 255) / 256, 256, 0, s>>>(A, h->val, h->v.p, 0);
    tfs_mixed_fill32(h, h->v.p, h->f.p);
    auto launch = [&]() {
        if (mode == TFS_FP64) launch_spmv_pq(h, s, false);
        else tfs_mixed_spmv_only(h, s);
    };
    for (int w = 0; w < 3; w++) launch();
    CKL("spmv warm-up");
    CK(cudaEventRecord(h->ev0, s));
    for (int r = 0; r < reps; r++) launch();
    CK(cudaEventRecord(h->ev1, s));
    CK(cudaEventSynchronize(h->ev1));
    CKL("spmv timing");
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, h->ev0, h->ev1));
    *ms = (double)t / reps;
    return TFS_OK;
}

// DIC preconditioner application (forward sweep, diagonal scaling, backward
// sweep: Prec_Solve.f90:46-67) timed alone: the factor is formed from val
// once, then `reps` applications to r = 1 are launched back to back.
extern "C" int tfs_time_prec(tfs_handle *h, const double *val, int mode, int reps, double *ms)
{
    if (!h || !val || !ms || reps < 1 || (mode != TFS_FP64 && mode != TFS_MIXED)) return TFS_ERR_ARG;
    CK(cudaSetDevice(h->device));
    int rc = prepare_values(h, val, 2);
    if (rc) return rc;
    if ((rc = form_prec(h, 2))) return rc;
    SellDev A = sell_of(h);
    cudaStream_t s = h->stream;
    k_diag_form<<<(h->n_int + 255) / 256, 256, 0, s>>>(A, h->val, h->v.r, 0);
    tfs_mixed_fill32(h, h->v.r, h->f.r);
    tfs_mixed_fill32(h, h->v.d, h->f.d);
    int count = 0;
    auto launch = [&]() -> int {
        if (mode == TFS_FP64)
            return launch_sweeps<double>(h, s, 1, h->v.r, nullptr, h->v.y, nullptr, h->v.z, nullptr, &count);
        return launch_sweeps<float>(h, s, 1, h->f.r, nullptr, h->f.y, nullptr, h->f.z, nullptr, &count);
    };
    for (int w = 0; w < 3; w++)
        if ((rc = launch())) return rc;
    CKL("prec warm-up");
    CK(cudaEventRecord(h->ev0, s));
    for (int r = 0; r < reps; r++)
        if ((rc = launch())) return rc;
    CK(cudaEventRecord(h->ev1, s));
    CK(cudaEventSynchronize(h->ev1));
    CKL("prec timing");
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, h->ev0, h->ev1));
    *ms = (double)t / reps;
    return TFS_OK;
}

// One DIC application with every sweep launch stamped: for each launch
// ("slot", in launch order) the global timer after its blocks' dependency
// waits (earliest) and at their ends (latest), relative to the first stamp.
// The kernels and the schedule are those of tfs_time_prec; the stamps add
// one load of the state and, per block, one barrier and two stores.
extern "C" int tfs_profile_prec(tfs_handle *h, const double *val, int mode, int max_slots, double *start_us,
                                double *end_us, int32_t *kind, int32_t *n_slots)
{
    if (!h || !val || !start_us || !end_us || !kind || !n_slots || max_slots < 1 ||
        (mode != TFS_FP64 && mode != TFS_MIXED))
        return TFS_ERR_ARG;
    double ms = 0.0;
    int rc = tfs_time_prec(h, val, mode, 3, &ms);   // factor formed, warm
    if (rc) return rc;
    if (h->dicb_used) {
        tfs_set_error_text("tfs_profile_prec: the one-block DIC has no level launches to stamp");
        return TFS_ERR_ARG;
    }
    cudaStream_t s = h->stream;
    int max_blocks = 1;
    for (int l = 0; l < h->n_levels; l++)
        max_blocks = std::max(max_blocks, (h->lvl_begin[l + 1] - h->lvl_begin[l] + h->level_tpb - 1) / h->level_tpb);
    const int stride = 2 * max_blocks, slots = 2 * h->n_levels + 2;
    unsigned long long *d_stamps = nullptr;
    CK(cudaMalloc(&d_stamps, sizeof(unsigned long long) * (size_t)stride * slots));
    CK(cudaMemsetAsync(d_stamps, 0, sizeof(unsigned long long) * (size_t)stride * slots, s));
    CK(cudaMemcpyAsync(&h->st->stamps, &d_stamps, sizeof d_stamps, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(&h->st->stamp_stride, &stride, sizeof stride, cudaMemcpyHostToDevice, s));
    h->profiling = true;
    h->stamp_next = 0;
    h->stamp_kind.clear();
    int count = 0;
    if (mode == TFS_FP64)
        rc = launch_sweeps<double>(h, s, 1, h->v.r, nullptr, h->v.y, nullptr, h->v.z, nullptr, &count);
    else
        rc = launch_sweeps<float>(h, s, 1, h->f.r, nullptr, h->f.y, nullptr, h->f.z, nullptr, &count);
    h->profiling = false;
    std::vector<unsigned long long> host((size_t)stride * slots);
    const unsigned long long *null_ptr = nullptr;
    cudaError_t e = cudaMemcpyAsync(host.data(), d_stamps, sizeof(unsigned long long) * host.size(),
                                    cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h->st->stamps, &null_ptr, sizeof null_ptr, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_stamps);
    if (rc) return rc;
    if (e != cudaSuccess) return tfs_engine_error(e, "tfs_profile_prec");
    const int n = std::min(h->stamp_next, max_slots);
    unsigned long long t_ref = ~0ull;
    std::vector<unsigned long long> lo(n, ~0ull), hi(n, 0ull);
    for (int k = 0; k < n; k++)
        for (int b = 0; b < max_blocks; b++) {
            const unsigned long long a = host[(size_t)k * stride + 2 * b], z = host[(size_t)k * stride + 2 * b + 1];
            if (!a) continue;
            lo[k] = std::min(lo[k], a);
            hi[k] = std::max(hi[k], z);
        }
    for (int k = 0; k < n; k++) t_ref = std::min(t_ref, lo[k]);
    for (int k = 0; k < n; k++) {
        start_us[k] = lo[k] == ~0ull ? -1.0 : (double)(lo[k] - t_ref) * 1e-3;
        end_us[k] = hi[k] == 0ull ? -1.0 : (double)(hi[k] - t_ref) * 1e-3;
        kind[k] = h->stamp_kind[k];
    }
    *n_slots = n;
    return TFS_OK;
}

// Autotuner of the single-solve launch shapes: every candidate is timed on
// the handle's own system with the same timers as tfs_time_spmv /
// tfs_time_prec, the fastest is kept, and the cached graphs (which hold the
// launch shapes) are dropped.
extern "C" int tfs_autotune(tfs_handle *h, const double *val, int mode, int prec, int reps,
                            tfs_tuning *out)
{
    if (!h || !val || !out || reps < 1 || (mode != TFS_FP64 && mode != TFS_MIXED) || prec < 0 || prec > 2)
        return TFS_ERR_ARG;
    memset(out, 0, sizeof(*out));
    int rc;
    if (prec == 2) {
        static const int cand[4] = {128, 256, 512, 1024};
        const int keep = h->level_tpb;
        int best = keep;
        double best_ms = 0.0;
        for (int k = 0; k < 4; k++) {
            h->level_tpb = cand[k];
            double ms = 0.0;
            if ((rc = tfs_time_prec(h, val, mode, reps, &ms))) { h->level_tpb = keep; return rc; }
            out->prec_ms[k] = ms;
            if (k == 0 || ms < best_ms) { best_ms = ms; best = cand[k]; }
        }
        h->level_tpb = best;
    } else if ((rc = ensure_layout(h, prec))) {
        return rc;
    }
    {
        // SpMV kernel x grid: the direct kernel and the software-pipelined
        // one (uniform-width matrices), each with 8 blocks per SM
        // (grid-stride) or one block per chunk.
        const int keep_grid = h->grid_spmv, keep_kind = h->spmv_kind;
        const int grids[2] = {h->grid, h->n_chunks};
        int kinds[2], nk = 0;
        kinds[nk++] = TFS_SPMV_DIRECT;
        if (h->sell_width > 0 && h->sell_width <= 8) kinds[nk++] = TFS_SPMV_PIPE;
        int best_grid = keep_grid, best_kind = keep_kind;
        double best_ms = 0.0;
        for (int a = 0; a < nk; a++)
            for (int k = 0; k < 2; k++) {
                h->spmv_kind = kinds[a];
                h->grid_spmv = grids[k];
                double ms = 0.0;
                if ((rc = tfs_time_spmv(h, val, mode, reps, &ms))) {
                    h->grid_spmv = keep_grid;
                    h->spmv_kind = keep_kind;
                    return rc;
                }
                if (kinds[a] == TFS_SPMV_DIRECT) out->spmv_ms[k] = ms;
                if (kinds[a] == TFS_SPMV_PIPE) out->spmv_pipe_ms[k] = ms;
                if ((a == 0 && k == 0) || ms < best_ms) {
                    best_ms = ms;
                    best_grid = grids[k];
                    best_kind = kinds[a];
                }
            }
        h->grid_spmv = best_grid;
        h->spmv_kind = best_kind;
    }
    // The part buffer holds TFS_NPART partials per chunk: both grids fit.
    drop_graphs(h);
    h->spmv_chunks = h->grid_spmv == h->n_chunks && h->grid_spmv != h->grid ? 1 : 0;
    if (h->sell_width > 0 && h->sell_width <= 8) h->spmv_pref = h->spmv_kind == TFS_SPMV_PIPE ? 1 : 0;
    out->level_tpb = h->level_tpb;
    out->spmv_chunks = h->grid_spmv == h->n_chunks && h->grid_spmv != h->grid ? 1 : 0;
    out->spmv_kernel = h->spmv_kind;
    return TFS_OK;
}

// ------------------------------------------------------ device helpers

extern "C" int tfs_use_device(int device)
{
    CK(cudaSetDevice(device));
    return TFS_OK;
}

extern "C" int tfs_device_alloc(size_t bytes, void **ptr)
{
    if (!ptr) return TFS_ERR_ARG;
    CK(cudaMalloc(ptr, bytes ? bytes : 1));
    return TFS_OK;
}

extern "C" int tfs_device_free(void *ptr)
{
    CK(cudaFree(ptr));
    return TFS_OK;
}

extern "C" int tfs_memcpy(void *dst, const void *src, size_t bytes)
{
    if ((!dst || !src) && bytes) return TFS_ERR_ARG;
    CK(cudaMemcpy(dst, src, bytes, cudaMemcpyDefault));
    return TFS_OK;
}

extern "C" int tfs_host_alloc(size_t bytes, void **ptr)
{
    if (!ptr) return TFS_ERR_ARG;
    CK(cudaMallocHost(ptr, bytes ? bytes : 1));
    return TFS_OK;
}

extern "C" int tfs_host_free(void *ptr)
{
    CK(cudaFreeHost(ptr));
    return TFS_OK;
}

extern "C" int tfs_copy(tfs_handle *h, void *dst, const void *src, size_t bytes)
{
    if (!h || (!dst && bytes) || (!src && bytes)) return TFS_ERR_ARG;
    CK(cudaSetDevice(h->device));
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, h->stream));
    return TFS_OK;
}

extern "C" int tfs_sync(tfs_handle *h)
{
    if (!h) return TFS_ERR_ARG;
    CK(cudaStreamSynchronize(h->stream));
    return TFS_OK;
}

extern "C" int tfs_timer_start(tfs_handle *h)
{
    if (!h) return TFS_ERR_ARG;
    if (!h->tev0) {
        CK(cudaEventCreate(&h->tev0));
        CK(cudaEventCreate(&h->tev1));
    }
    CK(cudaEventRecord(h->tev0, h->stream));
    return TFS_OK;
}

extern "C" int tfs_timer_stop(tfs_handle *h, double *ms)
{
    if (!h || !ms || !h->tev0) return TFS_ERR_ARG;
    CK(cudaEventRecord(h->tev1, h->stream));
    CK(cudaEventSynchronize(h->tev1));
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, h->tev0, h->tev1));
    *ms = (double)t;
    return TFS_OK;
}

// ------------------------------------------------------------ batches

#include "tfs_batch.cuh"

struct tfs_batch {
    int n = 0;
    int device = 0;
    int cluster = 8, tpb = 256;
    std::vector<tfs_handle *> hs;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    BatchSys *d_sys = nullptr, *h_sys = nullptr;
    BatchCtl *d_ctl = nullptr;
    int *d_order = nullptr;
    double last_ms = 0.0;
    int64_t launches = 0;
};

static void free_batch(tfs_batch *b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->d_sys) cudaFree(b->d_sys);
    if (b->d_ctl) cudaFree(b->d_ctl);
    if (b->d_order) cudaFree(b->d_order);
    if (b->h_sys) cudaFreeHost(b->h_sys);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

extern "C" int tfs_batch_create(int n_sys, tfs_handle *const *handles, tfs_batch **out)
{
    if (!out || n_sys < 1 || !handles) return TFS_ERR_ARG;
    *out = nullptr;
    for (int k = 0; k < n_sys; k++) {
        if (!handles[k]) return TFS_ERR_ARG;
        CK(cudaSetDevice(handles[k]->device));
        int rc = ensure_layout(handles[k], 1);
        if (rc) return rc;
    }
    tfs_batch *b = new tfs_batch;
    b->n = n_sys;
    b->hs.assign(handles, handles + n_sys);
    b->device = handles[0]->device;
#define CKB(call)                                                              \
    do {                                                                       \
        cudaError_t _e = (call);                                               \
        if (_e != cudaSuccess) { int _r = tfs_engine_error(_e, #call); free_batch(b); return _r; } \
    } while (0)
    CKB(cudaSetDevice(b->device));
    CKB(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    CKB(cudaEventCreate(&b->ev0));
    CKB(cudaEventCreate(&b->ev1));
    CKB(cudaMalloc(&b->d_sys, sizeof(BatchSys) * (size_t)n_sys));
    CKB(cudaMalloc(&b->d_ctl, sizeof(BatchCtl)));
    CKB(cudaMalloc(&b->d_order, sizeof(int) * (size_t)n_sys));
    CKB(cudaMallocHost(&b->h_sys, sizeof(BatchSys) * (size_t)n_sys));
    // Longest systems first.
    std::vector<int> order(n_sys);
    for (int k = 0; k < n_sys; k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        return handles[a]->nnz > handles[c]->nnz;
    });
    CKB(cudaMemcpy(b->d_order, order.data(), sizeof(int) * (size_t)n_sys, cudaMemcpyHostToDevice));
#undef CKB
    *out = b;
    return TFS_OK;
}

extern "C" int tfs_batch_release(tfs_batch *b)
{
    if (!b) return TFS_ERR_ARG;
    free_batch(b);
    return TFS_OK;
}

extern "C" int tfs_batch_configure(tfs_batch *b, int cluster_size, int threads_per_cta)
{
    if (!b || cluster_size < 1 || cluster_size > 16 || (cluster_size & (cluster_size - 1)) ||
        (threads_per_cta != 128 && threads_per_cta != 256 && threads_per_cta != TFS_BATCH_MAX_TPB))
        return TFS_ERR_ARG;
    b->cluster = cluster_size;
    b->tpb = threads_per_cta;
    return TFS_OK;
}

template <int METHOD, typename VT>
static int launch_batch_kernel(tfs_batch *b)
{
    auto kernel = k_batch<METHOD, VT>;
    if (b->cluster > 8) CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)b->cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3((unsigned)b->tpb);
    cfg.gridDim = dim3((unsigned)b->cluster);
    cfg.stream = b->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n_clusters = 0;
    CK(cudaOccupancyMaxActiveClusters(&n_clusters, kernel, &cfg));
    if (n_clusters < 1) {
        tfs_set_error_text("cluster configuration cannot be resident");
        return TFS_ERR_ARG;
    }
    if (n_clusters > b->n) n_clusters = b->n;
    cfg.gridDim = dim3((unsigned)(n_clusters * b->cluster));
    CK(cudaLaunchKernelEx(&cfg, kernel, b->d_sys, (const int *)b->d_order, b->n, b->d_ctl));
    return TFS_OK;
}

extern "C" int tfs_batch_solve_device(tfs_batch *b, int method, int prec, int mode,
                                      const double *const *d_val, double *const *d_x,
                                      double *const *d_r1, const int32_t *niter, const double *tol,
                                      int32_t *niter_out, double *ini_res, double *fin_res,
                                      int32_t *status)
{
    if (!b || !d_val || !d_x || !d_r1 || !niter || !tol || !niter_out || !ini_res || !fin_res || !status)
        return TFS_ERR_ARG;
    if ((method != TFS_CG && method != TFS_BICG) || prec < 0 || prec > 2 ||
        (mode != TFS_FP64 && mode != TFS_MIXED)) {
        tfs_set_error_text("batches run CG or BiCG with no, diagonal or DIC preconditioning");
        return TFS_ERR_ARG;
    }
    // BiCG iterates equal CG's (see tfs_solve_launch): one sequence suffices
    // unless the first system's handle asks for the literal two sequences,
    // which the batch runs with no or diagonal preconditioning only.
    if (method == TFS_BICG && !b->hs[0]->bicg_literal) method = TFS_CG;
    if (method == TFS_BICG && prec == 2) {
        tfs_set_error_text("the batch runs DIC with the CG sequence only (TFS_OPT_BICG = 0)");
        return TFS_ERR_ARG;
    }
    CK(cudaSetDevice(b->device));
    if (prec == 2)
        for (int k = 0; k < b->n; k++) {
            int rc = ensure_layout(b->hs[k], 2);   // the DIC level schedule
            if (rc) return rc;
        }
    int64_t max_nnz = 0;
    for (int k = 0; k < b->n; k++) {
        tfs_handle *h = b->hs[k];
        BatchSys &S = b->h_sys[k];
        memset(&S, 0, sizeof S);
        S.A = sell_of(h);
        S.val = h->val;
        S.val32 = h->val32;
        S.vmap = h->vmap;
        S.nnz_pad = h->nnz_pad;
        S.perm = h->perm;
        S.V = h->v;
        S.F = h->f;
        S.val_csr = d_val[k];
        S.b = d_r1[k];
        S.x = d_x[k];
        S.r_out = d_r1[k];
        S.tol = tol[k];
        S.niter_max = niter[k];
        S.prec = prec;
        S.lvl_begin = h->d_lvl_begin;
        S.n_levels = prec == 2 ? h->n_levels : 0;
        if (h->nnz_pad > max_nnz) max_nnz = h->nnz_pad;
    }
    CK(cudaMemcpyAsync(b->d_sys, b->h_sys, sizeof(BatchSys) * (size_t)b->n, cudaMemcpyHostToDevice, b->stream));
    CK(cudaEventRecord(b->ev0, b->stream));
    int gx = (int)((max_nnz + 255) / 256);
    if (gx > 64) gx = 64;
    if (gx < 1) gx = 1;
    k_batch_gather<<<dim3((unsigned)gx, (unsigned)b->n), 256, 0, b->stream>>>(b->d_sys, b->d_ctl, mode == TFS_MIXED);
    CKL("batch gather");
    int rc;
    if (method == TFS_CG && prec == 2)
        rc = mode == TFS_MIXED ? launch_batch_kernel<2, float>(b) : launch_batch_kernel<2, double>(b);
    else if (method == TFS_CG)
        rc = mode == TFS_MIXED ? launch_batch_kernel<0, float>(b) : launch_batch_kernel<0, double>(b);
    else rc = mode == TFS_MIXED ? launch_batch_kernel<1, float>(b) : launch_batch_kernel<1, double>(b);
    if (rc) return rc;
    CK(cudaEventRecord(b->ev1, b->stream));
    CK(cudaMemcpyAsync(b->h_sys, b->d_sys, sizeof(BatchSys) * (size_t)b->n, cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    b->last_ms = ms;
    b->launches = 2;
    int worst = TFS_OK;
    for (int k = 0; k < b->n; k++) {
        const BatchSys &S = b->h_sys[k];
        niter_out[k] = S.niter_out;
        if (S.early != 1) ini_res[k] = S.ini_res;
        fin_res[k] = S.fin_res;
        status[k] = S.status;
        if (S.status != TFS_OK && worst == TFS_OK) worst = S.status;
    }
    return worst;
}

extern "C" int tfs_batch_solve(tfs_batch *b, int method, int prec, int mode,
                               const double *const *val, double *const *x, double *const *r1,
                               const int32_t *niter, const double *tol, int32_t *niter_out,
                               double *ini_res, double *fin_res, int32_t *status)
{
    if (!b || !val || !x || !r1) return TFS_ERR_ARG;
    CK(cudaSetDevice(b->device));
    std::vector<const double *> dv(b->n);
    std::vector<double *> dx(b->n), dr(b->n);
    for (int k = 0; k < b->n; k++) {
        tfs_handle *h = b->hs[k];
        CK(cudaMemcpyAsync(h->stage_val, val[k], sizeof(double) * (size_t)h->nnz, cudaMemcpyHostToDevice, b->stream));
        CK(cudaMemcpyAsync(h->stage_b, r1[k], sizeof(double) * (size_t)h->n, cudaMemcpyHostToDevice, b->stream));
        CK(cudaMemcpyAsync(h->stage_x, x[k], sizeof(double) * (size_t)h->n, cudaMemcpyHostToDevice, b->stream));
        dv[k] = h->stage_val;
        dx[k] = h->stage_x;
        dr[k] = h->stage_b;
    }
    int rc = tfs_batch_solve_device(b, method, prec, mode, dv.data(), dx.data(), dr.data(), niter, tol,
                                    niter_out, ini_res, fin_res, status);
    if (rc != TFS_OK && rc != TFS_ERR_NONFINITE) return rc;
    for (int k = 0; k < b->n; k++) {
        tfs_handle *h = b->hs[k];
        CK(cudaMemcpyAsync(x[k], h->stage_x, sizeof(double) * (size_t)h->n, cudaMemcpyDeviceToHost, b->stream));
        CK(cudaMemcpyAsync(r1[k], h->stage_b, sizeof(double) * (size_t)h->n, cudaMemcpyDeviceToHost, b->stream));
    }
    CK(cudaStreamSynchronize(b->stream));
    return rc;
}

extern "C" int tfs_batch_last_ms(const tfs_batch *b, double *ms)
{
    if (!b || !ms) return TFS_ERR_ARG;
    *ms = b->last_ms;
    return TFS_OK;
}

extern "C" int tfs_batch_copy(tfs_batch *b, int n, void *const *dst, const void *const *src,
                              const size_t *bytes)
{
    if (!b || n < 0 || (n > 0 && (!dst || !src || !bytes))) return TFS_ERR_ARG;
    CK(cudaSetDevice(b->device));
    for (int k = 0; k < n; k++)
        CK(cudaMemcpyAsync(dst[k], src[k], bytes[k], cudaMemcpyDefault, b->stream));
    return TFS_OK;
}
