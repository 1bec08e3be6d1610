// tfs_server.cu -- a request loop for solves that arrive over time.
//
// Serving the Krylov path: callers submit solves of different systems as they
// arrive; one worker thread admits them onto the GPU while others are still
// running (continuous batching at the stream level: every admitted solve is
// one graph launch on its system's own stream, so the work of concurrent
// solves overlaps on the device), keeps every system's matrix layout,
// preconditioner and Krylov vectors resident between requests, and admits
// systems against a device-memory budget, evicting idle ones (least recently
// used) when a new one does not fit -- an evicted system is rebuilt from the
// host copy of its topology on its next request.  A system runs one request
// at a time (a handle is not re-entrant); requests of one system are served
// in arrival order.  Results do not depend on what else is running: each
// solve has its own handle state and fixed-order reductions.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "tfs_internal.h"

namespace {

using clk = std::chrono::steady_clock;

double ms_since(clk::time_point a, clk::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Request {
    int64_t ticket = 0, sys = 0;
    int method = 0, prec = 0, mode = 0;
    const double *val = nullptr, *b = nullptr;
    double *x = nullptr, *r1 = nullptr;
    int x0_zero = 0;
    bool host = false;   // val, x, r1 in host memory (copied on the system's stream)
    int32_t niter = 0;
    double tol = 0.0;
    clk::time_point t_submit, t_start, t_done;
    int state = 0;   // 0 queued, 1 running, 2 done
    tfs_result res{};
};

struct System {
    int32_t n = 0, nnz = 0;
    std::vector<int32_t> row1, col1, dia1;
    tfs_handle *h = nullptr;
    int64_t bytes = 0;
    bool busy = false;
    clk::time_point last_used;
};

}  // namespace

struct tfs_server {
    int device = 0;
    int64_t budget = 0, resident = 0;
    int max_inflight = 8;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread worker;
    bool stop = false;
    std::deque<Request *> queue;
    std::vector<Request *> running;
    std::map<int64_t, Request *> tickets;
    std::map<int64_t, System> systems;
    int64_t next_sys = 1, next_ticket = 1;
    tfs_server_stats stats{};
};

int64_t tfs_estimate_bytes(int32_t n, int32_t nnz)
{
    // Layout: rows padded to 1024 (+ up to 31 per DIC level), perm/rowinfo
    // (8 B/row), iperm (4 B/row), col/vmap/val/val32 (20 B/entry, SELL
    // padding ~5%), 16 binary64 + 16 binary32 vectors (192 B/row), partials;
    // fixed: staging val/b/x (8 B/entry + 16 B/row) and state.
    const int64_t n_pad = ((int64_t)n + 1023) / 1024 * 1024 + 32 * 64;
    return n_pad * 200 + (int64_t)n * 20 + (int64_t)nnz * 29 + (64 << 10);
}

static void release_system(tfs_server *S, System &sy)
{
    if (!sy.h) return;
    tfs_release(sy.h);
    sy.h = nullptr;
    S->resident -= sy.bytes;
    sy.bytes = 0;
    S->stats.evictions++;
}

// Make room for `need` bytes by evicting idle systems, least recently used
// first.  Caller holds the lock.
static bool make_room(tfs_server *S, int64_t need, int64_t keep)
{
    while (S->resident + need > S->budget) {
        System *victim = nullptr;
        for (auto &kv : S->systems) {
            System &sy = kv.second;
            if (!sy.h || sy.busy || kv.first == keep) continue;
            if (!victim || sy.last_used < victim->last_used) victim = &sy;
        }
        if (!victim) return false;
        release_system(S, *victim);
    }
    return true;
}

// Admit and launch one queued request if its system is idle and resident
// (or can be made resident).  Caller holds the lock.  Returns true if the
// request left the queue (launched or failed).
static bool try_start(tfs_server *S, Request *r)
{
    auto it = S->systems.find(r->sys);
    if (it == S->systems.end()) {
        r->res.status = TFS_ERR_ARG;
        r->state = 2;
        r->t_done = clk::now();
        return true;
    }
    System &sy = it->second;
    if (sy.busy) return false;
    if (!sy.h) {
        int64_t need = tfs_estimate_bytes(sy.n, sy.nnz);
        if (need > S->budget) {
            r->res.status = TFS_ERR_BUDGET;
            r->state = 2;
            r->t_done = clk::now();
            S->stats.refused++;
            return true;
        }
        if (!make_room(S, need, r->sys)) return false;   // wait for a system to go idle
        int rc = tfs_topology_register(sy.n, sy.nnz, sy.row1.data(), sy.col1.data(), sy.dia1.data(), &sy.h);
        if (rc) {
            r->res.status = rc;
            r->state = 2;
            r->t_done = clk::now();
            return true;
        }
        // Solves share the GPU here: PDL-chained vector kernels would park
        // their blocks at the dependency wait while other requests' kernels
        // could use the slots (measured 232 against 252 solves/s on the
        // serving trace), so the server's handles launch them plainly.
        sy.h->pdl_vec = 0;
        // Nor do they mark their column indices persisting in L2: the
        // resident systems would compete for the one set-aside.
        sy.h->l2_window = 0;
        sy.bytes = need;
        S->resident += need;
        S->stats.registrations++;
    }
    tfs_set_precision(sy.h, r->mode);
    r->t_start = clk::now();
    int rc = tfs_solve_launch(r->method, sy.h, r->val, r->x, r->r1, r->prec, r->niter, r->tol, !r->host,
                              r->host ? nullptr : r->b, r->x0_zero);
    if (rc) {
        r->res.status = rc;
        r->state = 2;
        r->t_done = clk::now();
        return true;
    }
    // The layout now exists: account its real size.
    S->resident += sy.h->device_bytes - sy.bytes;
    sy.bytes = sy.h->device_bytes;
    sy.busy = true;
    sy.last_used = r->t_start;
    r->state = 1;
    S->running.push_back(r);
    if ((int64_t)S->running.size() > S->stats.peak_running) S->stats.peak_running = (int64_t)S->running.size();
    return true;
}

static void finish(tfs_server *S, Request *r, System &sy)
{
    int32_t it = r->niter;
    double ini = 0.0, fin = 0.0;
    r->res.status = tfs_solve_collect(sy.h, &it, &ini, &fin);
    r->res.niter = it;
    r->res.ini_res = ini;
    r->res.fin_res = fin;
    r->res.device_begin_ns = (int64_t)sy.h->h_state->t_begin;
    r->res.device_end_ns = (int64_t)sy.h->h_state->t_end;
    r->t_done = clk::now();
    r->state = 2;
    sy.busy = false;
    sy.last_used = r->t_done;
    S->stats.completed++;
}

static void worker_main(tfs_server *S)
{
    cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lk(S->mu);
    while (!S->stop) {
        bool progressed = false;
        // Completions.
        for (size_t k = 0; k < S->running.size();) {
            Request *r = S->running[k];
            System &sy = S->systems[r->sys];
            cudaError_t e = cudaEventQuery(sy.h->ev_done);
            if (e == cudaErrorNotReady) { k++; continue; }
            if (e != cudaSuccess) {
                tfs_engine_error(e, "server: solve");
                r->res.status = TFS_ERR_CUDA;
                r->state = 2;
                r->t_done = clk::now();
                sy.busy = false;
            } else {
                finish(S, r, sy);
            }
            S->running.erase(S->running.begin() + (long)k);
            progressed = true;
        }
        if (progressed) S->cv_done.notify_all();
        // Admissions, in arrival order; a request whose system is busy does
        // not block later requests of other systems.
        for (auto it = S->queue.begin(); it != S->queue.end() && (int)S->running.size() < S->max_inflight;) {
            Request *r = *it;
            bool same_sys_earlier = false;
            for (auto jt = S->queue.begin(); jt != it; ++jt)
                if ((*jt)->sys == r->sys) { same_sys_earlier = true; break; }
            if (!same_sys_earlier && try_start(S, r)) {
                if (r->state == 2) S->cv_done.notify_all();
                it = S->queue.erase(it);
                progressed = true;
            } else {
                ++it;
            }
        }
        if (!progressed) {
            if (S->running.empty() && S->queue.empty())
                S->cv_work.wait(lk, [&] { return S->stop || !S->queue.empty(); });
            else
                S->cv_work.wait_for(lk, std::chrono::microseconds(20));
        }
    }
}

extern "C" int tfs_server_create(int device, int64_t hbm_budget_bytes, int max_inflight,
                                 tfs_server **out)
{
    if (!out || hbm_budget_bytes <= 0 || max_inflight < 1) return TFS_ERR_ARG;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return tfs_engine_error(e, "cudaSetDevice");
    tfs_server *S = new tfs_server;
    S->device = device;
    S->budget = hbm_budget_bytes;
    S->max_inflight = max_inflight;
    S->worker = std::thread(worker_main, S);
    *out = S;
    return TFS_OK;
}

extern "C" int tfs_server_destroy(tfs_server *S)
{
    if (!S) return TFS_ERR_ARG;
    {
        std::unique_lock<std::mutex> lk(S->mu);
        // Let running solves finish before the handles go.
        S->cv_done.wait(lk, [&] { return S->running.empty(); });
        S->stop = true;
    }
    S->cv_work.notify_all();
    S->worker.join();
    cudaSetDevice(S->device);
    for (auto &kv : S->systems)
        if (kv.second.h) tfs_release(kv.second.h);
    for (auto &kv : S->tickets) delete kv.second;
    for (Request *r : S->queue)
        if (!S->tickets.count(r->ticket)) delete r;
    delete S;
    return TFS_OK;
}

extern "C" int tfs_server_add_system(tfs_server *S, int32_t n, int32_t nnz, const int32_t *row1,
                                     const int32_t *col1, const int32_t *dia1, int64_t *sys_id)
{
    if (!S || !sys_id || n <= 0 || nnz < n || !row1 || !col1 || !dia1) return TFS_ERR_ARG;
    System sy;
    sy.n = n;
    sy.nnz = nnz;
    sy.row1.assign(row1, row1 + n + 1);
    sy.col1.assign(col1, col1 + nnz);
    sy.dia1.assign(dia1, dia1 + n);
    std::lock_guard<std::mutex> lk(S->mu);
    *sys_id = S->next_sys++;
    sy.last_used = clk::now();
    S->systems.emplace(*sys_id, std::move(sy));
    return TFS_OK;
}

static int submit(tfs_server *S, int64_t sys_id, int method, int prec, int mode, const double *d_val,
                  const double *d_b, double *d_x, double *d_r1, int x0_zero, int32_t niter, double tol,
                  bool host, int64_t *ticket)
{
    if (!S || !ticket || !d_val || !d_x || !d_r1) return TFS_ERR_ARG;
    if (method < TFS_CG || method > TFS_CGS || prec < 0 || prec > 2 ||
        (mode != TFS_FP64 && mode != TFS_MIXED))
        return TFS_ERR_ARG;
    Request *r = new Request;
    r->sys = sys_id;
    r->method = method;
    r->prec = prec;
    r->mode = mode;
    r->val = d_val;
    r->b = d_b;
    r->x0_zero = x0_zero;
    r->x = d_x;
    r->r1 = d_r1;
    r->niter = niter;
    r->tol = tol;
    r->host = host;
    r->t_submit = clk::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        r->ticket = S->next_ticket++;
        r->res.ticket = r->ticket;
        S->tickets[r->ticket] = r;
        S->queue.push_back(r);
        S->stats.submitted++;
    }
    S->cv_work.notify_one();
    *ticket = r->ticket;
    return TFS_OK;
}

extern "C" int tfs_server_submit(tfs_server *S, int64_t sys_id, int method, int prec, int mode,
                                 const double *d_val, const double *d_b, double *d_x, double *d_r1,
                                 int x0_zero, int32_t niter, double tol, int64_t *ticket)
{
    return submit(S, sys_id, method, prec, mode, d_val, d_b, d_x, d_r1, x0_zero, niter, tol, false, ticket);
}

extern "C" int tfs_server_submit_host(tfs_server *S, int64_t sys_id, int method, int prec, int mode,
                                      const double *val, double *x, double *r1, int x0_zero, int32_t niter,
                                      double tol, int64_t *ticket)
{
    return submit(S, sys_id, method, prec, mode, val, nullptr, x, r1, x0_zero, niter, tol, true, ticket);
}

extern "C" int tfs_server_wait(tfs_server *S, int64_t ticket, double timeout_s, tfs_result *out)
{
    if (!S || !out) return TFS_ERR_ARG;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->tickets.find(ticket);
    if (it == S->tickets.end()) return TFS_ERR_ARG;
    Request *r = it->second;
    bool ok = S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s < 0 ? 0 : timeout_s),
                                  [&] { return r->state == 2; });
    if (!ok) return TFS_ERR_TIMEOUT;
    *out = r->res;
    out->queued_ms = r->t_start.time_since_epoch().count() ? ms_since(r->t_submit, r->t_start) : ms_since(r->t_submit, r->t_done);
    out->run_ms = r->t_start.time_since_epoch().count() ? ms_since(r->t_start, r->t_done) : 0.0;
    out->latency_ms = ms_since(r->t_submit, r->t_done);
    S->tickets.erase(it);
    delete r;
    return TFS_OK;
}

extern "C" int tfs_server_get_stats(tfs_server *S, tfs_server_stats *out)
{
    if (!S || !out) return TFS_ERR_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    *out = S->stats;
    out->resident_bytes = S->resident;
    int64_t res = 0;
    for (auto &kv : S->systems)
        if (kv.second.h) res++;
    out->resident_systems = res;
    out->running = (int64_t)S->running.size();
    out->queued = (int64_t)S->queue.size();
    return TFS_OK;
}
