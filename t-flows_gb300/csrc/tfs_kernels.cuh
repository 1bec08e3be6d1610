// tfs_kernels.cuh -- binary64 kernels of the preconditioned Krylov solves.
//
// Every kernel keeps the reference's per-row arithmetic: a row sum starts
// where the Fortran loop starts (0.0, b(i) or x(i)) and adds the products of
// the row one at a time in ascending column order; products and sums are
// rounded separately (the library is compiled with --fmad=false); divisions
// and square roots are the IEEE-rounded operators.  Only the order of the dot
// product sums differs from the sequential i = 1..N loops of the reference:
// they are fixed-shape tree reductions (warp shuffles, then one partial per
// block, then the last block to finish sums the partials in block order), so
// a solve is bitwise reproducible from run to run.
#pragma once
#include <cfloat>
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "tfs_internal.h"

namespace tfs {

constexpr unsigned FULL = 0xffffffffu;
constexpr double TINY = 1.e-30;   // Sources/Shared/allp_mod.f90:40

__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

struct RowGeom {
    int len, dpos, off;
};
__device__ __forceinline__ RowGeom row_geom(const SellDev &A, int i)
{
    uint32_t info = __ldg(A.rowinfo + i);
    RowGeom g;
    g.len = (int)(info & 0xffffu);
    g.dpos = (int)(info >> 16);
    g.off = (A.width ? (i & ~31) * A.width : __ldg(A.slice_off + (i >> 5))) + (i & 31);
    return g;
}

// Gathers of the SpMV-type kernels through L1 (ld.global.nc, NC = true) or
// past it (ld.global.cg).  NC is only legal where the gathered vector is not
// written during the launch: the stand-alone SpMV and residual kernels.  With
// rows in RCM order the 256 rows of a block share many gathered entries, and
// caching them in L1 made the binary32 SpMV of the 128^3 system 5% faster
// (40.4 against 42.6 us).  The level sweeps (which read rows written earlier
// in the same launch or by a PDL predecessor) and the persistent batch kernel
// always use .cg.
#ifndef TFS_SPMV_NC
#define TFS_SPMV_NC true
#endif
template <bool NC, typename T>
__device__ __forceinline__ T gather(const T *p)
{
    if constexpr (NC) return __ldg(p);
    else return __ldcg(p);
}

// Sequential sum s - sum_{j0<=j<j1} a_j x_col(j) (SUB) or s + ... (ADD).
// Up to BW entries per pass: every column index and value of the pass is
// loaded, then every gather issued, and only then are the products summed in
// column order, so a row of up to BW entries costs three dependent memory
// round trips (geometry, entries, gathers) whatever its length.
// Four entries per pass: eight (one pass for the 7-entry rows of a hex
// mesh) raised the SpMV's registers from 32 to 40 and made it slower on the
// 128^3 system (43.8 against 40.1 us).
#ifndef TFS_ROW_BATCH
#define TFS_ROW_BATCH 4
#endif
template <bool SUB, typename VT, typename XT, typename AT, bool NC = false, int BW = TFS_ROW_BATCH>
__device__ __forceinline__ AT row_accum(AT s, const int *__restrict__ col,
                                        const VT *__restrict__ val,
                                        const XT *__restrict__ x, int off, int j0, int j1)
{
    for (int j = j0; j < j1; j += BW) {
        int k[BW];
        AT a[BW], xv[BW];
#pragma unroll
        for (int q = 0; q < BW; q++) {
            k[q] = 0;
            a[q] = (AT)0;
            if (j + q < j1) {
                const int e = off + ((j + q) << 5);
                k[q] = __ldg(col + e);
                a[q] = (AT)__ldg(val + e);
            }
        }
#pragma unroll
        for (int q = 0; q < BW; q++) xv[q] = (j + q < j1) ? (AT)gather<NC>(x + k[q]) : (AT)0;
#pragma unroll
        for (int q = 0; q < BW; q++)
            if (j + q < j1) {
                if (SUB) s = s - a[q] * xv[q];
                else s = s + a[q] * xv[q];
            }
    }
    return s;
}

// Two right-hand sides through one pass over the row (Bicg.f90:136-144).
template <bool SUB, typename VT, typename XT, typename AT, bool NC = false>
__device__ __forceinline__ void row_accum2(AT &s1, AT &s2, const int *__restrict__ col,
                                           const VT *__restrict__ val, const XT *__restrict__ x1,
                                           const XT *__restrict__ x2, int off, int j0, int j1)
{
    int j = j0;
    for (; j + 2 <= j1; j += 2) {
        int e0 = off + (j << 5), e1 = e0 + 32;
        int k0 = __ldg(col + e0), k1 = __ldg(col + e1);
        AT a0 = (AT)__ldg(val + e0), a1 = (AT)__ldg(val + e1);
        AT p0 = (AT)gather<NC>(x1 + k0), p1 = (AT)gather<NC>(x1 + k1), q0 = (AT)gather<NC>(x2 + k0),
           q1 = (AT)gather<NC>(x2 + k1);
        if (SUB) { s1 = s1 - a0 * p0; s2 = s2 - a0 * q0; s1 = s1 - a1 * p1; s2 = s2 - a1 * q1; }
        else     { s1 = s1 + a0 * p0; s2 = s2 + a0 * q0; s1 = s1 + a1 * p1; s2 = s2 + a1 * q1; }
    }
    for (; j < j1; j++) {
        int e = off + (j << 5);
        int k = __ldg(col + e);
        AT a = (AT)__ldg(val + e);
        AT p = (AT)gather<NC>(x1 + k), q = (AT)gather<NC>(x2 + k);
        if (SUB) { s1 = s1 - a * p; s2 = s2 - a * q; }
        else     { s1 = s1 + a * p; s2 = s2 + a * q; }
    }
}

// s + sum_j a_ij x_j (ADD) or s - ... (SUB) over the whole row i, for the
// SpMV-type kernels.  (Loading every entry slot of a uniform-width row
// before its length is known -- two dependent round trips instead of three
// -- measured no faster on the 128^3 system: 40.0 against 40.1 us, at 40
// registers instead of 32.)
template <bool SUB, typename VT, typename XT, typename AT, bool NC = false>
__device__ __forceinline__ AT row_spmv(AT s, const SellDev &A, const VT *__restrict__ val,
                                       const XT *__restrict__ x, int i)
{
    const RowGeom g = row_geom(A, i);
    return row_accum<SUB, VT, XT, AT, NC>(s, A.col, val, x, g.off, 0, g.len);
}

// Fixed-shape block sum of NV values; the result is valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double (*sm)[TFS_TPB / 32])
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] = v[k] + __shfl_down_sync(FULL, v[k], o);
        if (lane == 0) sm[k][warp] = v[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = sm[k][0];
#pragma unroll
            for (int w = 1; w < TFS_TPB / 32; w++) s = s + sm[k][w];
            v[k] = s;
        }
    }
}

// Sum over a warp of binary32 values, returned in binary64 by lane 0.  The
// running sum is a binary32 pair (hi, lo) updated with Knuth's TwoSum, so it
// carries about 48 significant bits without any binary64 instruction per
// lane (GB300's binary64 pipe is narrow: a binary64 shuffle reduction of
// every thread's partial kept it half busy in the binary32 vector kernels).
__device__ __forceinline__ void warp_sum_f2(float v, float &hi, float &lo)
{
    hi = v;
    lo = 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_down_sync(FULL, hi, o), l2 = __shfl_down_sync(FULL, lo, o);
        const float s = hi + h2;
        const float bp = s - hi;
        const float e = (hi - (s - bp)) + (h2 - bp);
        hi = s;
        lo = (lo + l2) + e;
    }
}

__device__ __forceinline__ double warp_sum_f(float v)
{
    float hi, lo;
    warp_sum_f2(v, hi, lo);
    return (double)hi + (double)lo;
}

// Block sum of NV binary32 values; the binary64 result is valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum_f(const float (&v)[NV], double (&out)[NV],
                                            double (*sm)[TFS_TPB / 32])
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        float hi, lo;
        warp_sum_f2(v[k], hi, lo);
        if (lane == 0) sm[k][warp] = (double)hi + (double)lo;   // binary64 in lane 0 only
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = sm[k][0];
#pragma unroll
            for (int w = 1; w < TFS_TPB / 32; w++) s = s + sm[k][w];
            out[k] = s;
        }
    }
}

// Second half of a single-pass grid reduction: thread 0 of every block
// publishes its block totals v, the last block to arrive sums the partials
// in block order.  Returns true in thread 0 of that last block, with the
// totals in v.
template <int NV>
__device__ __forceinline__ bool grid_publish(double (&v)[NV], double *__restrict__ part,
                                             unsigned int *counter, double (*sm)[TFS_TPB / 32])
{
    __shared__ unsigned int is_last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) part[k * gridDim.x + blockIdx.x] = v[k];
        __threadfence();
        is_last = (atomicAdd(counter, 1u) == gridDim.x - 1) ? 1u : 0u;
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
    double a[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) a[k] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += TFS_TPB) {
#pragma unroll
        for (int k = 0; k < NV; k++) a[k] = a[k] + __ldcg(part + k * gridDim.x + b);
    }
    __syncthreads();  // sm is reused
    block_sum<NV>(a, sm);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) v[k] = a[k];
        *counter = 0u;
        return true;
    }
    return false;
}

// Single-pass grid reduction of binary64 values (warp shuffles, then one
// partial per block, then the last block sums the partials in block order).
template <int NV>
__device__ __forceinline__ bool grid_reduce(double (&v)[NV], double *__restrict__ part,
                                            unsigned int *counter)
{
    __shared__ double sm[NV][TFS_TPB / 32];
    block_sum<NV>(v, sm);
    return grid_publish<NV>(v, part, counter, sm);
}

// The same for binary32 per-thread values (binary64 from the warp sums on).
// Returns true in thread 0 of the last block, with the totals in out.
template <int NV>
__device__ __forceinline__ bool grid_reduce_f(const float (&v)[NV], double (&out)[NV],
                                              double *__restrict__ part, unsigned int *counter)
{
    __shared__ double sm[NV][TFS_TPB / 32];
    block_sum_f<NV>(v, out, sm);
    return grid_publish<NV>(out, part, counter, sm);
}

// Row loops of the vector kernels: four chunks per step, with every load of
// the four rows issued before any of them is used (memory-level parallelism;
// the stores of one row could otherwise alias the loads of the next).
#define TFS_QUAD_BEGIN(nch)                                                   \
    for (int _c0 = blockIdx.x; _c0 < (nch); _c0 += 4 * (int)gridDim.x) {    \
        int _i[4];                                                           \
        bool _ok[4];                                                         \
        _Pragma("unroll") for (int _q = 0; _q < 4; _q++) {                   \
            int _c = _c0 + _q * (int)gridDim.x;                              \
            _ok[_q] = _c < (nch);                                            \
            _i[_q] = _ok[_q] ? _c * TFS_TPB + (int)threadIdx.x : 0;          \
        }
#define TFS_QLOAD(arr, ptr)                                                   \
    _Pragma("unroll") for (int _q = 0; _q < 4; _q++) arr[_q] = (ptr)[_i[_q]];
#define TFS_QUAD_FOR _Pragma("unroll") for (int _q = 0; _q < 4; _q++) if (_ok[_q])
#define TFS_QUAD_END }

__device__ __forceinline__ void set_cond(cudaGraphConditionalHandle cond, unsigned v)
{
    if (cond) cudaGraphSetConditional(cond, v);
}

// beta = rho / rho_old for the coming p update, once per iteration (a
// binary64 division is a long instruction sequence on GB300's narrow
// binary64 pipe; every thread dividing cost several microseconds).
__device__ __forceinline__ void publish_beta(DevState *st)
{
    const double b = st->rho / st->rho_old;
    st->beta = b;
    st->beta32 = (float)b;
}

// Convergence test and bookkeeping at the end of one iteration, run by one
// thread: Cg.f90:167-176 (Bicg.f90:180-189, Cgs.f90:212-221).
__device__ __forceinline__ void finish_iteration(DevState *st, double e2, double rho_next,
                                                 bool fused_rho, cudaGraphConditionalHandle cond)
{
    double err = sqrt(e2);
    st->error = err;
    st->fin_res = err;
    int it = st->iter;
    if (!(err <= DBL_MAX)) {                 // NaN or Inf: breakdown
        st->status = TFS_ERR_NONFINITE;
        st->done = 1;
        st->niter_out = (st->niter_max > 0 ? st->niter_max : 0) + 1;
    } else if (err < st->tol) {
        st->done = 1;
        st->niter_out = it;
    } else if (it >= st->niter_max) {        // DO loop exhausted: iter = niter + 1
        st->done = 1;
        st->niter_out = it + 1;
    } else {
        st->iter = it + 1;
        st->rho_old = st->rho;               // Cg.f90:176
        if (fused_rho) {
            st->rho = rho_next;
            publish_beta(st);
        }
    }
    st->loops = st->loops + 1;
    if (!st->done && st->loops >= st->loop_limit) {
        st->done = 1;
        st->status = TFS_ERR_TIMEOUT;
        st->niter_out = it + 1;
    }
    set_cond(cond, st->done ? 0u : 1u);
}

// ---------------------------------------------------------------- prologue

__global__ void k_init(DevState *st, const DevParams *prm, int prec)
{
    DevState s = {};
    s.tol = prm->tol;
    s.niter_max = prm->niter_max;
    s.prec = prec;
    s.iter = 1;
    s.loop_limit = (prm->niter_max > 0 ? prm->niter_max : 0) + 8;
    s.delta = 0.1;
    s.t_begin = gtimer();
    s.dicb_wait_ns = prm->dicb_wait_ns;
    *st = s;
}

// val (internal SELL order) <- val_csr (natural CSR order) through vmap.
__global__ void k_gather_val(const int *__restrict__ vmap, const DevParams *prm,
                             double *__restrict__ val, float *__restrict__ val32, int nnz_pad)
{
    const double *src = prm->val_csr;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nnz_pad; e += gridDim.x * blockDim.x) {
        int m = __ldg(vmap + e);
        double v = m >= 0 ? src[m] : 0.0;
        val[e] = v;
        if (val32) val32[e] = (float)v;
    }
}

// r <- b, x <- x0 in internal order; d <- a_ii (prec 1) or 1; ||b|| and the
// first early exit (Cg.f90:48-58).
__global__ void __launch_bounds__(TFS_TPB)
k_load(SellDev A, const double *__restrict__ val, const int *__restrict__ perm,
       const DevParams *prm, Vec64 V, DevState *st, double *part, int prec)
{
    const double *b = prm->b, *x0 = prm->x;
    const bool zero = prm->x0_zero != 0;
    double acc = 0.0;
    for (int c = blockIdx.x; c < A.n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        int o = __ldg(perm + i);
        double bi = 0.0, xi = 0.0;
        if (o >= 0) { bi = b[o]; xi = zero ? 0.0 : x0[o]; }
        V.r[i] = bi;
        V.x[i] = xi;
        acc = fma(bi, bi, acc);
        RowGeom g = row_geom(A, i);
        V.d[i] = (prec == 1 && g.len > 0) ? val[g.off + (g.dpos << 5)] : 1.0;
    }
    double v[1] = {acc};
    if (grid_reduce<1>(v, part, &st->counter)) {
        double bnrm2 = sqrt(v[0]);
        st->bnrm2 = bnrm2;
        if (bnrm2 < st->tol) {
            st->done = 1;
            st->early = 1;
            st->niter_out = 0;
            st->error = bnrm2;
            st->fin_res = bnrm2;
        }
    }
}

// r1 <- r1 - A x (Residual.f90:22-27), ||r0|| and the second early exit
// (Cg.f90:63-90).  For BiCG/CGS also r2 = r1 (Bicg.f90:91-93, Cgs.f90:71-73).
// rho of the first iteration is computed here when it needs no sweep.
// method: 0 CG, 1 BiCG, 2 CGS.
template <int METHOD>
__global__ void __launch_bounds__(TFS_TPB)
k_residual(SellDev A, const double *__restrict__ val, Vec64 V, DevState *st, double *part,
           int prec, cudaGraphConditionalHandle cond, int l0_rows = 0)
{
    if (st->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(cond, 0u);
        return;
    }
    const bool fused = (METHOD == 2) || prec != 2;
    double e2 = 0.0, rz = 0.0;
    for (int c = blockIdx.x; c < A.n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        RowGeom g = row_geom(A, i);
        double r = row_accum<true, double, double, double, TFS_SPMV_NC>(V.r[i], A.col, val, V.x, g.off, 0, g.len);
        V.r[i] = r;
        if (i < l0_rows) V.y[i] = r * V.d[i];   // forward sweep of DIC level 0
        if (METHOD != 0) V.r2[i] = r;
        e2 = fma(r, r, e2);
        if (METHOD == 2) rz = fma(r, r, rz);            // Cgs.f90:105-109, r2 = r1
        else if (fused) {                               // z = M^-1 r, kept for the p update
            double z = r / V.d[i];
            V.z[i] = z;
            if (METHOD == 1) V.z2[i] = z;
            rz = fma(r, z, rz);
        }
    }
    double v[2] = {e2, rz};
    if (grid_reduce<2>(v, part, &st->counter)) {
        double err = sqrt(v[0]);
        st->error = err;
        st->fin_res = err;
        st->ini_res = err;
        if (!(err <= DBL_MAX)) {
            st->status = TFS_ERR_NONFINITE;
            st->done = 1;
            st->niter_out = (st->niter_max > 0 ? st->niter_max : 0) + 1;
        } else if (err < st->tol) {
            st->done = 1;
            st->early = 2;
            st->niter_out = 0;
        } else if (st->niter_max <= 0) {     // zero-trip DO loop leaves iter = 1
            st->done = 1;
            st->niter_out = 1;
        } else if (fused) {
            st->rho = v[1];
        }
        set_cond(cond, st->done ? 0u : 1u);
    }
}

// ------------------------------------------------------- level-scheduled DIC

// ------------------------------------------------------ sweep rows

// Profiling stamps of one block of a sweep launch (tfs_profile_prec): the
// global timer after the dependency wait (t0) and once every thread of the
// block is done.
__device__ __forceinline__ void stamp_block(unsigned long long *stp, int stride, int slot,
                                            unsigned long long t0)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long *q = stp + (size_t)slot * stride + 2 * blockIdx.x;
        q[0] = t0;
        q[1] = gtimer();
    }
}

// One row of a sweep.  MODE 0: forward y = (b - L y) * D; MODE 1: backward
// z = (y/(D+TINY) - U z) * D; MODE 2: DIC form D_i = 1/(a_ii - sum D_k a^2).
// The first NP entries may come prefetched in kk/aa.  With skip (a finished
// solve) nothing is stored; the flag is tested only before the stores, so
// reading it does not delay the row's loads.
template <typename T, int NR, int MODE, int NP>
__device__ __forceinline__ void sweep_row(const SellDev &A, const T *__restrict__ val, T *d,
                                          const T *b1, const T *b2, T *o1, T *o2, const T *y1,
                                          const T *y2, int i, const RowGeom &g, const int *kk,
                                          const T *aa, bool skip = false)
{
    const int j0 = MODE == 1 ? g.dpos + 1 : 0, j1 = MODE == 1 ? g.len : g.dpos;
    if (g.len == 0) {
        if (skip) return;
        if (MODE == 2) d[i] = (T)1;
        else { o1[i] = (T)0; if (NR == 2) o2[i] = (T)0; }
        return;
    }
    T s1, s2 = (T)0, di = (T)0;
    if (MODE == 2) {
        s1 = __ldg(val + g.off + (g.dpos << 5));
    } else {
        di = d[i];
        if (MODE == 0) { s1 = b1[i]; if (NR == 2) s2 = b2[i]; }
        else { s1 = y1[i] / (di + (T)TINY); if (NR == 2) s2 = y2[i] / (di + (T)TINY); }
    }
    // Entries in ascending column order: the prefetched ones first.
    int j = j0;
#pragma unroll
    for (int q = 0; q < NP; q++) {
        if (j < j1) {
            const int k = kk[q];
            const T a = aa[q];
            if (MODE == 2) s1 = s1 - __ldcg(d + k) * a * a;
            else {
                s1 = s1 - a * __ldcg(o1 + k);
                if (NR == 2) s2 = s2 - a * __ldcg(o2 + k);
            }
            j++;
        }
    }
    for (; j < j1; j++) {
        const int ee = g.off + (j << 5);
        const int k = __ldg(A.col + ee);
        const T a = __ldg(val + ee);
        if (MODE == 2) s1 = s1 - __ldcg(d + k) * a * a;
        else {
            s1 = s1 - a * __ldcg(o1 + k);
            if (NR == 2) s2 = s2 - a * __ldcg(o2 + k);
        }
    }
    if (skip) return;
    if (MODE == 2) { d[i] = (T)1 / s1; return; }
    o1[i] = s1 * di;
    if (NR == 2) o2[i] = s2 * di;
}

// ------------------------------------------------ one launch per level
//
// The default schedule: one kernel per large level, launched with
// programmatic dependent launch (PDL).  A level kernel first reads what does
// not depend on the previous level (row geometry and its first column
// indices and values: TFS_FWD_PRE_SLOTS forward, TFS_BWD_SLOTS backward,
// four otherwise), then lets the next level's kernel start
// (cudaTriggerProgrammaticLaunchCompletion) and waits for the previous one
// (cudaGridDependencySynchronize), so launch latency and prefetch overlap the
// previous level.  The small trailing levels run in one single-block kernel
// (k_sweep_tail) with __syncthreads() between levels.  One row per thread:
// two or four rows per thread (fewer thread slots per level, so the next
// level's blocks could become resident earlier) measured 1.4x and 2.3x
// slower on the 128^3 system, since a thread's rows then run their dependent
// gathers one after the other.
// Backward row (MODE 1 of sweep_row) whose start value s = y_i / (D_i +
// TINY) and D_i were computed before the dependency wait.  The gathers of
// the prefetched entries are all issued before the first update (here and
// in sweep_row_fwd_pre): __ldcg is a volatile load, so one guarded by its
// own entry test and followed by its update went out only after the
// previous update, one memory round trip per entry.  Issued together they
// cost one round trip per row: on the 128^3 system a binary32 DIC
// application took 97.8 against 115.2 us, with the same arithmetic in the
// same order.
template <typename T, int NR, int NP>
__device__ __forceinline__ void sweep_row_bwd_pre(const SellDev &A, const T *__restrict__ val, T *o1, T *o2,
                                                  int i, const RowGeom &g, const int *kk, const T *aa, T s1,
                                                  T s2, T di, bool skip)
{
    if (g.len == 0) {
        if (skip) return;
        o1[i] = (T)0;
        if (NR == 2) o2[i] = (T)0;
        return;
    }
    const int j0 = g.dpos + 1, j1 = g.len;
    T x1[NP], x2[NP];
#pragma unroll
    for (int q = 0; q < NP; q++) {
        x1[q] = (T)0;
        x2[q] = (T)0;
        if (j0 + q < j1) {
            x1[q] = __ldcg(o1 + kk[q]);
            if (NR == 2) x2[q] = __ldcg(o2 + kk[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < NP; q++)
        if (j0 + q < j1) {
            s1 = s1 - aa[q] * x1[q];
            if (NR == 2) s2 = s2 - aa[q] * x2[q];
        }
    int j = j0 + NP < j1 ? j0 + NP : j1;
    for (; j < j1; j++) {
        const int ee = g.off + (j << 5);
        const int k = __ldg(A.col + ee);
        const T a = __ldg(val + ee);
        s1 = s1 - a * __ldcg(o1 + k);
        if (NR == 2) s2 = s2 - a * __ldcg(o2 + k);
    }
    if (skip) return;
    o1[i] = s1 * di;
    if (NR == 2) o2[i] = s2 * di;
}

// Forward row (MODE 0 of sweep_row) whose right-hand side b_i and D_i were
// loaded before the dependency wait; gathers issued as in sweep_row_bwd_pre.
template <typename T, int NR, int NP>
__device__ __forceinline__ void sweep_row_fwd_pre(const SellDev &A, const T *__restrict__ val, T *o1, T *o2,
                                                  int i, const RowGeom &g, const int *kk, const T *aa, T s1,
                                                  T s2, T di, bool skip)
{
    if (g.len == 0) {
        if (skip) return;
        o1[i] = (T)0;
        if (NR == 2) o2[i] = (T)0;
        return;
    }
    const int j1 = g.dpos;
    T x1[NP], x2[NP];
#pragma unroll
    for (int q = 0; q < NP; q++) {
        x1[q] = (T)0;
        x2[q] = (T)0;
        if (q < j1) {
            x1[q] = __ldcg(o1 + kk[q]);
            if (NR == 2) x2[q] = __ldcg(o2 + kk[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < NP; q++)
        if (q < j1) {
            s1 = s1 - aa[q] * x1[q];
            if (NR == 2) s2 = s2 - aa[q] * x2[q];
        }
    int j = j1 < NP ? j1 : NP;
    for (; j < j1; j++) {
        const int ee = g.off + (j << 5);
        const int k = __ldg(A.col + ee);
        const T a = __ldg(val + ee);
        s1 = s1 - a * __ldcg(o1 + k);
        if (NR == 2) s2 = s2 - a * __ldcg(o2 + k);
    }
    if (skip) return;
    o1[i] = s1 * di;
    if (NR == 2) o2[i] = s2 * di;
}

//
// PREY (backward sweep after a tail kernel, which releases its dependants
// only once it has passed its own wait, so the forward sweep is complete
// when this kernel starts): the row's start value y_i / (D_i + TINY) is
// computed before the wait, taking the division off the dependent chain.
#define TFS_FWD_PRE_SLOTS 6   // forward level kernels: slots loaded before the dependency wait
// Backward level kernels (PREY): binary32 six (mixed 128^3 DIC-CG 17.31
// against 17.14 solves/s with four), binary64 four (six spill at its
// 40-register cap: 7.46 against 7.68 solves/s).
#define TFS_BWD_PRE_SLOTS 6
#define TFS_BWD_SLOTS(T) (sizeof(T) == 4 ? TFS_BWD_PRE_SLOTS : 4)
// Level kernels of 256 threads: binary64 held to 40 registers (6 blocks per
// SM; the backward kernel would take 48, 5 blocks): 7.43 against 7.36
// binary64 solves/s at 128^3; binary32 to 32 (8 blocks per SM, what the
// compiler picks unbounded; allowed 40 it took 40 and lost 7%).  Other
// block sizes (TFS_OPT_LEVEL_TPB) at most 64 registers.
template <typename T, int NR, int MODE, int BS = TFS_TPB, bool PREY = false>
__global__ void __launch_bounds__(BS, BS == 256 ? (sizeof(T) == 8 ? 6 : 8) : (BS >= 1024 ? 1 : 1024 / BS))
k_sweep_level(SellDev A, const T *__restrict__ val, T *d, const T *b1, const T *b2, T *o1,
              T *o2, const T *y1, const T *y2, int row0, int row1, DevState *st, int tag)
{
    // tag = first launch of the application | slot << 1 (profiling stamps)
    const int first = tag & 1;
    const int i = row0 + blockIdx.x * BS + threadIdx.x;
    const bool active = i < row1;
    RowGeom g{0, 0, 0};
    int kk[TFS_FWD_PRE_SLOTS] = {};
    T aa[TFS_FWD_PRE_SLOTS] = {};
    if (active) {
        if (MODE == 0 && A.width > 0) {
            // Uniform slice width: the first slots are where they are
            // whatever the row's geometry says, so their loads do not wait
            // for it (slots past the row's length hold column 0, value 0).
            // Six slots hold every lower entry of a 7-entry row: measured on
            // the 128^3 system 4 / 6 / 8 slots 126.2 / 116.9 / 119.3 us per
            // DIC application (14.92 / 15.54 / 15.31 solves/s mixed, before
            // the row routines issued their gathers together).  Backward
            // levels load their slots after the geometry (TFS_BWD_SLOTS).
            const int off = (i & ~31) * A.width + (i & 31);
            g = row_geom(A, i);
#pragma unroll
            for (int q = 0; q < TFS_FWD_PRE_SLOTS; q++)
                if (q < A.width) {
                    kk[q] = __ldg(A.col + off + (q << 5));
                    aa[q] = __ldg(val + off + (q << 5));
                }
        } else {
            g = row_geom(A, i);
            const int j0 = MODE == 1 ? g.dpos + 1 : 0, j1 = MODE == 1 ? g.len : g.dpos;
            // as many as the forward row routine below takes from kk / aa
#pragma unroll
            for (int q = 0; q < (MODE == 0 && PREY ? TFS_FWD_PRE_SLOTS : MODE == 1 && PREY ? TFS_BWD_SLOTS(T) : 4); q++)
                if (j0 + q < j1) {
                    int ee = g.off + ((j0 + q) << 5);
                    kk[q] = __ldg(A.col + ee);
                    aa[q] = __ldg(val + ee);
                }
        }
    }
    T pdi = (T)0, ps1 = (T)0, ps2 = (T)0;
    if (MODE == 1 && PREY && active && g.len > 0) {
        pdi = d[i];
        ps1 = y1[i] / (pdi + (T)TINY);
        if (NR == 2) ps2 = y2[i] / (pdi + (T)TINY);
    }
    // Forward sweep: the right-hand side and D come from kernels that
    // completed before the level chain started, so they load before the
    // wait as well (PREY = true for MODE 0).
    if (MODE == 0 && PREY && active && g.len > 0) {
        pdi = d[i];
        ps1 = b1[i];
        if (NR == 2) ps2 = b2[i];
    }
    cudaTriggerProgrammaticLaunchCompletion();
    cudaGridDependencySynchronize();
    const bool skip = st->done != 0;
    unsigned long long *const stp = st->stamps;
    const unsigned long long t0 = stp ? gtimer() : 0ull;
    if (MODE == 0 && first && blockIdx.x == 0 && threadIdx.x == 0) st->t_sweep0 = gtimer();
    if (MODE == 1 && PREY) {
        if (active) sweep_row_bwd_pre<T, NR, TFS_BWD_SLOTS(T)>(A, val, o1, o2, i, g, kk, aa, ps1, ps2, pdi, skip);
    } else if (MODE == 0 && PREY) {
        if (active) sweep_row_fwd_pre<T, NR, TFS_FWD_PRE_SLOTS>(A, val, o1, o2, i, g, kk, aa, ps1, ps2, pdi, skip);
    } else if (active) {
        sweep_row<T, NR, MODE, 4>(A, val, d, b1, b2, o1, o2, y1, y2, i, g, kk, aa, skip);
    }
    if (stp) stamp_block(stp, st->stamp_stride, tag >> 1, t0);
}

// Levels [l_begin, l_end) of a sweep in one block (descending for MODE 1);
// every level has at most TFS_SWEEP_TPB rows, one row per thread.  While a
// level is computed, the row geometry and the first entries of the thread's
// row of the next level are already being loaded, so each level costs little
// more than its dependent gathers and a __syncthreads().
template <typename T, int NR, int MODE>
__global__ void __launch_bounds__(TFS_SWEEP_TPB)
k_sweep_tail(SellDev A, const T *__restrict__ val, T *d, const T *b1, const T *b2, T *o1,
             T *o2, const T *y1, const T *y2, const int *__restrict__ lvl_begin, int l_begin,
             int l_end, DevState *st, int first)
{
    const int nl = l_end - l_begin;
    auto level_of = [&](int q) { return MODE == 1 ? l_end - 1 - q : l_begin + q; };
    auto fetch = [&](int q, int &i, RowGeom &g, int (&kk)[4], T (&aa)[4]) {
        const int lev = level_of(q);
        i = __ldg(lvl_begin + lev) + (int)threadIdx.x;
        const int r1 = __ldg(lvl_begin + lev + 1);
        g = RowGeom{0, 0, 0};
        if (i >= r1) { i = -1; return; }
        g = row_geom(A, i);
        const int j0 = MODE == 1 ? g.dpos + 1 : 0, j1 = MODE == 1 ? g.len : g.dpos;
#pragma unroll
        for (int q2 = 0; q2 < 4; q2++)
            if (j0 + q2 < j1) {
                int ee = g.off + ((j0 + q2) << 5);
                kk[q2] = __ldg(A.col + ee);
                aa[q2] = __ldg(val + ee);
            }
    };
    int i = -1, ni = -1;
    RowGeom g, ng;
    int kk[4] = {0, 0, 0, 0}, nkk[4] = {0, 0, 0, 0};
    T aa[4] = {(T)0, (T)0, (T)0, (T)0}, naa[4] = {(T)0, (T)0, (T)0, (T)0};
    if (nl > 0) fetch(0, i, g, kk, aa);
    cudaTriggerProgrammaticLaunchCompletion();
    cudaGridDependencySynchronize();
    if (st->done) return;
    if (MODE == 0 && first && threadIdx.x == 0) st->t_sweep0 = gtimer();
    for (int q = 0; q < nl; q++) {
        if (q + 1 < nl) fetch(q + 1, ni, ng, nkk, naa);
        if (i >= 0) sweep_row<T, NR, MODE, 4>(A, val, d, b1, b2, o1, o2, y1, y2, i, g, kk, aa);
        __syncthreads();
        i = ni;
        g = ng;
#pragma unroll
        for (int q2 = 0; q2 < 4; q2++) { kk[q2] = nkk[q2]; aa[q2] = naa[q2]; }
    }
}

// Both tails of one preconditioner application in one block: the forward
// sweep of the tail levels (ascending), then their backward sweep
// (descending).  The backward rows of the tail depend only on tail rows and on
// their own forward value, all produced by this block, so no grid-wide step
// separates the two halves.
template <typename T, int NR>
__global__ void __launch_bounds__(TFS_SWEEP_TPB)
k_sweep_tail2(SellDev A, const T *__restrict__ val, T *d, const T *b1, const T *b2, T *y1, T *y2,
              T *z1, T *z2, const int *__restrict__ lvl_begin, int l_begin, int l_end, DevState *st, int slot)
{
    // The trigger follows the wait: the backward level kernels launched
    // after a tail read the forward sweep's output before their own wait.
    cudaGridDependencySynchronize();
    cudaTriggerProgrammaticLaunchCompletion();
    const bool skip = st->done != 0;
    unsigned long long *const stp = st->stamps;
    const unsigned long long t0 = stp ? gtimer() : 0ull;
    const int nl = l_end - l_begin;
    for (int q = 0; q < nl; q++) {
        const int lev = l_begin + q;
        const int r1 = __ldg(lvl_begin + lev + 1);
        for (int i = __ldg(lvl_begin + lev) + threadIdx.x; i < r1; i += TFS_SWEEP_TPB) {
            RowGeom g = row_geom(A, i);
            sweep_row<T, NR, 0, 0>(A, val, d, b1, b2, y1, y2, nullptr, nullptr, i, g, nullptr, nullptr, skip);
        }
        __syncthreads();
    }
    for (int q = 0; q < nl; q++) {
        const int lev = l_end - 1 - q;
        const int r1 = __ldg(lvl_begin + lev + 1);
        for (int i = __ldg(lvl_begin + lev) + threadIdx.x; i < r1; i += TFS_SWEEP_TPB) {
            RowGeom g = row_geom(A, i);
            sweep_row<T, NR, 1, 0>(A, val, d, nullptr, nullptr, z1, z2, y1, y2, i, g, nullptr, nullptr, skip);
        }
        __syncthreads();
    }
    if (stp) stamp_block(stp, st->stamp_stride, slot, t0);
}

// Both tails by one block when the tail has at most TFS_SWEEP_TPB rows in
// all (one row per thread) and the matrix has uniform slice width W <= 8:
// every thread loads its row's geometry, entries, right-hand side and
// diagonal before cudaGridDependencySynchronize (none of them is written by
// the level kernels this launch may overlap: b and D come from kernels that
// completed before the first level kernel of the sweep started), so a level
// step is only the gathers of the rows written in the steps before, the
// row's arithmetic and a block barrier.  Per-row arithmetic as sweep_row.
template <typename T>
__global__ void __launch_bounds__(TFS_SWEEP_TPB)
k_sweep_tail1(SellDev A, const T *__restrict__ val, const T *d, const T *b, T *y, T *z,
              const int *__restrict__ lvl_begin, int l_begin, int l_end, DevState *st, int slot)
{
    const int i = __ldg(lvl_begin + l_begin) + (int)threadIdx.x;
    const bool mine = i < __ldg(lvl_begin + l_end);
    int lev = -1;
    RowGeom g{0, 0, 0};
    int kk[8];
    T aa[8];
    T bi = (T)0, di = (T)0;
#pragma unroll
    for (int j = 0; j < 8; j++) { kk[j] = 0; aa[j] = (T)0; }
    if (mine) {
        lev = l_begin;
        while (__ldg(lvl_begin + lev + 1) <= i) lev++;
        g = row_geom(A, i);
#pragma unroll
        for (int j = 0; j < 8; j++)
            if (j < g.len) {
                kk[j] = __ldg(A.col + g.off + (j << 5));
                aa[j] = __ldg(val + g.off + (j << 5));
            }
        if (g.len > 0) { bi = b[i]; di = d[i]; }
    }
    cudaGridDependencySynchronize();
    cudaTriggerProgrammaticLaunchCompletion();   // after the wait, as in k_sweep_tail2
    const bool skip = st->done != 0;
    unsigned long long *const stp = st->stamps;
    const unsigned long long t0 = stp ? gtimer() : 0ull;
    // The tail's own rows keep their values in shared memory as well (a
    // level's gathers of rows of earlier tail levels are shared-memory loads
    // after the block barrier); the values of rows below the tail, final
    // since the dependency wait, are all gathered at once right after it.
    __shared__ T ty[TFS_SWEEP_TPB], tz[TFS_SWEEP_TPB];
    const int r0 = __ldg(lvl_begin + l_begin);
    T xv[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        xv[j] = (T)0;
        if (mine && j < g.dpos && kk[j] < r0) xv[j] = __ldcg(y + kk[j]);
    }
    T yi = (T)0;
    for (int l = l_begin; l < l_end; l++) {
        if (lev == l) {
            if (g.len == 0) {
                if (!skip) y[i] = (T)0;
                ty[threadIdx.x] = (T)0;
            } else {
                T s = bi;
#pragma unroll
                for (int j = 0; j < 8; j++)
                    if (j < g.dpos) s = s - aa[j] * (kk[j] < r0 ? xv[j] : ty[kk[j] - r0]);
                yi = s * di;
                if (!skip) y[i] = yi;
                ty[threadIdx.x] = yi;
            }
        }
        __syncthreads();
    }
    // Every row's backward start value, all at once after the forward half
    // (one division per thread instead of one on every backward step).
    const T q0 = (mine && g.len > 0) ? yi / (di + (T)TINY) : (T)0;
    for (int l = l_end - 1; l >= l_begin; l--) {
        if (lev == l) {
            if (g.len == 0) {
                if (!skip) z[i] = (T)0;
                tz[threadIdx.x] = (T)0;
            } else {
                T s = q0;
#pragma unroll
                for (int j = 0; j < 8; j++)
                    if (j > g.dpos && j < g.len) s = s - aa[j] * (kk[j] >= r0 ? tz[kk[j] - r0] : __ldcg(z + kk[j]));
                const T zi = s * di;
                if (!skip) z[i] = zi;
                tz[threadIdx.x] = zi;
            }
        }
        __syncthreads();
    }
    if (stp) stamp_block(stp, st->stamp_stride, slot, t0);
}

// rho after the sweeps: CG (r, z) (Cg.f90:108-112); BiCG (z1, r2) (Bicg.f90:113-117).
template <int METHOD>
__global__ void __launch_bounds__(TFS_TPB)
k_dot_rho(int n_chunks, Vec64 V, DevState *st, double *part)
{
    // PDL secondary (a no-op when launched plainly): wait for the
    // predecessor before reading anything, then let the successor launch.
    cudaGridDependencySynchronize();
    cudaTriggerProgrammaticLaunchCompletion();
    const bool stop = st->done != 0;
    double acc = 0.0;
    TFS_QUAD_BEGIN(n_chunks)
        double a[4], b[4];
        TFS_QLOAD(a, METHOD == 0 ? V.r : V.z);
        TFS_QLOAD(b, METHOD == 0 ? V.z : V.r2);
        if (stop) return;
        TFS_QUAD_FOR acc = fma(a[_q], b[_q], acc);
    TFS_QUAD_END
    if (stop) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->sweep_ns += gtimer() - st->t_sweep0;
        st->sweep_n += 1;
    }
    double v[1] = {acc};
    if (grid_reduce<1>(v, part, &st->counter)) {
        st->rho = v[0];
        if (st->iter > 1) publish_beta(st);
    }
}

// ---------------------------------------------------------------- CG body

// p = z (first iteration) or z + beta p (Cg.f90:114-123); z = r/d unless the
// DIC sweeps produced it (FROMZ).
template <bool FROMZ>
__global__ void __launch_bounds__(TFS_TPB) k_cg_p(int n_chunks, Vec64 V, const DevState *st)
{
    cudaGridDependencySynchronize();   // PDL secondary, as k_dot_rho
    cudaTriggerProgrammaticLaunchCompletion();
    const bool stop = st->done != 0;
    const int it = st->iter;
    const double beta = st->beta;            // rho / rho_old, published once
    TFS_QUAD_BEGIN(n_chunks)
        double z[4], p[4];
        if (FROMZ) { TFS_QLOAD(z, V.z); }
        else { double r[4], d[4]; TFS_QLOAD(r, V.r); TFS_QLOAD(d, V.d); TFS_QUAD_FOR z[_q] = r[_q] / d[_q]; }
        TFS_QLOAD(p, V.p);
        if (stop) return;
        TFS_QUAD_FOR V.p[_i[_q]] = it == 1 ? z[_q] : z[_q] + beta * p[_q];
    TFS_QUAD_END
}

// q = A p (Cg.f90:128-134) fused with (p, q) and alpha = rho / (p, q)
// (Cg.f90:148-153).
__global__ void __launch_bounds__(TFS_TPB)
k_spmv_pq(SellDev A, const double *__restrict__ val, const double *__restrict__ p,
          double *__restrict__ q, DevState *st, double *part)
{
    // The finished-solve flag is tested after the first row's loads are
    // issued (here and in the other per-iteration kernels), so that its
    // load does not delay them.
    const bool stop = st->done != 0;
    if (!stop && blockIdx.x == 0 && threadIdx.x == 0) st->t_spmv0 = gtimer();
    double acc = 0.0;
    for (int c = blockIdx.x; c < A.n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        double s = row_spmv<false, double, double, double, TFS_SPMV_NC>(0.0, A, val, p, i);
        if (stop) return;
        q[i] = s;
        acc = fma(p[i], s, acc);
    }
    if (stop) return;
    double v[1] = {acc};
    if (grid_reduce<1>(v, part, &st->counter)) {
        st->alpha = st->rho / v[0];
        st->spmv_ns += gtimer() - st->t_spmv0;
        st->spmv_n += 1;
    }
}

// x += alpha p, r -= alpha q (Cg.f90:159-162), ||r|| and the test; with
// FUSED also rho of the next iteration, (r, r/d).
template <bool FUSED>
__global__ void __launch_bounds__(TFS_TPB)
k_cg_update(int n_chunks, Vec64 V, DevState *st, double *part, cudaGraphConditionalHandle cond,
            int l0_rows = 0)
{
    // PDL secondary; no early trigger: the DIC level chain of the next
    // iteration reads r before its own waits.
    cudaGridDependencySynchronize();
    const bool stop = st->done != 0;
    const double alfa = st->alpha;
    double e2 = 0.0, rz = 0.0;
    TFS_QUAD_BEGIN(n_chunks)
        double x[4], p[4], r[4], q[4], d[4];
        TFS_QLOAD(x, V.x); TFS_QLOAD(p, V.p); TFS_QLOAD(r, V.r); TFS_QLOAD(q, V.q);
        if (FUSED) { TFS_QLOAD(d, V.d); }
        if (stop) break;
        TFS_QUAD_FOR {
            const int i = _i[_q];
            V.x[i] = x[_q] + alfa * p[_q];
            double rn = r[_q] - alfa * q[_q];
            V.r[i] = rn;
            // DIC level 0 has no lower neighbours: its forward sweep y = r D.
            if (i < l0_rows) V.y[i] = rn * V.d[i];
            e2 = fma(rn, rn, e2);
            if (FUSED) { double z = rn / d[_q]; V.z[i] = z; rz = fma(rn, z, rz); }
        }
    TFS_QUAD_END
    if (stop) {
        if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(cond, 0u);
        return;
    }
    double v[2] = {e2, rz};
    if (grid_reduce<2>(v, part, &st->counter)) finish_iteration(st, v[0], v[1], FUSED, cond);
}

// -------------------------------------------------------------- BiCG body

template <bool FROMZ>
__global__ void __launch_bounds__(TFS_TPB) k_bicg_p(int n_chunks, Vec64 V, const DevState *st)
{
    if (st->done) return;
    const int it = st->iter;
    const double beta = it == 1 ? 0.0 : st->beta;
    TFS_QUAD_BEGIN(n_chunks)
        double z1[4], z2[4], p1[4], p2[4];
        if (FROMZ) { TFS_QLOAD(z1, V.z); TFS_QLOAD(z2, V.z2); }
        else {
            double r1[4], r2[4], d[4];
            TFS_QLOAD(r1, V.r); TFS_QLOAD(r2, V.r2); TFS_QLOAD(d, V.d);
            TFS_QUAD_FOR { z1[_q] = r1[_q] / d[_q]; z2[_q] = r2[_q] / d[_q]; }
        }
        TFS_QLOAD(p1, V.p); TFS_QLOAD(p2, V.p2);
        TFS_QUAD_FOR {
            const int i = _i[_q];
            if (it == 1) { V.p[i] = z1[_q]; V.p2[i] = z2[_q]; }
            else { V.p[i] = z1[_q] + beta * p1[_q]; V.p2[i] = z2[_q] + beta * p2[_q]; }
        }
    TFS_QUAD_END
}

// q1 = A p1 and q2 = A p2 in one pass over A (Bicg.f90:136-144), fused with
// (p2, q1) and alpha (Bicg.f90:160-165).
__global__ void __launch_bounds__(TFS_TPB)
k_spmv2_pq(SellDev A, const double *__restrict__ val, Vec64 V, DevState *st, double *part)
{
    if (st->done) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->t_spmv0 = gtimer();
    double acc = 0.0;
    for (int c = blockIdx.x; c < A.n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        RowGeom g = row_geom(A, i);
        double s1 = 0.0, s2 = 0.0;
        row_accum2<false, double, double, double, TFS_SPMV_NC>(s1, s2, A.col, val, V.p, V.p2, g.off, 0, g.len);
        V.q[i] = s1;
        V.q2[i] = s2;
        acc = fma(V.p2[i], s1, acc);
    }
    double v[1] = {acc};
    if (grid_reduce<1>(v, part, &st->counter)) {
        st->alpha = st->rho / v[0];
        st->spmv_ns += gtimer() - st->t_spmv0;
        st->spmv_n += 1;
    }
}

// x += alpha p1, r1 -= alpha q1, r2 -= alpha q2 (Bicg.f90:171-175), ||r1||,
// test; with FUSED rho of the next iteration (r1/d, r2).
template <bool FUSED>
__global__ void __launch_bounds__(TFS_TPB)
k_bicg_update(int n_chunks, Vec64 V, DevState *st, double *part, cudaGraphConditionalHandle cond)
{
    if (st->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(cond, 0u);
        return;
    }
    const double alfa = st->alpha;
    double e2 = 0.0, rz = 0.0;
    TFS_QUAD_BEGIN(n_chunks)
        double x[4], p[4], r1[4], q1[4], r2[4], q2[4], d[4];
        TFS_QLOAD(x, V.x); TFS_QLOAD(p, V.p); TFS_QLOAD(r1, V.r); TFS_QLOAD(q1, V.q);
        TFS_QLOAD(r2, V.r2); TFS_QLOAD(q2, V.q2);
        if (FUSED) { TFS_QLOAD(d, V.d); }
        TFS_QUAD_FOR {
            const int i = _i[_q];
            V.x[i] = x[_q] + alfa * p[_q];
            double a1 = r1[_q] - alfa * q1[_q];
            double a2 = r2[_q] - alfa * q2[_q];
            V.r[i] = a1;
            V.r2[i] = a2;
            e2 = fma(a1, a1, e2);
            if (FUSED) {
                double z1 = a1 / d[_q];
                V.z[i] = z1;
                V.z2[i] = a2 / d[_q];
                rz = fma(z1, a2, rz);
            }
        }
    TFS_QUAD_END
    double v[2] = {e2, rz};
    if (grid_reduce<2>(v, part, &st->counter)) finish_iteration(st, v[0], v[1], FUSED, cond);
}

// --------------------------------------------------------------- CGS body

// u1 = r1 + beta q1, u2 = u1 + beta (q1 + beta u2) (Cgs.f90:111-122); with
// FUSEDP also p2 = u2 / d (Prec_Solve for prec 0/1).
template <bool FUSEDP>
__global__ void __launch_bounds__(TFS_TPB) k_cgs_u(int n_chunks, Vec64 V, const DevState *st)
{
    if (st->done) return;
    const int it = st->iter;
    const double beta = it == 1 ? 0.0 : st->beta;
    for (int c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        double u1, u2;
        if (it == 1) { u1 = V.r[i]; u2 = u1; }
        else {
            double q1 = V.q[i];
            u1 = V.r[i] + beta * q1;
            u2 = u1 + beta * (q1 + beta * V.u2[i]);
        }
        V.u1[i] = u1;
        V.u2[i] = u2;
        if (FUSEDP) V.p2[i] = u2 / V.d[i];
    }
}

// v2 = A p2 (Cgs.f90:132-139) with (r2, v2) and alpha (Cgs.f90:153-158).
__global__ void __launch_bounds__(TFS_TPB)
k_spmv_v(SellDev A, const double *__restrict__ val, Vec64 V, DevState *st, double *part)
{
    if (st->done) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->t_spmv0 = gtimer();
    double acc = 0.0;
    for (int c = blockIdx.x; c < A.n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        RowGeom g = row_geom(A, i);
        double s = row_accum<false, double, double, double, TFS_SPMV_NC>(0.0, A.col, val, V.p2, g.off, 0, g.len);
        V.v2[i] = s;
        acc = fma(V.r2[i], s, acc);
    }
    double v[1] = {acc};
    if (grid_reduce<1>(v, part, &st->counter)) {
        st->alpha = st->rho / v[0];
        st->spmv_ns += gtimer() - st->t_spmv0;
        st->spmv_n += 1;
    }
}

// q1 = u1 - alpha v2 (Cgs.f90:163-165), w = u1 + q1 (Cgs.f90:170-172); with
// FUSEDP p1 = w / d, else w is stored for the DIC sweeps.
template <bool FUSEDP>
__global__ void __launch_bounds__(TFS_TPB) k_cgs_q(int n_chunks, Vec64 V, const DevState *st)
{
    if (st->done) return;
    const double alfa = st->alpha;
    for (int c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        double u1 = V.u1[i];
        double q1 = u1 - alfa * V.v2[i];
        V.q[i] = q1;
        double w = u1 + q1;
        if (FUSEDP) V.p[i] = w / V.d[i];
        else V.w[i] = w;
    }
}

// x += alpha p1 (Cgs.f90:178-180); q2 = A p1 (Cgs.f90:185-191);
// r1 -= alpha q2 (Cgs.f90:205-207); ||r1||, test, rho = (r1, r2) of the next
// iteration.  q2 is used only here and is not stored.
__global__ void __launch_bounds__(TFS_TPB)
k_cgs_spmv_r(SellDev A, const double *__restrict__ val, Vec64 V, DevState *st, double *part,
             cudaGraphConditionalHandle cond)
{
    if (st->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(cond, 0u);
        return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) st->t_spmv0 = gtimer();
    const double alfa = st->alpha;
    double e2 = 0.0, rr = 0.0;
    for (int c = blockIdx.x; c < A.n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        V.x[i] = V.x[i] + alfa * V.p[i];
        RowGeom g = row_geom(A, i);
        double q2 = row_accum<false, double, double, double, TFS_SPMV_NC>(0.0, A.col, val, V.p, g.off, 0, g.len);
        double r1 = V.r[i] - alfa * q2;
        V.r[i] = r1;
        e2 = fma(r1, r1, e2);
        rr = fma(r1, V.r2[i], rr);
    }
    double v[2] = {e2, rr};
    if (grid_reduce<2>(v, part, &st->counter)) {
        st->spmv_ns += gtimer() - st->t_spmv0;
        st->spmv_n += 1;
        finish_iteration(st, v[0], v[1], true, cond);
    }
}

// --------------------------------------------------------------- epilogue

// x and r1 back to natural order.
__global__ void k_store(int n_int, const int *__restrict__ perm, const double *__restrict__ x,
                        const double *__restrict__ r, const DevParams *prm, DevState *st)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) st->t_end = gtimer();
    double *xo = prm->x, *ro = prm->r_out;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_int; i += gridDim.x * blockDim.x) {
        int o = __ldg(perm + i);
        if (o >= 0) { xo[o] = x[i]; ro[o] = r[i]; }
    }
}

// ------------------------------------------------------ single routines

__global__ void k_perm_in(int n_int, const int *__restrict__ perm, const double *__restrict__ src,
                          double *__restrict__ dst)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_int; i += gridDim.x * blockDim.x) {
        int o = __ldg(perm + i);
        dst[i] = o >= 0 ? src[o] : 0.0;
    }
}

__global__ void k_perm_out(int n_int, const int *__restrict__ perm, const double *__restrict__ src,
                           double *__restrict__ dst)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_int; i += gridDim.x * blockDim.x) {
        int o = __ldg(perm + i);
        if (o >= 0) dst[o] = src[i];
    }
}

// Diagonal of the preconditioner for prec 0 / 1 (Prec_Form.f90:24-27, 45-49).
__global__ void k_diag_form(SellDev A, const double *__restrict__ val, double *d, int prec)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n_int; i += gridDim.x * blockDim.x) {
        RowGeom g = row_geom(A, i);
        d[i] = (prec == 1 && g.len > 0) ? val[g.off + (g.dpos << 5)] : 1.0;
    }
}

// x = b / d (Prec_Solve.f90:35-38; with d = 1 the copy of :71-74).
__global__ void k_diag_apply(int n_int, const double *__restrict__ d, const double *__restrict__ b,
                             double *__restrict__ x)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_int; i += gridDim.x * blockDim.x)
        x[i] = b[i] / d[i];
}

// ------------------------------------------------- dependency analysis

// One relaxation pass of level(i) = max(0, 1 + max_{k in dep(i)} level(k)),
// dep(i) = the rows i must wait for (lrow/lcol, all k < i).  Levels only grow
// and never exceed their fixed point, so passes run in place until one
// changes nothing.
__global__ void k_level_pass(int n, const int *__restrict__ lrow, const int *__restrict__ lcol,
                             int *level, int *changed)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int l = 0;
        for (int j = __ldg(lrow + i); j < __ldg(lrow + i + 1); j++) {
            int lk = ((volatile int *)level)[__ldg(lcol + j)] + 1;
            l = lk > l ? lk : l;
        }
        if (l > level[i]) {
            level[i] = l;
            *changed = 1;
        }
    }
}

}  // namespace tfs
