// tfs_mixed.cuh -- kernels of the mixed-precision (TFS_MIXED) Krylov solves.
//
// The Krylov recurrences run on binary32 matrix values and binary32 vectors
// (r, p, q, z, ...), which cuts the bytes per iteration by about a third.
// Binary64 is kept where the accuracy is decided:
//   - every dot product (rho, (p,q), ||r||) is summed in binary32 over a
//     thread's own few rows (about 7 for a 2M-row system), over the 32 lanes
//     of a warp as a compensated binary32 pair (TwoSum, about 48 bits), and
//     in binary64 across warps and blocks -- GB300's binary64 pipe is narrow,
//     and binary64 conversions and shuffles per thread made these kernels
//     FP64-bound;
//   - alpha and beta are binary64 scalars;
//   - the solution x is binary64: the binary32 corrections alpha * p are
//     summed in a binary32 vector e, which is added to x in binary64 (and
//     cleared) right before every binary64 true residual;
//   - the true residual r = b - A x is recomputed in binary64 with the
//     binary64 matrix ("reliable update" defect correction) whenever the
//     binary32 recursive residual has dropped by the factor delta (0.1) since
//     the last true residual, or claims convergence, or the iteration limit
//     is reached.  The binary32 residual is then replaced by the true one and
//     the search direction is kept, so the Krylov space is not restarted.
// Convergence is declared only on a binary64 true residual, so fin_res and
// r1 on return are b - A x in binary64.
#pragma once
#include "tfs_kernels.cuh"

namespace tfs {

__global__ void k_mx_cast(int n_int, const double *__restrict__ src, float *__restrict__ dst)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_int; i += gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

// Binary64 true residual r = b - A x (b kept in V.u1), copied to the binary32
// residual, with ||r|| and the next rho.  INIT: the first residual of the
// solve (Residual.f90 + Cg.f90:75-90 semantics, b saved first, shadow r2 set).
template <int METHOD, bool INIT>
__global__ void __launch_bounds__(TFS_TPB)
k_mx_true(SellDev A, const double *__restrict__ val, Vec64 V, Vec32 F, DevState *st,
          double *part, int prec, cudaGraphConditionalHandle cond, int l0_rows = 0)
{
    // PDL secondary (a no-op when launched plainly).  No early trigger: a
    // DIC level chain launched after this kernel reads r before its own
    // waits, so it must start only once this kernel has completed.
    cudaGridDependencySynchronize();
    if (st->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(cond, 0u);
        return;
    }
    if (!INIT && !st->need_true) {
        if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(cond, 1u);
        return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) st->t_spmv0 = gtimer();
    const bool fused = (METHOD == 2) || prec != 2;
    double e2 = 0.0, rz = 0.0;
    for (int c = blockIdx.x; c < A.n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        double b;
        if (INIT) { b = V.r[i]; V.u1[i] = b; F.e[i] = 0.f; } else b = V.u1[i];
        RowGeom g = row_geom(A, i);
        double r = row_accum<true, double, double, double, TFS_SPMV_NC>(b, A.col, val, V.x, g.off, 0, g.len);
        V.r[i] = r;
        float r32 = (float)r;
        F.r[i] = r32;
        // DIC level 0 has no lower neighbours: its forward sweep is y = r D,
        // done here (and in k_mx_cg_update4) instead of in a level kernel.
        if (i < l0_rows) F.y[i] = r32 * F.d[i];
        // The shadow residual of the reference's BiCG equals r1 at every step
        // (it starts as r1 and is driven by A, not A^T), so a reliable update
        // resets it together with r1; CGS keeps its initial shadow.
        if (METHOD == 1 || (INIT && METHOD == 2)) F.r2[i] = r32;
        e2 = fma(r, r, e2);
        if (METHOD == 2) rz = fma((double)r32, (double)F.r2[i], rz);
        else if (fused) {
            float d32 = F.d[i], z = r32 / d32;
            F.z[i] = z;
            if (METHOD == 0) rz = fma((double)r32, (double)z, rz);
            else {
                F.z2[i] = z;
                rz = fma((double)z, (double)r32, rz);
            }
        }
    }
    double v[2] = {e2, rz};
    if (grid_reduce<2>(v, part, &st->counter)) {
        double err = sqrt(v[0]);
        st->r_true = err;
        st->true_res += 1;
        st->spmv_ns += gtimer() - st->t_spmv0;
        st->spmv_n += 1;
        if (INIT) {
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
            } else if (st->niter_max <= 0) {
                st->done = 1;
                st->niter_out = 1;
            } else if (fused) {
                st->rho = v[1];
            }
            set_cond(cond, st->done ? 0u : 1u);
        } else {
            st->need_true = 0;
            finish_iteration(st, v[0], v[1], fused, cond);
        }
    }
}

// x += e in binary64 and e = 0, right before a binary64 true residual.
__global__ void __launch_bounds__(TFS_TPB) k_mx_fold(int n_chunks, Vec64 V, Vec32 F, const DevState *st)
{
    if (st->done || !st->need_true) return;
    TFS_QUAD_BEGIN(n_chunks)
        float e[4];
        double x[4];
        TFS_QLOAD(e, F.e); TFS_QLOAD(x, V.x);
        TFS_QUAD_FOR { V.x[_i[_q]] = x[_q] + (double)e[_q]; F.e[_i[_q]] = 0.f; }
    TFS_QUAD_END
}

// End of a binary32 iteration: either finish it on the recursive residual or
// hand over to k_mx_true for a binary64 residual first.
__device__ __forceinline__ void mx_end_iteration(DevState *st, double e2, double rz, bool fused)
{
    double est = sqrt(e2);
    if (!(est <= DBL_MAX) || est < st->tol || est < st->delta * st->r_true ||
        st->iter >= st->niter_max) {
        st->need_true = 1;
        st->error = est;
    } else {
        finish_iteration(st, e2, rz, fused, 0);
    }
}

template <typename T>
__device__ __forceinline__ double dd(T v) { return (double)v; }

// rho = (r, z) / (z1, r2) after binary32 sweeps.
template <int METHOD>
__global__ void __launch_bounds__(TFS_TPB) k_mx_dot_rho(int n_chunks, Vec32 F, DevState *st, double *part)
{
    if (st->done || st->need_true) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->sweep_ns += gtimer() - st->t_sweep0;
        st->sweep_n += 1;
    }
    float acc = 0.f;
    TFS_QUAD_BEGIN(n_chunks)
        float a[4], b[4];
        TFS_QLOAD(a, METHOD == 0 ? F.r : F.z);
        TFS_QLOAD(b, METHOD == 0 ? F.z : F.r2);
        TFS_QUAD_FOR acc = fmaf(a[_q], b[_q], acc);
    TFS_QUAD_END
    const float av[1] = {acc};
    double v[1];
    if (grid_reduce_f<1>(av, v, part, &st->counter)) {
        st->rho = v[0];
        if (st->iter > 1) publish_beta(st);
    }
}

// ---------------------------------------------------------------- CG

template <bool FROMZ>
__global__ void __launch_bounds__(TFS_TPB) k_mx_cg_p(int n_chunks, Vec32 F, const DevState *st)
{
    if (st->done || st->need_true) return;
    const int it = st->iter;
    const float beta = it == 1 ? 0.f : st->beta32;
    TFS_QUAD_BEGIN(n_chunks)
        float z[4], p[4];
        if (FROMZ) { TFS_QLOAD(z, F.z); }
        else { float r[4], d[4]; TFS_QLOAD(r, F.r); TFS_QLOAD(d, F.d); TFS_QUAD_FOR z[_q] = r[_q] / d[_q]; }
        TFS_QLOAD(p, F.p);
        TFS_QUAD_FOR F.p[_i[_q]] = it == 1 ? z[_q] : fmaf(beta, p[_q], z[_q]);
    TFS_QUAD_END
}

// q = A p in binary32 with (p, q) in binary64 and alpha.
__global__ void __launch_bounds__(TFS_TPB)
k_mx_spmv_pq(SellDev A, const float *__restrict__ val, const float *__restrict__ p,
             float *__restrict__ q, DevState *st, double *part)
{
    // The skip flags are tested after the first row's loads are issued (here
    // and in the other per-iteration kernels), so that reading them does not
    // delay those loads.
    const bool stop = (st->done | st->need_true) != 0;
    if (!stop && blockIdx.x == 0 && threadIdx.x == 0) st->t_spmv0 = gtimer();
    float acc = 0.f;
    for (int c = blockIdx.x; c < A.n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        float s = row_spmv<false, float, float, float, TFS_SPMV_NC>(0.f, A, val, p, i);
        if (stop) return;
        q[i] = s;
        acc = fmaf(p[i], s, acc);
    }
    if (stop) return;
    const float a1[1] = {acc};
    double v[1];
    if (grid_reduce_f<1>(a1, v, part, &st->counter)) {
        st->alpha = st->rho / v[0];
        st->alpha32 = (float)st->alpha;
        st->spmv_ns += gtimer() - st->t_spmv0;
        st->spmv_n += 1;
    }
}

template <bool FUSED>
__global__ void __launch_bounds__(TFS_TPB)
k_mx_cg_update(int n_chunks, Vec64 V, Vec32 F, DevState *st, double *part)
{
    if (st->done || st->need_true) return;
    const double alfa = st->alpha;
    const float alfa32 = (float)alfa;
    float e2 = 0.f, rz = 0.f;
    TFS_QUAD_BEGIN(n_chunks)
        float e[4], p[4], r[4], q[4], d[4];
        TFS_QLOAD(e, F.e); TFS_QLOAD(p, F.p); TFS_QLOAD(r, F.r); TFS_QLOAD(q, F.q);
        if (FUSED) { TFS_QLOAD(d, F.d); }
        TFS_QUAD_FOR {
            const int i = _i[_q];
            F.e[i] = fmaf(alfa32, p[_q], e[_q]);
            float rn = fmaf(-alfa32, q[_q], r[_q]);
            F.r[i] = rn;
            e2 = fmaf(rn, rn, e2);
            if (FUSED) { float z = rn / d[_q]; F.z[i] = z; rz = fmaf(rn, z, rz); }
        }
    TFS_QUAD_END
    const float av[2] = {e2, rz};
    double v[2];
    if (grid_reduce_f<2>(av, v, part, &st->counter)) mx_end_iteration(st, v[0], v[1], FUSED);
}

// ---------------------------------------------------- CG, four rows per thread
//
// The binary32 CG vector kernels with 16-byte loads: a thread handles four
// consecutive rows per step (n_int is a multiple of 1024, the vectors are
// 16-byte aligned), grid-stride over the 8-blocks-per-SM grid of the other
// vector kernels.  On the 128^3 system this beat both the scalar four-chunk
// kernels (11.7 against 11.5 solves/s) and one 1024-row block per four-row
// group over the whole vector (11.0 solves/s, more partial sums to reduce).

__global__ void __launch_bounds__(TFS_TPB) k_mx_cg_p4(int n4, Vec32 F, const DevState *st)
{
    // PDL secondary (a no-op when launched plainly): wait for the
    // predecessor before reading anything, then let the successor launch.
    cudaGridDependencySynchronize();
    cudaTriggerProgrammaticLaunchCompletion();
    const bool stop = (st->done | st->need_true) != 0;
    const int it = st->iter;
    const float beta = st->beta32;           // (float)(rho / rho_old), published once
    const float4 *z4 = (const float4 *)F.z;
    float4 *p4 = (float4 *)F.p;
    for (int v = blockIdx.x * TFS_TPB + threadIdx.x; v < n4; v += gridDim.x * TFS_TPB) {
        float4 z = z4[v], p = p4[v];
        if (stop) return;
        if (it == 1) p4[v] = z;
        else p4[v] = make_float4(fmaf(beta, p.x, z.x), fmaf(beta, p.y, z.y), fmaf(beta, p.z, z.z), fmaf(beta, p.w, z.w));
    }
}

__global__ void __launch_bounds__(TFS_TPB) k_mx_dot_rho4(int n4, Vec32 F, DevState *st, double *part)
{
    // PDL secondary (a no-op when launched plainly): wait for the
    // predecessor before reading anything, then let the successor launch.
    cudaGridDependencySynchronize();
    cudaTriggerProgrammaticLaunchCompletion();
    const bool stop = (st->done | st->need_true) != 0;
    const float4 *r4 = (const float4 *)F.r, *z4 = (const float4 *)F.z;
    float acc = 0.f;
    for (int v = blockIdx.x * TFS_TPB + threadIdx.x; v < n4; v += gridDim.x * TFS_TPB) {
        float4 r = r4[v], z = z4[v];
        if (stop) return;
        acc = fmaf(r.x, z.x, acc); acc = fmaf(r.y, z.y, acc); acc = fmaf(r.z, z.z, acc); acc = fmaf(r.w, z.w, acc);
    }
    if (stop) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->sweep_ns += gtimer() - st->t_sweep0;
        st->sweep_n += 1;
    }
    const float a1[1] = {acc};
    double v1[1];
    if (grid_reduce_f<1>(a1, v1, part, &st->counter)) {
        st->rho = v1[0];
        if (st->iter > 1) publish_beta(st);
    }
}

template <bool FUSED>
__global__ void __launch_bounds__(TFS_TPB) k_mx_cg_update4(int n4, Vec32 F, DevState *st, double *part,
                                                           int l0_rows4 = 0)
{
    cudaGridDependencySynchronize();   // PDL secondary, as k_mx_cg_p4
    cudaTriggerProgrammaticLaunchCompletion();
    const bool stop = (st->done | st->need_true) != 0;
    const float a = st->alpha32;             // (float) alpha, published once
    const float4 *p4 = (const float4 *)F.p, *q4 = (const float4 *)F.q, *d4 = (const float4 *)F.d;
    float4 *e4 = (float4 *)F.e, *r4 = (float4 *)F.r, *zz4 = (float4 *)F.z;
    float e2 = 0.f, rz = 0.f;
    for (int v = blockIdx.x * TFS_TPB + threadIdx.x; v < n4; v += gridDim.x * TFS_TPB) {
        float4 p = p4[v], q = q4[v], r = r4[v], e = e4[v], d;
        if (FUSED) d = d4[v];
        if (stop) return;
        e4[v] = make_float4(fmaf(a, p.x, e.x), fmaf(a, p.y, e.y), fmaf(a, p.z, e.z), fmaf(a, p.w, e.w));
        r = make_float4(fmaf(-a, q.x, r.x), fmaf(-a, q.y, r.y), fmaf(-a, q.z, r.z), fmaf(-a, q.w, r.w));
        r4[v] = r;
        if (v < l0_rows4) {   // forward sweep of DIC level 0: y = r D (no lower neighbours)
            const float4 dd = d4[v];
            ((float4 *)F.y)[v] = make_float4(r.x * dd.x, r.y * dd.y, r.z * dd.z, r.w * dd.w);
        }
        e2 = fmaf(r.x, r.x, e2); e2 = fmaf(r.y, r.y, e2); e2 = fmaf(r.z, r.z, e2); e2 = fmaf(r.w, r.w, e2);
        if (FUSED) {
            float4 z = make_float4(r.x / d.x, r.y / d.y, r.z / d.z, r.w / d.w);
            zz4[v] = z;
            rz = fmaf(r.x, z.x, rz); rz = fmaf(r.y, z.y, rz); rz = fmaf(r.z, z.z, rz); rz = fmaf(r.w, z.w, rz);
        }
    }
    if (stop) return;
    const float a2[2] = {e2, rz};
    double v2[2];
    if (grid_reduce_f<2>(a2, v2, part, &st->counter)) mx_end_iteration(st, v2[0], v2[1], FUSED);
}

__global__ void __launch_bounds__(TFS_TPB) k_mx_fold4(int n4, Vec64 V, Vec32 F, const DevState *st)
{
    cudaGridDependencySynchronize();   // PDL secondary, as k_mx_cg_p4
    cudaTriggerProgrammaticLaunchCompletion();
    if (st->done || !st->need_true) return;
    float4 *e4 = (float4 *)F.e;
    double2 *x2 = (double2 *)V.x;
    for (int v = blockIdx.x * TFS_TPB + threadIdx.x; v < n4; v += gridDim.x * TFS_TPB) {
        float4 e = e4[v];
        double2 xa = x2[2 * v], xb = x2[2 * v + 1];
        xa.x += (double)e.x; xa.y += (double)e.y; xb.x += (double)e.z; xb.y += (double)e.w;
        x2[2 * v] = xa;
        x2[2 * v + 1] = xb;
        e4[v] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// The last kernel of the DIC application of CG: the backward sweep of
// level 0 (rows [0, l0_rows), as k_sweep_level) fused with rho = (r, z) over
// all rows (the job of k_dot_rho / k_mx_dot_rho4): a thread adds r_i z_i of
// its own level-0 row from the value it just computed, and of the rows above
// level 0 (final since the earlier level kernels) over a grid-stride loop.
// Binary32 (T = float, compensated warp sums) or binary64 (fma partials).
template <typename T>
__global__ void __launch_bounds__(TFS_TPB)
k_sweep0_rho(SellDev A, const T *__restrict__ val, const T *d, const T *r, T *z, const T *y, int l0_rows,
             int n_int, DevState *st, double *part)
{
    const int i = blockIdx.x * TFS_TPB + threadIdx.x;
    const bool active = i < l0_rows;
    RowGeom g{0, 0, 0};
    int kk[TFS_BWD_PRE_SLOTS] = {};
    T aa[TFS_BWD_PRE_SLOTS] = {};
    if (active) {
        g = row_geom(A, i);
#pragma unroll
        for (int q = 0; q < TFS_BWD_SLOTS(T); q++)
            if (g.dpos + 1 + q < g.len) {
                const int ee = g.off + ((g.dpos + 1 + q) << 5);
                kk[q] = __ldg(A.col + ee);
                aa[q] = __ldg(val + ee);
            }
    }
    // Level 0's forward values and r come from kernels that completed before
    // the sweep's first level kernel started: the row's start value
    // y_i / (D_i + TINY) and r_i are ready before the wait.
    T di = (T)0, s0 = (T)0, ri = (T)0;
    if (active && g.len > 0) {
        di = d[i];
        s0 = y[i] / (di + (T)TINY);
        ri = r[i];
    }
    cudaTriggerProgrammaticLaunchCompletion();
    cudaGridDependencySynchronize();
    const bool stop = (st->done | st->need_true) != 0;
    T acc = (T)0;
    if (active) {
        if (g.len == 0) {
            if (!stop) z[i] = (T)0;   // padding row: r_i z_i adds (r_i = 0) * 0
            if (!stop) {
                if constexpr (sizeof(T) == 4) acc = fmaf(r[i], (T)0, acc);
                else acc = fma(r[i], (T)0, acc);
            }
        } else {
            // the prefetched entries' gathers all issued before the first
            // update (as in the level kernels' row routines)
            T sv = s0;
            const int j0 = g.dpos + 1;
            constexpr int NP = TFS_BWD_SLOTS(T);
            T xz[NP];
#pragma unroll
            for (int q = 0; q < NP; q++) {
                xz[q] = (T)0;
                if (j0 + q < g.len) xz[q] = __ldcg(z + kk[q]);
            }
#pragma unroll
            for (int q = 0; q < NP; q++)
                if (j0 + q < g.len) sv = sv - aa[q] * xz[q];
            int j = j0 + NP < g.len ? j0 + NP : g.len;
            for (; j < g.len; j++) {
                const int ee = g.off + (j << 5);
                sv = sv - __ldg(val + ee) * __ldcg(z + __ldg(A.col + ee));
            }
            const T zi = sv * di;
            if (!stop) {
                z[i] = zi;
                if constexpr (sizeof(T) == 4) acc = fmaf(ri, zi, acc);
                else acc = fma(ri, zi, acc);
            }
        }
    }
    for (int k = l0_rows + blockIdx.x * TFS_TPB + threadIdx.x; k < n_int; k += gridDim.x * TFS_TPB) {
        if constexpr (sizeof(T) == 4) acc = fmaf(r[k], __ldcg(z + k), acc);
        else acc = fma(r[k], __ldcg(z + k), acc);
    }
    if (stop) return;
    double v[1];
    bool last;
    if constexpr (sizeof(T) == 4) {
        const float av[1] = {acc};
        last = grid_reduce_f<1>(av, v, part, &st->counter);
    } else {
        v[0] = acc;
        last = grid_reduce<1>(v, part, &st->counter);
    }
    if (last) {
        st->rho = v[0];
        if (st->iter > 1) publish_beta(st);
        st->sweep_ns += gtimer() - st->t_sweep0;
        st->sweep_n += 1;
    }
}

// -------------------------------------------------------------- BiCG

template <bool FROMZ>
__global__ void __launch_bounds__(TFS_TPB) k_mx_bicg_p(int n_chunks, Vec32 F, const DevState *st)
{
    if (st->done || st->need_true) return;
    const int it = st->iter;
    const float beta = it == 1 ? 0.f : st->beta32;
    TFS_QUAD_BEGIN(n_chunks)
        float z1[4], z2[4], p1[4], p2[4];
        if (FROMZ) { TFS_QLOAD(z1, F.z); TFS_QLOAD(z2, F.z2); }
        else {
            float r1[4], r2[4], d[4];
            TFS_QLOAD(r1, F.r); TFS_QLOAD(r2, F.r2); TFS_QLOAD(d, F.d);
            TFS_QUAD_FOR { z1[_q] = r1[_q] / d[_q]; z2[_q] = r2[_q] / d[_q]; }
        }
        TFS_QLOAD(p1, F.p); TFS_QLOAD(p2, F.p2);
        TFS_QUAD_FOR {
            const int i = _i[_q];
            if (it == 1) { F.p[i] = z1[_q]; F.p2[i] = z2[_q]; }
            else { F.p[i] = fmaf(beta, p1[_q], z1[_q]); F.p2[i] = fmaf(beta, p2[_q], z2[_q]); }
        }
    TFS_QUAD_END
}

__global__ void __launch_bounds__(TFS_TPB)
k_mx_spmv2_pq(SellDev A, const float *__restrict__ val, Vec32 F, DevState *st, double *part)
{
    if (st->done || st->need_true) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->t_spmv0 = gtimer();
    float acc = 0.f;
    for (int c = blockIdx.x; c < A.n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        RowGeom g = row_geom(A, i);
        float s1 = 0.f, s2 = 0.f;
        row_accum2<false, float, float, float, TFS_SPMV_NC>(s1, s2, A.col, val, F.p, F.p2, g.off, 0, g.len);
        F.q[i] = s1;
        F.q2[i] = s2;
        acc = fmaf(F.p2[i], s1, acc);
    }
    const float av[1] = {acc};
    double v[1];
    if (grid_reduce_f<1>(av, v, part, &st->counter)) {
        st->alpha = st->rho / v[0];
        st->alpha32 = (float)st->alpha;
        st->spmv_ns += gtimer() - st->t_spmv0;
        st->spmv_n += 1;
    }
}

template <bool FUSED>
__global__ void __launch_bounds__(TFS_TPB)
k_mx_bicg_update(int n_chunks, Vec64 V, Vec32 F, DevState *st, double *part)
{
    if (st->done || st->need_true) return;
    const double alfa = st->alpha;
    const float alfa32 = (float)alfa;
    float e2 = 0.f, rz = 0.f;
    TFS_QUAD_BEGIN(n_chunks)
        float e[4], p[4], r1[4], q1[4], r2[4], q2[4], d[4];
        TFS_QLOAD(e, F.e); TFS_QLOAD(p, F.p); TFS_QLOAD(r1, F.r); TFS_QLOAD(q1, F.q);
        TFS_QLOAD(r2, F.r2); TFS_QLOAD(q2, F.q2);
        if (FUSED) { TFS_QLOAD(d, F.d); }
        TFS_QUAD_FOR {
            const int i = _i[_q];
            F.e[i] = fmaf(alfa32, p[_q], e[_q]);
            float a1 = fmaf(-alfa32, q1[_q], r1[_q]);
            float a2 = fmaf(-alfa32, q2[_q], r2[_q]);
            F.r[i] = a1;
            F.r2[i] = a2;
            e2 = fmaf(a1, a1, e2);
            if (FUSED) {
                float z1 = a1 / d[_q];
                F.z[i] = z1;
                F.z2[i] = a2 / d[_q];
                rz = fmaf(z1, a2, rz);
            }
        }
    TFS_QUAD_END
    const float av[2] = {e2, rz};
    double v[2];
    if (grid_reduce_f<2>(av, v, part, &st->counter)) mx_end_iteration(st, v[0], v[1], FUSED);
}

// --------------------------------------------------------------- CGS

template <bool FUSEDP>
__global__ void __launch_bounds__(TFS_TPB) k_mx_cgs_u(int n_chunks, Vec32 F, const DevState *st)
{
    if (st->done || st->need_true) return;
    const int it = st->iter;
    const float beta = it == 1 ? 0.f : st->beta32;
    for (int c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        float u1, u2;
        if (it == 1) { u1 = F.r[i]; u2 = u1; }
        else {
            float q1 = F.q[i];
            u1 = F.r[i] + beta * q1;
            u2 = u1 + beta * (q1 + beta * F.u2[i]);
        }
        F.u1[i] = u1;
        F.u2[i] = u2;
        if (FUSEDP) F.p2[i] = u2 / F.d[i];
    }
}

__global__ void __launch_bounds__(TFS_TPB)
k_mx_spmv_v(SellDev A, const float *__restrict__ val, Vec32 F, DevState *st, double *part)
{
    if (st->done || st->need_true) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->t_spmv0 = gtimer();
    float acc = 0.f;
    for (int c = blockIdx.x; c < A.n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        RowGeom g = row_geom(A, i);
        float s = row_accum<false, float, float, float, TFS_SPMV_NC>(0.f, A.col, val, F.p2, g.off, 0, g.len);
        F.v2[i] = s;
        acc = fmaf(F.r2[i], s, acc);
    }
    const float av[1] = {acc};
    double v[1];
    if (grid_reduce_f<1>(av, v, part, &st->counter)) {
        st->alpha = st->rho / v[0];
        st->alpha32 = (float)st->alpha;
        st->spmv_ns += gtimer() - st->t_spmv0;
        st->spmv_n += 1;
    }
}

template <bool FUSEDP>
__global__ void __launch_bounds__(TFS_TPB) k_mx_cgs_q(int n_chunks, Vec32 F, const DevState *st)
{
    if (st->done || st->need_true) return;
    const float alfa32 = (float)st->alpha;
    for (int c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        float u1 = F.u1[i];
        float q1 = u1 - alfa32 * F.v2[i];
        F.q[i] = q1;
        float w = u1 + q1;
        if (FUSEDP) F.p[i] = w / F.d[i];
        else F.w[i] = w;
    }
}

__global__ void __launch_bounds__(TFS_TPB)
k_mx_cgs_spmv_r(SellDev A, const float *__restrict__ val, Vec64 V, Vec32 F, DevState *st,
                double *part)
{
    if (st->done || st->need_true) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->t_spmv0 = gtimer();
    const double alfa = st->alpha;
    const float alfa32 = (float)alfa;
    float e2 = 0.f, rr = 0.f;
    for (int c = blockIdx.x; c < A.n_chunks; c += gridDim.x) {
        int i = c * TFS_TPB + threadIdx.x;
        F.e[i] = fmaf(alfa32, F.p[i], F.e[i]);
        RowGeom g = row_geom(A, i);
        float q2 = row_accum<false, float, float, float, TFS_SPMV_NC>(0.f, A.col, val, F.p, g.off, 0, g.len);
        float r1 = fmaf(-alfa32, q2, F.r[i]);
        F.r[i] = r1;
        e2 = fmaf(r1, r1, e2);
        rr = fmaf(r1, F.r2[i], rr);
    }
    const float av[2] = {e2, rr};
    double v[2];
    if (grid_reduce_f<2>(av, v, part, &st->counter)) {
        st->spmv_ns += gtimer() - st->t_spmv0;
        st->spmv_n += 1;
        mx_end_iteration(st, v[0], v[1], true);
    }
}

}  // namespace tfs
