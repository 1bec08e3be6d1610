// tfs_batch.cuh -- many independent systems in one persistent launch.
//
// Each system of a batch is solved, start to finish, by one thread-block
// cluster (C CTAs on C SMs, 2 <= C <= 16).  Clusters take systems from a
// queue sorted by decreasing size (longest first), so a batch of uneven
// systems packs onto the GPU and small systems fill the gaps left by large
// ones.  Inside a cluster every synchronisation is the hardware cluster
// barrier, and every reduction sums one partial per CTA through distributed
// shared memory in CTA-rank order: there are no spin-waits, and a system's
// result depends only on (C, threads per CTA), never on which cluster ran it
// or on what else was in the batch -- a system gives bitwise the same result
// alone and in any mix.
//
// Methods: CG and BiCG (A, not A^T, on the shadow system) with no or diagonal
// preconditioning, and CG (hence the reference's BiCG, whose iterates are
// CG's) with DIC preconditioning: the factor (Prec_Form.f90:32-40) and both
// triangular sweeps (Prec_Solve.f90:46-67) run level by level over the
// system's DIC level schedule, the cluster's threads sharing each level's
// rows and the cluster barrier between levels; every row keeps the
// reference's arithmetic.  Binary64 (the reference's per-row arithmetic) or
// mixed precision (binary32 iteration, binary64 reliable updates, as
// tfs_mixed.cuh; the factor formed in binary64 and rounded once).
#pragma once
#include <cooperative_groups.h>

#include "tfs_kernels.cuh"

namespace tfs {

namespace cg = cooperative_groups;

// One system of a batch (device memory, written by the host per solve).
struct BatchSys {
    SellDev A;
    const double *val;        // SELL binary64 values (gathered by the kernel)
    float *val32;             // SELL binary32 values (mixed)
    const int *vmap;          // SELL -> CSR position
    int nnz_pad;
    const int *perm;          // internal -> natural row
    Vec64 V;
    Vec32 F;
    const double *val_csr;    // caller's CSR values (natural order)
    const double *b;          // caller's right-hand side (natural order)
    double *x;                // caller's x (natural order, in/out)
    double *r_out;            // r1 on return (natural order)
    double tol;
    int niter_max;
    int prec;
    const int *lvl_begin;     // DIC level schedule (prec 2): first row of every level, n_levels + 1
    int n_levels;
    // outputs
    int niter_out, status, early, true_res;
    double ini_res, fin_res;
};

struct BatchCtl {
    unsigned int head;        // next queue position
    unsigned int pad;
};

#define TFS_BATCH_MAX_TPB 512
// Resident CTAs of 512 threads per SM the kernel is compiled for (at most
// 65536 / (512 * 3) = 42 registers, with some spilling).  Measured on the
// 256-system batch (mixed, best cluster shape each): 1 -> 422, 2 -> 499,
// 3 -> 584, 4 -> 545 solves/s; the latency-bound solves gain more from
// resident warps than they lose to the spills.
#ifndef TFS_BATCH_MIN_BLOCKS
#define TFS_BATCH_MIN_BLOCKS 3
#endif

// Sum of NV values over the cluster: block sum, one partial per CTA in
// shared memory, cluster barrier, every thread adds the C partials in rank
// order.  Two partial slots alternate, so a slot is rewritten only after the
// next barrier, by which time every reader of its previous contents is done.
//
// AT is the type of the per-thread partials: binary64, or binary32 in the
// mixed solves, whose warp sums then go through warp_sum_f (compensated
// binary32, no binary64 instruction per lane).
template <int NV, typename AT = double>
__device__ __forceinline__ void cluster_sum(const AT (&in)[NV], double (&v)[NV], double (*s_part)[4],
                                            int &parity, cg::cluster_group &cl)
{
    __shared__ double sm[NV][TFS_BATCH_MAX_TPB / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double w;
        if constexpr (sizeof(AT) == 4) {
            w = warp_sum_f(in[k]);
        } else {
            w = in[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) w = w + __shfl_down_sync(FULL, w, o);
        }
        if (lane == 0) sm[k][warp] = w;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = sm[k][0];
            for (int w = 1; w < nw; w++) s = s + sm[k][w];
            s_part[parity][k] = s;
        }
    }
    cl.sync();
    const unsigned C = cl.num_blocks();
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double s = 0.0;
        for (unsigned r = 0; r < C; r++) {
            double(*rp)[4] = cl.map_shared_rank(s_part, r);
            s = s + rp[parity][k];
        }
        v[k] = s;
    }
    parity ^= 1;
}

template <typename VT>
struct BatchVecs;
template <>
struct BatchVecs<double> {
    double *r, *r2, *p, *p2, *q, *q2, *z, *z2;
    __device__ BatchVecs(const BatchSys &S)
        : r(S.V.r), r2(S.V.r2), p(S.V.p), p2(S.V.p2), q(S.V.q), q2(S.V.q2), z(S.V.z), z2(S.V.z2) {}
};
template <>
struct BatchVecs<float> {
    float *r, *r2, *p, *p2, *q, *q2, *z, *z2;
    __device__ BatchVecs(const BatchSys &S)
        : r(S.F.r), r2(S.F.r2), p(S.F.p), p2(S.F.p2), q(S.F.q), q2(S.F.q2), z(S.F.z), z2(S.F.z2) {}
};

// The whole solve of one system by the calling cluster.  VT = double:
// binary64 with the reference's per-row arithmetic; VT = float: mixed.
// Per-thread dot-product partial: binary64 fma in the binary64 solves (the
// values are binary64 already), binary32 fmaf in the mixed ones.
template <typename AccT, typename VT>
__device__ __forceinline__ AccT acc_fma(VT a, VT b, AccT c)
{
    if constexpr (sizeof(AccT) == 4) return fmaf((float)a, (float)b, c);
    else return fma((double)a, (double)b, c);
}

// DIC factor of one system (binary64, Prec_Form.f90:32-40): levels
// ascending, the cluster's threads sharing each level's rows, the cluster
// barrier between levels (its release/acquire makes every CTA's stores
// visible; gathers read past L1).
__device__ void batch_dic_form(const SellDev &A, const double *val, double *d, const int *lvl_begin, int nl,
                               int gtid, int stride, cg::cluster_group &cl)
{
    for (int l = 0; l < nl; l++) {
        const int r1 = __ldg(lvl_begin + l + 1);
        for (int i = __ldg(lvl_begin + l) + gtid; i < r1; i += stride) {
            const RowGeom g = row_geom(A, i);
            if (g.len == 0) { d[i] = 1.0; continue; }
            double s = __ldg(val + g.off + (g.dpos << 5));
            for (int j = 0; j < g.dpos; j++) {
                const int ee = g.off + (j << 5);
                const double a = __ldg(val + ee);
                s = s - __ldcg(d + __ldg(A.col + ee)) * a * a;
            }
            d[i] = 1.0 / s;
        }
        cl.sync();
    }
}

// z = M^-1 r with the DIC factor d (Prec_Solve.f90:46-67): forward sweep
// into y, levels ascending, then y / (D + TINY) and the backward sweep into
// z, levels descending; returns the thread's partial of (r, z).  r must be
// complete (a cluster barrier after its stores).
template <typename VT, typename AccT>
__device__ AccT batch_dic_apply(const SellDev &A, const VT *val, const VT *d, const VT *r, VT *y, VT *z,
                                const int *lvl_begin, int nl, int gtid, int stride, cg::cluster_group &cl)
{
    for (int l = 0; l < nl; l++) {
        const int r1 = __ldg(lvl_begin + l + 1);
        for (int i = __ldg(lvl_begin + l) + gtid; i < r1; i += stride) {
            const RowGeom g = row_geom(A, i);
            if (g.len == 0) { y[i] = (VT)0; continue; }
            VT s = __ldcg(r + i);
            for (int j = 0; j < g.dpos; j++) {
                const int ee = g.off + (j << 5);
                s = s - __ldg(val + ee) * __ldcg(y + __ldg(A.col + ee));
            }
            y[i] = s * __ldcg(d + i);
        }
        cl.sync();
    }
    AccT rz = (AccT)0;
    for (int l = nl - 1; l >= 0; l--) {
        const int r1 = __ldg(lvl_begin + l + 1);
        for (int i = __ldg(lvl_begin + l) + gtid; i < r1; i += stride) {
            const RowGeom g = row_geom(A, i);
            if (g.len == 0) { z[i] = (VT)0; continue; }
            const VT di = __ldcg(d + i);
            VT s = __ldcg(y + i) / (di + (VT)TINY);
            for (int j = g.dpos + 1; j < g.len; j++) {
                const int ee = g.off + (j << 5);
                s = s - __ldg(val + ee) * __ldcg(z + __ldg(A.col + ee));
            }
            const VT zi = s * di;
            z[i] = zi;
            if constexpr (sizeof(AccT) == 4) rz = fmaf((float)__ldcg(r + i), (float)zi, rz);
            else rz = fma((double)__ldcg(r + i), (double)zi, rz);
        }
        cl.sync();
    }
    return rz;
}

template <int METHOD, typename VT>
__device__ void batch_solve_one(BatchSys &S, cg::cluster_group &cl, double (*s_part)[4], int &parity)
{
    constexpr bool MIXED = sizeof(VT) == 4;
    using AccT = VT;
    const int C = (int)cl.num_blocks();
    const int stride = C * (int)blockDim.x;
    const int gtid = (int)cl.block_rank() * (int)blockDim.x + (int)threadIdx.x;
    const SellDev A = S.A;
    const int n_int = A.n_int;
    const Vec64 V = S.V;
    const Vec32 F = S.F;
    BatchVecs<VT> W(S);
    const VT *valT;
    if constexpr (MIXED) valT = S.val32; else valT = S.val;
    const double tol = S.tol;
    const int niter_max = S.niter_max;
    const bool diag = S.prec == 1;
    // METHOD 2: the CG sequence with DIC preconditioning (its own instance,
    // so that the DIC sweeps add no registers to the other kernels)
    constexpr bool dic = METHOD == 2;
    VT *yT;
    if constexpr (MIXED) yT = F.y; else yT = V.y;

    // b, x0 in internal order, d, ||b|| (Cg.f90:48-58).  The values were
    // gathered into SELL order by k_batch_gather before this launch.
    double acc[2] = {0.0, 0.0};
    for (int i = gtid; i < n_int; i += stride) {
        int o = __ldg(S.perm + i);
        double bi = 0.0, xi = 0.0;
        if (o >= 0) { bi = S.b[o]; xi = S.x[o]; }
        V.r[i] = bi;
        V.u1[i] = bi;
        V.x[i] = xi;
        acc[0] = fma(bi, bi, acc[0]);
    }
    for (int i = gtid; i < n_int; i += stride) {
        RowGeom g = row_geom(A, i);
        double di = (diag && g.len > 0) ? S.val[g.off + (g.dpos << 5)] : 1.0;
        V.d[i] = di;
        if (MIXED) { F.d[i] = (float)di; F.e[i] = 0.f; }
    }
    if (dic) {
        cl.sync();
        batch_dic_form(A, S.val, V.d, S.lvl_begin, S.n_levels, gtid, stride, cl);
        if (MIXED)
            for (int i = gtid; i < n_int; i += stride) F.d[i] = (float)__ldcg(V.d + i);
    }
    {
        const double a1[1] = {acc[0]};
        double v1[1];
        cluster_sum<1>(a1, v1, s_part, parity, cl);
        double bnrm2 = sqrt(v1[0]);
        if (bnrm2 < tol) {
            // Early exit 1: x, r1 untouched, ini_res untouched (Cg.f90:55-58).
            if (cl.block_rank() == 0 && threadIdx.x == 0) {
                S.niter_out = 0; S.early = 1; S.fin_res = bnrm2; S.status = TFS_OK; S.true_res = 0;
            }
            return;
        }
    }
    // True residual r = b - A x; r2 = r (shadow); z = M^-1 r; ||r0||; rho.
    auto true_residual = [&](bool init, double &e2, double &rz) {
        e2 = 0.0;
        rz = 0.0;
        for (int i = gtid; i < n_int; i += stride) {
            RowGeom g = row_geom(A, i);
            double r = row_accum<true, double, double, double, false, 4>(V.u1[i], A.col, S.val, V.x, g.off, 0, g.len);
            V.r[i] = r;
            e2 = fma(r, r, e2);
            VT rT = (VT)r;
            if (MIXED) W.r[i] = rT;
            if (dic) continue;   // z and (r, z) from the sweeps below
            VT dT = MIXED ? (VT)F.d[i] : (VT)V.d[i];
            VT z = rT / dT;
            W.z[i] = z;
            if (METHOD == 1) {
                // The shadow residual equals r1 (see k_mx_true): reset both.
                W.r2[i] = rT;
                W.z2[i] = z;
                rz = fma((double)z, (double)rT, rz);
            } else {
                rz = fma((double)rT, (double)z, rz);
            }
        }
    };
    double e2, rz;
    true_residual(true, e2, rz);
    if (dic) {
        cl.sync();
        rz = (double)batch_dic_apply<VT, double>(A, valT, MIXED ? (const VT *)F.d : (const VT *)V.d, W.r, yT, W.z,
                                                 S.lvl_begin, S.n_levels, gtid, stride, cl);
    }
    const double a2[2] = {e2, rz};
    double v2[2];
    cluster_sum<2>(a2, v2, s_part, parity, cl);
    double err = sqrt(v2[0]);
    double ini = err, rho = v2[1], rho_old = 0.0, r_true = err;
    int true_res = 1, status = TFS_OK, niter_out = 0, early = 0;
    int iter = 1;
    bool done = false;
    if (!(err <= DBL_MAX)) { status = TFS_ERR_NONFINITE; niter_out = (niter_max > 0 ? niter_max : 0) + 1; done = true; }
    else if (err < tol) { niter_out = 0; early = 2; done = true; }
    else if (niter_max <= 0) { niter_out = 1; done = true; }

    while (!done) {
        // p = z + beta p (Cg.f90:114-123; both directions for BiCG).
        const double beta = iter == 1 ? 0.0 : rho / rho_old;
        const VT betaT = (VT)beta;
        for (int i0 = gtid; i0 < n_int; i0 += 2 * stride) {
            const int i1 = i0 + stride;
            const bool ok1 = i1 < n_int;
            // z past L1: with DIC other threads of the cluster wrote it
            VT z0 = __ldcg(W.z + i0), p0 = W.p[i0], z1 = ok1 ? __ldcg(W.z + i1) : (VT)0,
               p1 = ok1 ? W.p[i1] : (VT)0;
            VT a0 = (VT)0, b0 = (VT)0, a1 = (VT)0, b1 = (VT)0;
            if (METHOD == 1) {
                a0 = W.z2[i0]; b0 = W.p2[i0];
                if (ok1) { a1 = W.z2[i1]; b1 = W.p2[i1]; }
            }
            W.p[i0] = iter == 1 ? z0 : z0 + betaT * p0;
            if (METHOD == 1) W.p2[i0] = iter == 1 ? a0 : a0 + betaT * b0;
            if (ok1) {
                W.p[i1] = iter == 1 ? z1 : z1 + betaT * p1;
                if (METHOD == 1) W.p2[i1] = iter == 1 ? a1 : a1 + betaT * b1;
            }
        }
        cl.sync();
        // q = A p and alpha (Cg.f90:128-153 / Bicg.f90:136-165).
        AccT pq = (AccT)0;
        if (METHOD == 1) {
            for (int i = gtid; i < n_int; i += stride) {
                RowGeom g = row_geom(A, i);
                VT s1 = (VT)0, s2 = (VT)0;
                row_accum2<false, VT, VT, VT>(s1, s2, A.col, valT, W.p, W.p2, g.off, 0, g.len);
                W.q[i] = s1;
                W.q2[i] = s2;
                pq = acc_fma(W.p2[i], s1, pq);
            }
        } else {
            // Four rows per thread and step, all loads before any store.
            for (int i0 = gtid; i0 < n_int; i0 += 4 * stride) {
                int ii[4];
                VT sv[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    ii[q] = i0 + q * stride;
                    sv[q] = (VT)0;
                    if (ii[q] < n_int) {
                        RowGeom g = row_geom(A, ii[q]);
                        sv[q] = row_accum<false, VT, VT, VT, false, 4>((VT)0, A.col, valT, W.p, g.off, 0, g.len);
                    }
                }
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (ii[q] < n_int) {
                        W.q[ii[q]] = sv[q];
                        pq = acc_fma(W.p[ii[q]], sv[q], pq);
                    }
            }
        }
        const AccT a1[1] = {pq};
        double v1[1];
        cluster_sum<1, AccT>(a1, v1, s_part, parity, cl);
        const double alfa = rho / v1[0];
        const VT alfaT = (VT)alfa;
        // x (or e) += alpha p, r -= alpha q, z = M^-1 r, ||r||, next rho.
        AccT e2a = (AccT)0, rza = (AccT)0;
        if (METHOD == 1) {
            for (int i = gtid; i < n_int; i += stride) {
                if (MIXED) F.e[i] = fmaf((float)alfaT, (float)W.p[i], F.e[i]);
                else V.x[i] = V.x[i] + alfa * (double)W.p[i];
                VT r1 = W.r[i] - alfaT * W.q[i];
                W.r[i] = r1;
                VT dT = MIXED ? (VT)F.d[i] : (VT)V.d[i];
                VT z1 = r1 / dT;
                W.z[i] = z1;
                e2a = acc_fma(r1, r1, e2a);
                VT r2 = W.r2[i] - alfaT * W.q2[i];
                W.r2[i] = r2;
                W.z2[i] = r2 / dT;
                rza = acc_fma(z1, r2, rza);
            }
        } else {
            for (int i0 = gtid; i0 < n_int; i0 += 4 * stride) {
                int ii[4];
                VT pv[4], rv[4], qv[4], dv[4];
                double xv[4];
                float ev[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    ii[q] = i0 + q * stride;
                    const int i = ii[q] < n_int ? ii[q] : i0;
                    pv[q] = W.p[i]; rv[q] = W.r[i]; qv[q] = W.q[i];
                    dv[q] = MIXED ? (VT)F.d[i] : (VT)V.d[i];
                    if (MIXED) ev[q] = F.e[i]; else xv[q] = V.x[i];
                }
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    if (ii[q] >= n_int) continue;
                    const int i = ii[q];
                    if (MIXED) F.e[i] = fmaf((float)alfaT, (float)pv[q], ev[q]);
                    else V.x[i] = xv[q] + alfa * (double)pv[q];
                    VT r1 = rv[q] - alfaT * qv[q];
                    W.r[i] = r1;
                    e2a = acc_fma(r1, r1, e2a);
                    if (dic) continue;
                    VT z1 = r1 / dv[q];
                    W.z[i] = z1;
                    rza = acc_fma(r1, z1, rza);
                }
            }
        }
        if (dic) {
            cl.sync();
            rza = batch_dic_apply<VT, AccT>(A, valT, MIXED ? (const VT *)F.d : (const VT *)V.d, W.r, yT, W.z,
                                            S.lvl_begin, S.n_levels, gtid, stride, cl);
        }
        const AccT a3[2] = {e2a, rza};
        double v3[2];
        cluster_sum<2, AccT>(a3, v3, s_part, parity, cl);
        double est = sqrt(v3[0]);
        double rho_next = v3[1];
        bool need_true = MIXED && (!(est <= DBL_MAX) || est < tol || est < 0.1 * r_true || iter >= niter_max);
        if (need_true) {
            for (int i = gtid; i < n_int; i += stride) {
                V.x[i] = V.x[i] + (double)F.e[i];
                F.e[i] = 0.f;
            }
            cl.sync();
            true_residual(false, e2, rz);
            if (dic) {
                cl.sync();
                rz = (double)batch_dic_apply<VT, double>(A, valT, MIXED ? (const VT *)F.d : (const VT *)V.d, W.r,
                                                         yT, W.z, S.lvl_begin, S.n_levels, gtid, stride, cl);
            }
            const double a4[2] = {e2, rz};
            double v4[2];
            cluster_sum<2>(a4, v4, s_part, parity, cl);
            est = sqrt(v4[0]);
            rho_next = v4[1];
            r_true = est;
            true_res++;
        }
        err = est;
        if (!(err <= DBL_MAX)) { status = TFS_ERR_NONFINITE; niter_out = (niter_max > 0 ? niter_max : 0) + 1; done = true; }
        else if (err < tol) { niter_out = iter; done = true; }
        else if (iter >= niter_max) { niter_out = iter + 1; done = true; }
        else { iter++; rho_old = rho; rho = rho_next; }
    }
    cl.sync();
    // x and r1 back to natural order.
    for (int i = gtid; i < n_int; i += stride) {
        int o = __ldg(S.perm + i);
        if (o >= 0) { S.x[o] = V.x[i]; S.r_out[o] = V.r[i]; }
    }
    if (cl.block_rank() == 0 && threadIdx.x == 0) {
        S.niter_out = niter_out; S.status = status; S.early = early; S.true_res = true_res;
        S.ini_res = ini; S.fin_res = err;
    }
}

// SELL values of every system from the callers' CSR values (blockIdx.y =
// system), and the queue head reset for the launch that follows.
__global__ void k_batch_gather(BatchSys *sys, BatchCtl *ctl, int mixed)
{
    const BatchSys &S = sys[blockIdx.y];
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) ctl->head = 0u;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < S.nnz_pad; e += gridDim.x * blockDim.x) {
        int m = __ldg(S.vmap + e);
        double v = m >= 0 ? S.val_csr[m] : 0.0;
        ((double *)S.val)[e] = v;
        if (mixed) S.val32[e] = (float)v;
    }
}

template <int METHOD, typename VT>
__global__ void __launch_bounds__(TFS_BATCH_MAX_TPB, TFS_BATCH_MIN_BLOCKS)
k_batch(BatchSys *sys, const int *order, int n_sys, BatchCtl *ctl)
{
    cg::cluster_group cl = cg::this_cluster();
    __shared__ double s_part[2][4];
    __shared__ int s_sys;
    int parity = 0;
    for (;;) {
        if (cl.block_rank() == 0 && threadIdx.x == 0) s_sys = (int)atomicAdd(&ctl->head, 1u);
        cl.sync();
        const int q = *cl.map_shared_rank(&s_sys, 0);
        cl.sync();   // every CTA has read rank 0's s_sys before it changes
        if (q >= n_sys) break;
        batch_solve_one<METHOD, VT>(sys[order[q]], cl, s_part, parity);
        cl.sync();
    }
}

}  // namespace tfs
