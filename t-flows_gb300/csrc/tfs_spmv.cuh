// tfs_spmv.cuh -- q = A p fused with (p, q) and alpha (Cg.f90:128-153) for
// uniform-width SELL-32 matrices (every slice W <= 8 slots wide: the
// 7-entry rows of a hex mesh).
//
// The direct kernels (k_spmv_pq, k_mx_spmv_pq) walk a dependent chain per
// row -- row geometry, then the column indices and values in passes of four,
// then the gathers of p -- five memory round trips per row, one row after
// the other, so they wait on load latency with no unit of the SM busy.
// k_spmv_pq_pipe keeps the direct kernels' rows, per-thread order of the
// dot-product terms and block and grid reductions (so bitwise the same q,
// (p, q) and alpha) and is software-pipelined in registers: while the
// gathers and values of the current row are in flight, the column indices
// and geometry of the thread's next row are loaded, so a row costs one round
// trip.  Staging the matrix stream in shared memory instead (cp.async.bulk
// with mbarrier completion from one thread, or 16-byte cp.async from every
// thread, 2-4 stages) measured slower on the 128^3 system (binary32 37-48
// against 35.7 us, binary64 104-129 against 74.6 us): the stages cap the
// resident blocks at 3-4 per SM and every chunk ends in a barrier, while the
// matrix stream is not the bound.
#pragma once
#include "tfs_kernels.cuh"

namespace tfs {

#ifndef TFS_SPMV_NOALLOC
#define TFS_SPMV_NOALLOC 1
#endif
// Read-once matrix stream (values, column indices, geometry) loaded without
// allocating in L1, so that L1 holds the gathered p: binary32 SpMV 31.2
// against 32.8 us on the 128^3 system (binary64 unchanged, 73.8 us).
__device__ __forceinline__ int ld_stream(const int *a)
{
    int v;
    if (TFS_SPMV_NOALLOC) asm("ld.global.nc.L1::no_allocate.b32 %0, [%1];" : "=r"(v) : "l"(a));
    else v = __ldg(a);
    return v;
}
__device__ __forceinline__ uint32_t ld_stream(const uint32_t *a)
{
    uint32_t v;
    if (TFS_SPMV_NOALLOC) asm("ld.global.nc.L1::no_allocate.b32 %0, [%1];" : "=r"(v) : "l"(a));
    else v = __ldg(a);
    return v;
}
__device__ __forceinline__ float ld_stream(const float *a)
{
    float v;
    if (TFS_SPMV_NOALLOC) asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(a));
    else v = __ldg(a);
    return v;
}
__device__ __forceinline__ double ld_stream(const double *a)
{
    double v;
    if (TFS_SPMV_NOALLOC) asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(a));
    else v = __ldg(a);
    return v;
}

__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }

// q = A p; (p, q); alpha, software-pipelined over the thread's rows c *
// 256 + tid, c = blockIdx.x, blockIdx.x + gridDim.x, ... (the direct
// kernels' rows and order).  W: the matrix's uniform slice width.
// Minimum resident blocks per SM asked of the compiler (register cap).
// Unconstrained (1) is kept: on the 128^3 system the binary32 kernel runs
// at 52 registers (4 blocks per SM) in 31.5 us; capped to 47 or 40
// registers (5 or 6 blocks, no spills) with the grid at 5 or 6 blocks per
// SM it took 30.8-30.9 us, inside the run-to-run spread, and capped to 32
// (8 blocks, with spills) 36.9 us; binary64 73.8 us at 64 registers
// against 73.8 us at 48 (5 blocks, small spills).
#ifndef TFS_PIPE_MINB32
#define TFS_PIPE_MINB32 1
#endif
#ifndef TFS_PIPE_MINB64
#define TFS_PIPE_MINB64 1
#endif
template <typename VT, bool MIXED, int W>
__global__ void __launch_bounds__(TFS_TPB, sizeof(VT) == 4 ? TFS_PIPE_MINB32 : TFS_PIPE_MINB64)
k_spmv_pq_pipe(SellDev A, const VT *__restrict__ val, const VT *__restrict__ p, VT *__restrict__ q,
               DevState *st, double *part)
{
    const int tid = threadIdx.x, nch = A.n_chunks;
    int c = blockIdx.x;
    // column indices and geometry of the thread's next row
    int nk[W];
    uint32_t ninfo = 0u;
    if (c < nch) {
        const int i = c * TFS_TPB + tid;
        const int off = (i & ~31) * W + (i & 31);
        ninfo = ld_stream(A.rowinfo + i);
#pragma unroll
        for (int j = 0; j < W; j++) nk[j] = ld_stream(A.col + off + 32 * j);
    }
    cudaGridDependencySynchronize();   // PDL secondary of the p update (a no-op when launched plainly)
    cudaTriggerProgrammaticLaunchCompletion();
    const bool stop = MIXED ? (st->done | st->need_true) != 0 : st->done != 0;
    if (stop) return;
    if (blockIdx.x == 0 && tid == 0) st->t_spmv0 = gtimer();
    VT acc = (VT)0;
    for (; c < nch; c += gridDim.x) {
        const int i = c * TFS_TPB + tid;
        const int off = (i & ~31) * W + (i & 31);
        const int len = (int)(ninfo & 0xffffu);
        VT a[W], x[W];
#pragma unroll
        for (int j = 0; j < W; j++) {
            a[j] = (VT)0;
            x[j] = (VT)0;
            if (j < len) {
                x[j] = gather<TFS_SPMV_NC>(p + nk[j]);
                a[j] = ld_stream(val + off + 32 * j);
            }
        }
        const VT pi = p[i];
        const int cn = c + gridDim.x;
        if (cn < nch) {
            const int in = cn * TFS_TPB + tid;
            const int offn = (in & ~31) * W + (in & 31);
            ninfo = ld_stream(A.rowinfo + in);
#pragma unroll
            for (int j = 0; j < W; j++) nk[j] = ld_stream(A.col + offn + 32 * j);
        }
        VT s = (VT)0;
#pragma unroll
        for (int j = 0; j < W; j++)
            if (j < len) s = s + a[j] * x[j];
        q[i] = s;
        acc = fma_t(pi, s, acc);
    }
    double v[1];
    bool last;
    if constexpr (MIXED) {
        const float a1[1] = {(float)acc};
        last = grid_reduce_f<1>(a1, v, part, &st->counter);
    } else {
        v[0] = (double)acc;
        last = grid_reduce<1>(v, part, &st->counter);
    }
    if (last) {
        st->alpha = st->rho / v[0];
        if constexpr (MIXED) st->alpha32 = (float)st->alpha;
        st->spmv_ns += gtimer() - st->t_spmv0;
        st->spmv_n += 1;
    }
}

}  // namespace tfs
