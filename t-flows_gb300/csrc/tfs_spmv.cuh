// tfs_spmv.cuh -- q = A p fused with (p, q) and alpha (Cg.f90:128-153) for
// uniform-width SELL-32 matrices (every slice W <= 8 slots wide: the
// 7-entry rows of a hex mesh).
//
// The direct kernels (k_spmv_pq, k_mx_spmv_pq) walk a dependent chain per
// row -- row geometry, then the column indices and values in passes of four,
// then the gathers of p -- five memory round trips per row, one row after
// the other, so they wait on load latency at about half of the HBM
// bandwidth with no unit of the SM busy.  Two replacements, both with the
// direct kernels' rows, per-thread order of the dot-product terms and block
// and grid reductions (so bitwise the same q, (p, q) and alpha):
//
//   k_spmv_pq_pipe   software-pipelined in registers: while the gathers and
//                    values of the current row are in flight, the column
//                    indices and geometry of the thread's next row are
//                    loaded, so a row costs one round trip;
//   k_spmv_pq_bulk   the column indices, values and geometry of the coming
//                    256-row chunks streamed into shared memory by bulk
//                    asynchronous copies (cp.async.bulk + mbarrier) issued by
//                    one thread, the block consuming one chunk per step;
//   k_spmv_pq_async  the same ring of stages filled by every thread with
//                    16-byte asynchronous copies (cp.async.cg, completion by
//                    commit groups).
//
// The two staged kernels work over `vgrid` virtual blocks (the direct
// kernels' grid): a resident block takes the virtual blocks b, b +
// gridDim.x, ... in turn, each over its chunks vb, vb + vgrid, ..., and
// publishes one partial per virtual block; the last virtual block to publish
// sums the vgrid partials in order.  Every wait on one of its mbarriers is
// bounded (TFS_BULK_WAIT_NS of global time): a wait that runs out sets
// TFS_ERR_TIMEOUT and done in the solve state, and the block waits (again
// bounded) for the copies it still has in flight before it returns.
#pragma once
#include "tfs_kernels.cuh"

namespace tfs {

#define TFS_BULK_MAX_STAGES 4
#ifndef TFS_BULK_WAIT_NS
#define TFS_BULK_WAIT_NS 200000000ull   // 0.2 s
#endif

// Bytes of one stage: column indices, values, row geometry of 256 rows.
// All three parts are multiples of 16 bytes (256 * 4 * W, 256 * 8 * W, 1024).
template <typename VT>
__host__ __device__ __forceinline__ int bulk_stage_bytes(int width)
{
    return TFS_TPB * width * (int)(sizeof(int) + sizeof(VT)) + TFS_TPB * (int)sizeof(uint32_t);
}

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" : : "r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes the initialised barriers visible to the asynchronous proxy.
__device__ __forceinline__ void mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;" : : : "memory");
    asm volatile("fence.proxy.async.shared::cta;" : : : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 : : "r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// Global -> shared bulk copy, completion counted on bar (16-byte aligned
// addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 : : "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, unsigned parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
    return ok != 0u;
}

// Wait for the phase of the given parity; false after TFS_BULK_WAIT_NS.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
    if (mbar_test(bar, parity)) return true;
    const unsigned long long t0 = gtimer();
    for (;;) {
        for (int k = 0; k < 64; k++)
            if (mbar_test(bar, parity)) return true;
        if (gtimer() - t0 > TFS_BULK_WAIT_NS) return false;
    }
}

__device__ __forceinline__ void bulk_timeout(DevState *st)
{
    st->status = TFS_ERR_TIMEOUT;
    st->done = 1;
    st->niter_out = st->iter + 1;
    __threadfence();
}

__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }

// Publication of one virtual block's totals (grid_publish with the virtual
// block vb of vgrid in place of blockIdx.x of gridDim.x).
template <int NV>
__device__ __forceinline__ bool grid_publish_vb(double (&v)[NV], double *__restrict__ part,
                                                unsigned int *counter, double (*sm)[TFS_TPB / 32],
                                                int vb, int vgrid)
{
    __shared__ unsigned int is_last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) part[k * vgrid + vb] = v[k];
        __threadfence();
        is_last = (atomicAdd(counter, 1u) == (unsigned)vgrid - 1u) ? 1u : 0u;
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
    double a[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) a[k] = 0.0;
    for (int b = threadIdx.x; b < vgrid; b += TFS_TPB) {
#pragma unroll
        for (int k = 0; k < NV; k++) a[k] = a[k] + __ldcg(part + k * vgrid + b);
    }
    __syncthreads();
    block_sum<NV>(a, sm);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) v[k] = a[k];
        *counter = 0u;
        return true;
    }
    return false;
}

// q = A p; (p, q); alpha = rho / (p, q) (Cg.f90:128-153).  VT = double: the
// binary64 iteration (k_spmv_pq); VT = float: the binary32 iteration of the
// mixed solve (k_mx_spmv_pq, which also skips while a true residual is due
// and publishes alpha rounded to binary32).  Dynamic shared memory: `stages`
// stages of bulk_stage_bytes<VT>(A.width) bytes.
template <typename VT, bool MIXED>
__global__ void __launch_bounds__(TFS_TPB)
k_spmv_pq_bulk(SellDev A, const VT *__restrict__ val, const VT *__restrict__ p, VT *__restrict__ q,
               DevState *st, double *part, int vgrid, int stages)
{
    extern __shared__ __align__(128) unsigned char ring[];
    __shared__ __align__(8) uint64_t full[TFS_BULK_MAX_STAGES];
    __shared__ double sm[1][TFS_TPB / 32];
    const int W = A.width, tid = threadIdx.x, nch = A.n_chunks;
    const unsigned col_bytes = (unsigned)(TFS_TPB * W * (int)sizeof(int));
    const unsigned val_bytes = (unsigned)(TFS_TPB * W * (int)sizeof(VT));
    const unsigned stage_bytes = (unsigned)bulk_stage_bytes<VT>(W);

    // Producer (thread 0): the next chunk of this block's sequence.
    int pvb = blockIdx.x, pc = blockIdx.x, issued = 0;
    auto issue = [&]() {
        while (pvb < vgrid && pc >= nch) {
            pvb += gridDim.x;
            pc = pvb;
        }
        if (pvb >= vgrid) return;
        const int sk = issued % stages;
        unsigned char *tile = ring + (size_t)sk * stage_bytes;
        const size_t e0 = (size_t)pc * TFS_TPB * W;
        mbar_expect_tx(&full[sk], col_bytes + val_bytes + TFS_TPB * 4u);
        bulk_g2s(tile, A.col + e0, col_bytes, &full[sk]);
        bulk_g2s(tile + col_bytes, val + e0, val_bytes, &full[sk]);
        bulk_g2s(tile + col_bytes + val_bytes, A.rowinfo + (size_t)pc * TFS_TPB, TFS_TPB * 4u, &full[sk]);
        issued++;
        pc += vgrid;
    };
    // Thread 0: wait (bounded) for the copies issued after the first
    // `consumed` chunks.
    auto drain = [&](int consumed) {
        for (int k = consumed; k < issued; k++)
            if (!mbar_wait(&full[k % stages], (unsigned)(k / stages) & 1u)) return;
    };

    if (tid == 0) {
        for (int k = 0; k < stages; k++) mbar_init(&full[k], 1u);
        mbar_init_fence();
    }
    __syncthreads();
    if (tid == 0)
        for (int k = 0; k < stages; k++) issue();
    const bool stop = MIXED ? (st->done | st->need_true) != 0 : st->done != 0;
    if (stop) {
        if (tid == 0) drain(0);
        return;
    }
    if (blockIdx.x == 0 && tid == 0) st->t_spmv0 = gtimer();

    const int sl = tid >> 5, ln = tid & 31;
    int k = 0;   // chunks consumed by this block
    for (int vb = blockIdx.x; vb < vgrid; vb += gridDim.x) {
        VT acc = (VT)0;
        for (int c = vb; c < nch; c += vgrid, k++) {
            const int sk = k % stages;
            const unsigned char *tile = ring + (size_t)sk * stage_bytes;
            const bool ok = mbar_wait(&full[sk], (unsigned)(k / stages) & 1u);
            if (ok) {
                const int *tc = (const int *)tile + sl * 32 * W + ln;
                const VT *tv = (const VT *)(tile + col_bytes) + sl * 32 * W + ln;
                const uint32_t info = ((const uint32_t *)(tile + col_bytes + val_bytes))[tid];
                const int len = (int)(info & 0xffffu);
                int kk[8];
                VT a[8], x[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    kk[j] = 0;
                    a[j] = (VT)0;
                    if (j < len) {
                        kk[j] = tc[32 * j];
                        a[j] = tv[32 * j];
                    }
                }
#pragma unroll
                for (int j = 0; j < 8; j++) x[j] = (j < len) ? gather<TFS_SPMV_NC>(p + kk[j]) : (VT)0;
                VT s = (VT)0;
#pragma unroll
                for (int j = 0; j < 8; j++)
                    if (j < len) s = s + a[j] * x[j];
                const int i = c * TFS_TPB + tid;
                q[i] = s;
                acc = fma_t(p[i], s, acc);
            }
            // Every thread is done with the stage (or a wait ran out).
            if (__syncthreads_or(!ok)) {
                if (tid == 0) {
                    bulk_timeout(st);
                    drain(k);
                }
                return;
            }
            if (tid == 0) {
                asm volatile("fence.proxy.async.shared::cta;" : : : "memory");
                issue();
            }
        }
        double v[1];
        if constexpr (MIXED) {
            const float a1[1] = {(float)acc};
            block_sum_f<1>(a1, v, sm);
        } else {
            v[0] = (double)acc;
            block_sum<1>(v, sm);
        }
        if (grid_publish_vb<1>(v, part, &st->counter, sm, vb, vgrid)) {
            st->alpha = st->rho / v[0];
            if constexpr (MIXED) st->alpha32 = (float)st->alpha;
            st->spmv_ns += gtimer() - st->t_spmv0;
            st->spmv_n += 1;
        }
    }
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" : : "r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit()
{
    asm volatile("cp.async.commit_group;" : : : "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" : : "n"(N) : "memory");
}

// As k_spmv_pq_bulk, with the stages filled by all threads of the block
// with 16-byte cp.async copies: STAGES - 1 chunks are in flight while one is
// consumed.  A step waits for the thread's own copies of the chunk
// (cp.async.wait_group), then a block barrier makes every thread's copies
// visible and frees the stage consumed in the step before, which the same
// step refills.  The waits are on the block's own in-bounds copies.
template <typename VT, bool MIXED, int STAGES>
__global__ void __launch_bounds__(TFS_TPB)
k_spmv_pq_async(SellDev A, const VT *__restrict__ val, const VT *__restrict__ p, VT *__restrict__ q,
                DevState *st, double *part, int vgrid)
{
    extern __shared__ __align__(128) unsigned char ring[];
    __shared__ double sm[1][TFS_TPB / 32];
    const int W = A.width, tid = threadIdx.x, nch = A.n_chunks;
    const unsigned col_bytes = (unsigned)(TFS_TPB * W * (int)sizeof(int));
    const unsigned val_bytes = (unsigned)(TFS_TPB * W * (int)sizeof(VT));
    const unsigned stage_bytes = (unsigned)bulk_stage_bytes<VT>(W);

    // The block's chunk sequence, walked identically by every thread.
    int pvb = blockIdx.x, pc = blockIdx.x, issued = 0;
    auto issue = [&]() {
        while (pvb < vgrid && pc >= nch) {
            pvb += gridDim.x;
            pc = pvb;
        }
        if (pvb < vgrid) {
            unsigned char *tile = ring + (size_t)(issued % STAGES) * stage_bytes;
            const char *gc = (const char *)(A.col + (size_t)pc * TFS_TPB * W);
            const char *gv = (const char *)(val + (size_t)pc * TFS_TPB * W);
            const char *gi = (const char *)(A.rowinfo + (size_t)pc * TFS_TPB);
            for (unsigned o = tid * 16u; o < col_bytes; o += TFS_TPB * 16u) cp_async16(tile + o, gc + o);
            for (unsigned o = tid * 16u; o < val_bytes; o += TFS_TPB * 16u)
                cp_async16(tile + col_bytes + o, gv + o);
            if (tid < TFS_TPB / 4) cp_async16(tile + col_bytes + val_bytes + tid * 16u, gi + tid * 16u);
            pc += vgrid;
        }
        issued++;
        cp_async_commit();
    };

#pragma unroll
    for (int k = 0; k < STAGES - 1; k++) issue();
    const bool stop = MIXED ? (st->done | st->need_true) != 0 : st->done != 0;
    if (stop) {
        cp_async_wait<0>();
        return;
    }
    if (blockIdx.x == 0 && tid == 0) st->t_spmv0 = gtimer();

    const int sl = tid >> 5, ln = tid & 31;
    int k = 0;   // chunks consumed by this block
    for (int vb = blockIdx.x; vb < vgrid; vb += gridDim.x) {
        VT acc = (VT)0;
        for (int c = vb; c < nch; c += vgrid, k++) {
            cp_async_wait<STAGES - 2>();
            __syncthreads();
            issue();
            const unsigned char *tile = ring + (size_t)(k % STAGES) * stage_bytes;
            const int *tc = (const int *)tile + sl * 32 * W + ln;
            const VT *tv = (const VT *)(tile + col_bytes) + sl * 32 * W + ln;
            const uint32_t info = ((const uint32_t *)(tile + col_bytes + val_bytes))[tid];
            const int len = (int)(info & 0xffffu);
            int kk[8];
            VT a[8], x[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                kk[j] = 0;
                a[j] = (VT)0;
                if (j < len) {
                    kk[j] = tc[32 * j];
                    a[j] = tv[32 * j];
                }
            }
#pragma unroll
            for (int j = 0; j < 8; j++) x[j] = (j < len) ? gather<TFS_SPMV_NC>(p + kk[j]) : (VT)0;
            VT s = (VT)0;
#pragma unroll
            for (int j = 0; j < 8; j++)
                if (j < len) s = s + a[j] * x[j];
            const int i = c * TFS_TPB + tid;
            q[i] = s;
            acc = fma_t(p[i], s, acc);
        }
        double v[1];
        if constexpr (MIXED) {
            const float a1[1] = {(float)acc};
            block_sum_f<1>(a1, v, sm);
        } else {
            v[0] = (double)acc;
            block_sum<1>(v, sm);
        }
        if (grid_publish_vb<1>(v, part, &st->counter, sm, vb, vgrid)) {
            st->alpha = st->rho / v[0];
            if constexpr (MIXED) st->alpha32 = (float)st->alpha;
            st->spmv_ns += gtimer() - st->t_spmv0;
            st->spmv_n += 1;
        }
    }
    cp_async_wait<0>();
}

// q = A p; (p, q); alpha, software-pipelined over the thread's rows c *
// 256 + tid, c = blockIdx.x, blockIdx.x + gridDim.x, ... (the direct
// kernels' rows and order).  W: the matrix's uniform slice width.
// Minimum resident blocks per SM asked of the compiler (register cap).
// Unconstrained (1) measured best on the 128^3 system: binary32 35.7 us at
// 40 registers against 36.9 us capped to 32 (8 blocks, with spills);
// binary64 74.6 against 75.4 us at 56.
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
        ninfo = __ldg(A.rowinfo + i);
#pragma unroll
        for (int j = 0; j < W; j++) nk[j] = __ldg(A.col + off + 32 * j);
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
                a[j] = __ldg(val + off + 32 * j);
            }
        }
        const VT pi = p[i];
        const int cn = c + gridDim.x;
        if (cn < nch) {
            const int in = cn * TFS_TPB + tid;
            const int offn = (in & ~31) * W + (in & 31);
            ninfo = __ldg(A.rowinfo + in);
#pragma unroll
            for (int j = 0; j < W; j++) nk[j] = __ldg(A.col + offn + 32 * j);
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
