// tfs_dic.cuh -- one DIC preconditioner application in one cooperative launch.
//
// z = M^-1 r with M the diagonal incomplete Cholesky factor (forward sweep,
// diagonal scaling, backward sweep: Prec_Solve.f90:46-67) as one persistent
// kernel instead of one launch per level.  All blocks are co-resident
// (cooperative launch), each block owns a fixed set of rows of every level
// (row = level start + block * 256 + thread, grid-stride), and the levels are
// separated by a grid barrier.  While a block waits at a barrier it has
// already loaded the geometry and the first four column indices and values of
// its rows of the next level, so a level costs its dependent gathers plus one
// barrier.  The small trailing levels run in block 0 alone (__syncthreads
// between levels) between the two sweeps.
//
// Every row does exactly sweep_row's arithmetic (the reference's order of
// terms), so the result is bitwise the per-level schedule's.  Rows of one
// level never read each other, so the gathers of all of a thread's rows of a
// level are issued before any of its results is stored.
//
// With FUSE the kernel also finishes the CG step that follows the
// preconditioner (Cg.f90:100-123): rho = (r, z) reduced over the grid (one
// partial per block, summed in block order by the last block to arrive at
// the final barrier) and p = z + beta p.
//
// Every barrier wait is bounded: a block that polls more than TFS_BAR_SPINS
// times raises the abort flag, every block returns at its next barrier, and
// the solve ends with TFS_ERR_TIMEOUT.
#pragma once
#include <type_traits>

#include "tfs_kernels.cuh"

namespace tfs {

#define TFS_BAR_SPINS (1u << 22)
#define TFS_DIC_TPB 1024

// Polling load: relaxed, so that a spinning thread does not invalidate its
// SM's L1 (where the other warps keep the prefetched matrix entries) on
// every poll; the caller fences once when the wait is over.
__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned atom_add_release_u32(unsigned *p, unsigned v)
{
    unsigned old;
    asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" : : "l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void bar_abort(DevState *st)
{
    atomicExch(&st->bar_abort, 1u);
    st->status = TFS_ERR_TIMEOUT;
    st->done = 1;
    st->niter_out = st->iter + 1;
    __threadfence();
}

// The grid barrier counts arrivals on one counter that only grows within a
// solve (it starts at zero with the solve's state): the k-th barrier since
// the solve began is complete when the counter reaches k * gridDim.x, and the
// block whose arrival makes it so publishes k in bar_gen (release); the
// others poll bar_gen (relaxed) and fence once it has reached k.  Thread 0
// of every block keeps k in `gen`.
//
// Arrival of thread 0 (after __syncthreads, so the block's writes precede
// it); true for the block that completes generation gen + 1.
__device__ __forceinline__ bool bar_arrive(DevState *st, unsigned gen)
{
    const unsigned old = atom_add_release_u32(&st->bar_count, 1u);
    return old == (gen + 1u) * gridDim.x - 1u;
}

// Thread 0 waits until generation target is complete; false on abort.
__device__ __forceinline__ bool bar_wait(DevState *st, unsigned target)
{
    unsigned spins = 0;
    while ((int)(ld_relaxed_u32(&st->bar_gen) - target) < 0) {
        if ((spins & 63u) == 63u && ld_relaxed_u32(&st->bar_abort)) return false;
        if (++spins > TFS_BAR_SPINS) { bar_abort(st); return false; }
    }
    __threadfence();
    return true;
}

// Split grid barrier: bar_split_arrive (all threads) orders the block's
// writes and lets thread 0 arrive without waiting, so the block can load
// what the next level needs from constant data while the others arrive;
// bar_split_wait returns once every block has arrived (false in every
// thread when the barrier was aborted).
__device__ __forceinline__ void bar_split_arrive(DevState *st, unsigned &gen, int &last)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        last = bar_arrive(st, gen) ? 1 : 0;
        gen += 1u;
        if (last) st_release_u32(&st->bar_gen, gen);
    }
}

__device__ __forceinline__ bool bar_split_wait(DevState *st, unsigned gen, int last)
{
    __shared__ int s_okw;
    if (threadIdx.x == 0) s_okw = last ? 1 : (bar_wait(st, gen) ? 1 : 0);
    __syncthreads();
    return s_okw != 0;
}

__device__ __forceinline__ bool grid_barrier(DevState *st, unsigned &gen)
{
    int last = 0;
    bar_split_arrive(st, gen, last);
    return bar_split_wait(st, gen, last);
}

// Sum over a block of TFS_DIC_TPB threads; the binary64 result is valid in
// thread 0.  Binary32 values go through warp_sum_f.
template <typename AT>
__device__ __forceinline__ double dic_block_sum(AT v, double *sm)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double w;
    if constexpr (sizeof(AT) == 4) {
        w = warp_sum_f(v);
    } else {
        w = v;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) w = w + __shfl_down_sync(FULL, w, o);
    }
    if (lane == 0) sm[warp] = w;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0) {
        s = sm[0];
        for (int k = 1; k < TFS_DIC_TPB / 32; k++) s = s + sm[k];
    }
    return s;
}

// The rows of one level a thread owns, R at a time, with the data that does
// not depend on other rows loaded ahead.
template <typename T, int R>
struct DicRows {
    int i[R];
    RowGeom g[R];
    int kk[R][4];
    T aa[R][4];

    template <int MODE>
    __device__ __forceinline__ void fetch(const SellDev &A, const T *__restrict__ val, int first, int r1,
                                          int stride)
    {
#pragma unroll
        for (int r = 0; r < R; r++) {
            i[r] = first + r * stride;
            g[r] = RowGeom{0, 0, 0};
#pragma unroll
            for (int q = 0; q < 4; q++) { kk[r][q] = 0; aa[r][q] = (T)0; }
            if (i[r] < r1) {
                g[r] = row_geom(A, i[r]);
                const int j0 = MODE == 1 ? g[r].dpos + 1 : 0, j1 = MODE == 1 ? g[r].len : g[r].dpos;
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (j0 + q < j1) {
                        const int ee = g[r].off + ((j0 + q) << 5);
                        kk[r][q] = __ldg(A.col + ee);
                        aa[r][q] = __ldg(val + ee);
                    }
            } else {
                i[r] = -1;
            }
        }
    }

    // MODE 0: o = y from b (forward); MODE 1: o = z from y (backward).  With
    // RZ, acc += r_i z_i for every backward row (r = rr).
    template <int MODE, bool RZ, typename AT>
    __device__ __forceinline__ void run(const SellDev &A, const T *__restrict__ val, const T *d,
                                        const T *b, const T *y, T *o, const T *rr, AT &acc)
    {
        T s[R], di[R], xg[R][4];
#pragma unroll
        for (int r = 0; r < R; r++) {
            s[r] = (T)0;
            di[r] = (T)0;
            if (i[r] >= 0 && g[r].len > 0) {
                di[r] = d[i[r]];
                if (MODE == 0) s[r] = b[i[r]];
                else s[r] = y[i[r]] / (di[r] + (T)TINY);
            }
            const int j0 = MODE == 1 ? g[r].dpos + 1 : 0, j1 = MODE == 1 ? g[r].len : g[r].dpos;
#pragma unroll
            for (int q = 0; q < 4; q++) xg[r][q] = (i[r] >= 0 && j0 + q < j1) ? __ldcg(o + kk[r][q]) : (T)0;
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            if (i[r] < 0) continue;
            if (g[r].len == 0) { o[i[r]] = (T)0; continue; }
            const int j0 = MODE == 1 ? g[r].dpos + 1 : 0, j1 = MODE == 1 ? g[r].len : g[r].dpos;
            T sr = s[r];
            int j = j0;
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (j < j1) { sr = sr - aa[r][q] * xg[r][q]; j++; }
            for (; j < j1; j++) {
                const int ee = g[r].off + (j << 5);
                sr = sr - __ldg(val + ee) * __ldcg(o + __ldg(A.col + ee));
            }
            const T out = sr * di[r];
            o[i[r]] = out;
            if (RZ) {
                if constexpr (sizeof(AT) == 4) acc = fmaf(rr[i[r]], out, acc);
                else acc = fma((double)rr[i[r]], (double)out, acc);
            }
        }
    }
};

// One level (rows [r0, r1)) by the whole grid; the first R rows of the
// thread were fetched ahead into `cur`.
template <typename T, int R, int MODE, bool RZ, typename AT>
__device__ __forceinline__ void dic_level(DicRows<T, R> &cur, const SellDev &A, const T *__restrict__ val,
                                          const T *d, const T *b, const T *y, T *o, const T *rr,
                                          int r0, int r1, int tid, int stride, AT &acc)
{
    cur.template run<MODE, RZ>(A, val, d, b, y, o, rr, acc);
    for (int first = r0 + tid + R * stride; first < r1; first += R * stride) {
        cur.template fetch<MODE>(A, val, first, r1, stride);
        cur.template run<MODE, RZ>(A, val, d, b, y, o, rr, acc);
    }
}

// Levels [l_begin, l_end) by one block, forward then backward.
template <typename T, bool RZ, typename AT>
__device__ __forceinline__ void dic_tail(const SellDev &A, const T *__restrict__ val, const T *d,
                                         const T *b, T *y, T *z, const int *__restrict__ lvl_begin,
                                         int l_begin, int l_end, AT &acc)
{
    DicRows<T, 1> row;
    for (int lev = l_begin; lev < l_end; lev++) {
        const int r1 = __ldg(lvl_begin + lev + 1);
        for (int i = __ldg(lvl_begin + lev) + threadIdx.x; i < r1; i += blockDim.x) {
            row.template fetch<0>(A, val, i, r1, 0);
            row.template run<0, false>(A, val, d, b, nullptr, y, nullptr, acc);
        }
        __syncthreads();
    }
    for (int lev = l_end - 1; lev >= l_begin; lev--) {
        const int r1 = __ldg(lvl_begin + lev + 1);
        for (int i = __ldg(lvl_begin + lev) + threadIdx.x; i < r1; i += blockDim.x) {
            row.template fetch<1>(A, val, i, r1, 0);
            row.template run<1, RZ>(A, val, d, nullptr, y, z, b, acc);
        }
        __syncthreads();
    }
}

// z = M^-1 b (b is the residual r); levels [0, n_big) are swept by the grid,
// [n_big, n_levels) by block 0.  FUSE: rho = (r, z), p = z + beta p.
template <typename T, int R, bool FUSE>
__global__ void __launch_bounds__(TFS_DIC_TPB, 1)
k_dic_apply(SellDev A, const T *__restrict__ val, const T *d, const T *b, T *y, T *z, T *p,
            const int *__restrict__ lvl_begin, int n_big, int n_levels, int n_int, DevState *st,
            double *part)
{
    if (st->done) return;
    using AT = typename std::conditional<sizeof(T) == 4, float, double>::type;
    const int tid = blockIdx.x * TFS_DIC_TPB + threadIdx.x, stride = gridDim.x * TFS_DIC_TPB;
    const bool fuse = FUSE && !st->need_true;
    if (FUSE && blockIdx.x == 0 && threadIdx.x == 0) st->t_sweep0 = gtimer();
    AT acc = (AT)0;
    DicRows<T, R> cur;
    unsigned gen = 0;   // barriers completed since the solve began (thread 0)
    int last = 0;
    if (threadIdx.x == 0) gen = ld_relaxed_u32(&st->bar_gen);
    // Forward sweep over the large levels; while a level's barrier completes
    // the block loads the geometry of its rows of the next level.
    if (n_big > 0) cur.template fetch<0>(A, val, __ldg(lvl_begin) + tid, __ldg(lvl_begin + 1), stride);
    for (int l = 0; l < n_big; l++) {
        const int r0 = __ldg(lvl_begin + l), r1 = __ldg(lvl_begin + l + 1);
        dic_level<T, R, 0, false>(cur, A, val, d, b, nullptr, y, nullptr, r0, r1, tid, stride, acc);
        bar_split_arrive(st, gen, last);
        if (l + 1 < n_big)
            cur.template fetch<0>(A, val, __ldg(lvl_begin + l + 1) + tid, __ldg(lvl_begin + l + 2), stride);
        else
            cur.template fetch<1>(A, val, __ldg(lvl_begin + n_big - 1) + tid, __ldg(lvl_begin + n_big), stride);
        if (!bar_split_wait(st, gen, last)) return;
    }
    // Both tails in block 0.
    if (n_big < n_levels) {
        if (blockIdx.x == 0) {
            if (fuse) dic_tail<T, true>(A, val, d, b, y, z, lvl_begin, n_big, n_levels, acc);
            else dic_tail<T, false>(A, val, d, b, y, z, lvl_begin, n_big, n_levels, acc);
        }
        if (n_big > 0 && !grid_barrier(st, gen)) return;
    }
    // Backward sweep over the large levels, descending.
    for (int l = n_big - 1; l >= 0; l--) {
        const int r0 = __ldg(lvl_begin + l), r1 = __ldg(lvl_begin + l + 1);
        if (fuse) dic_level<T, R, 1, true>(cur, A, val, d, nullptr, y, z, b, r0, r1, tid, stride, acc);
        else dic_level<T, R, 1, false>(cur, A, val, d, nullptr, y, z, b, r0, r1, tid, stride, acc);
        if (l > 0) {
            bar_split_arrive(st, gen, last);
            cur.template fetch<1>(A, val, __ldg(lvl_begin + l - 1) + tid, __ldg(lvl_begin + l), stride);
            if (!bar_split_wait(st, gen, last)) return;
        }
    }
    if (!fuse) return;

    // rho = (r, z): block sums, then the last block to arrive sums them in
    // block order, publishes rho and releases the others.
    __shared__ double sm[TFS_DIC_TPB / 32];
    __shared__ int s_last, s_ok;
    const double bsum = dic_block_sum<AT>(acc, sm);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = bsum;
        const int l = bar_arrive(st, gen) ? 1 : 0;
        gen += 1u;
        s_last = l;
        s_ok = l ? 1 : (bar_wait(st, gen) ? 1 : 0);
        if (l) __threadfence();
    }
    __syncthreads();
    if (s_last) {
        double a = 0.0;
        for (int k = threadIdx.x; k < (int)gridDim.x; k += TFS_DIC_TPB) a = a + __ldcg(part + k);
        __syncthreads();
        const double total = dic_block_sum<double>(a, sm);
        if (threadIdx.x == 0) {
            st->rho = total;
            if (st->iter > 1) publish_beta(st);
            st->sweep_ns += gtimer() - st->t_sweep0;
            st->sweep_n += 1;
            st_release_u32(&st->bar_gen, gen);
        }
        __syncthreads();   // the other threads of this block read rho below
    }
    if (!s_ok) return;
    // p = z (first iteration) or z + beta p (Cg.f90:114-123).
    const int it = st->iter;
    if constexpr (sizeof(T) == 4) {
        const float beta = it == 1 ? 0.f : __ldcg(&st->beta32);
        const float4 *z4 = (const float4 *)z;
        float4 *p4 = (float4 *)p;
        for (int k = tid; k < n_int / 4; k += stride) {
            const float4 zz = __ldcg(z4 + k);
            if (it == 1) p4[k] = zz;
            else {
                const float4 pp = __ldcg(p4 + k);
                p4[k] = make_float4(fmaf(beta, pp.x, zz.x), fmaf(beta, pp.y, zz.y), fmaf(beta, pp.z, zz.z),
                                    fmaf(beta, pp.w, zz.w));
            }
        }
    } else {
        const double beta = it == 1 ? 0.0 : __ldcg(&st->beta);
        for (int k = tid; k < n_int; k += stride) {
            const double zz = __ldcg(z + k);
            p[k] = it == 1 ? zz : zz + beta * __ldcg(p + k);
        }
    }
}

// ------------------------------------------------ slabs with neighbour waits
//
// The same application as one cooperative launch without grid barriers.
// Block b owns the rows whose reverse Cuthill-McKee position lies in slab b
// of G equal slabs, in every level (a contiguous range of each level, whose
// rows are in RCM order: seg[L * (G + 1) + b] .. seg[L * (G + 1) + b + 1]).
// A row's neighbours lie within the RCM bandwidth, so the rows a block reads
// belong to the blocks dep[b].x .. dep[b].y, a few slabs around its own.  A
// block sweeps its rows level by level (forward 0..nl-1, then backward
// nl-1..0: 2 nl steps) and after every step publishes the step number in its
// progress word (release); before a step it waits until every block of its
// range has published the step before (acquire) -- the level structure
// guarantees that the rows it reads were written in earlier steps.  No block
// waits for the whole grid.  Progress words only grow: step s of the e-th
// application is published as e * (2 nl + 1) + s, e counted in ectl[0] by
// the last block to finish (ectl[1] counts arrivals), so nothing is cleared
// between applications.  Deadlock-free: all blocks are co-resident
// (cooperative launch) and step 1 waits for nobody.  Every wait is bounded
// (TFS_BAR_SPINS polls, abort flag, TFS_ERR_TIMEOUT); an aborted block still
// arrives at the end, so the application counter stays consistent.
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u64(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" : : "l"(p), "l"(v) : "memory");
}

template <typename T, int R>
__global__ void __launch_bounds__(TFS_DIC_TPB, R == 1 ? 2 : 1)
k_dic_slab(SellDev A, const T *__restrict__ val, const T *d, const T *b, T *y, T *z,
           const int *__restrict__ seg, const int2 *__restrict__ dep, int nl,
           unsigned long long *prog, unsigned long long *ectl, DevState *st)
{
    using AT = typename std::conditional<sizeof(T) == 4, float, double>::type;
    const int G = gridDim.x, blk = blockIdx.x;
    const unsigned long long steps = 2ull * (unsigned long long)nl + 1ull;
    const unsigned long long base = *(volatile unsigned long long *)ectl * steps;
    const int2 rng = __ldg(dep + blk);
    const bool active = st->done == 0;
    if (active && blk == 0 && threadIdx.x == 0) st->t_sweep0 = gtimer();
    AT acc = (AT)0;
    DicRows<T, R> cur;
    for (int k = 0; active && k < 2 * nl; k++) {
        const int mode = k < nl ? 0 : 1;
        const int lev = k < nl ? k : 2 * nl - 1 - k;
        const int r0 = __ldg(seg + lev * (G + 1) + blk), r1 = __ldg(seg + lev * (G + 1) + blk + 1);
        // Loads that do not depend on other rows go ahead of the wait.
        if (mode == 0) cur.template fetch<0>(A, val, r0 + threadIdx.x, r1, TFS_DIC_TPB);
        else cur.template fetch<1>(A, val, r0 + threadIdx.x, r1, TFS_DIC_TPB);
        // Steps 1 (forward level 0) and nl + 1 (backward top level) read no
        // other block's rows of this application.
        if (k != 0 && k != nl) {
            const int j = rng.x + (int)threadIdx.x;
            bool fail = false;
            if (j <= rng.y && j != blk) {
                const unsigned long long want = base + (unsigned long long)k;
                unsigned spins = 0;
                while (ld_acquire_u64(prog + j) < want) {
                    if ((spins & 63u) == 63u && ld_relaxed_u32(&st->bar_abort)) { fail = true; break; }
                    if (++spins > TFS_BAR_SPINS) { bar_abort(st); fail = true; break; }
                }
                __threadfence();
            }
            if (__syncthreads_or(fail)) break;
        }
        if (mode == 0) dic_level<T, R, 0, false>(cur, A, val, d, b, nullptr, y, nullptr, r0, r1, threadIdx.x,
                                                 TFS_DIC_TPB, acc);
        else dic_level<T, R, 1, false>(cur, A, val, d, nullptr, y, z, nullptr, r0, r1, threadIdx.x,
                                       TFS_DIC_TPB, acc);
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            st_release_u64(prog + blk, base + (unsigned long long)(k + 1));
        }
    }
    // Every block arrives once; the last one advances the application count.
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(ectl + 1, 1ull) == (unsigned long long)G - 1ull) {
            if (active) {
                st->sweep_ns += gtimer() - st->t_sweep0;
                st->sweep_n += 1;
            }
            ectl[1] = 0ull;
            __threadfence();
            st_release_u64(ectl, ectl[0] + 1ull);
        }
    }
}

}  // namespace tfs
