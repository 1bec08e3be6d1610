// tfs_dic_block.cuh -- a whole DIC preconditioner application (or the DIC
// recurrence of Prec_Form) in one thread block, for systems whose vector fits
// in shared memory.
//
// The meshes T-FlowS ships are small and, in their own cell numbering, have
// deep level schedules (the 14,490-cell plain_50 mesh: 148 levels of about
// 100 rows).  Launched level by level, or level-looped through global memory
// in one block, each of the ~300 dependent level steps of an application
// costs three L2 round trips (row geometry, entries, gathers of rows written
// one step earlier by other threads) -- about 1.8 us.  Here the swept vector
// lives in shared memory (one binary64 or binary32 value per row, in place:
// y, then y / (D + TINY), then z), so the gathers of a step are shared-memory
// loads; the rows' geometry, entries, diagonal and right-hand side are pulled
// into L1 by prefetches issued DICB_AHEAD levels before the level runs (each
// level's rows are contiguous SELL slices, so a level is three contiguous
// ranges), and a step costs its L1 hits, its shared-memory gathers, the
// row's arithmetic and one __syncthreads.
//
// Every row does exactly sweep_row's arithmetic (the reference's order of
// terms: Prec_Solve.f90:46-67, Prec_Form.f90:32-40), so the results are
// bitwise those of the per-level schedule.
#pragma once
#include "tfs_kernels.cuh"

namespace tfs {

#define TFS_DICB_TPB 1024
#ifndef DICB_AHEAD
#define DICB_AHEAD 4
#endif

__device__ __forceinline__ void prefetch_l1(const void *p)
{
    asm volatile("prefetch.global.L1 [%0];" : : "l"(p));
}

// L1 prefetch of everything level l's rows read from global memory: their
// SELL entries (column indices and values), geometry, diagonal and (forward)
// right-hand side.  Levels start and end on slice boundaries (32 rows).
template <typename T, int MODE>
__device__ __forceinline__ void prefetch_level(const SellDev &A, const T *val, const T *d, const T *b,
                                               const int *lvl_begin, int l)
{
    const int r0 = __ldg(lvl_begin + l), r1 = __ldg(lvl_begin + l + 1);
    if (r1 <= r0) return;
    const int e0 = A.width ? r0 * A.width : __ldg(A.slice_off + (r0 >> 5));
    const int e1 = A.width ? r1 * A.width : __ldg(A.slice_off + (r1 >> 5));
    const int tid = threadIdx.x;
    for (int e = e0 + tid * 32; e < e1; e += TFS_DICB_TPB * 32) prefetch_l1(A.col + e);
    for (int e = e0 + tid * (128 / (int)sizeof(T)); e < e1; e += TFS_DICB_TPB * (128 / (int)sizeof(T)))
        prefetch_l1(val + e);
    for (int i = r0 + tid * 32; i < r1; i += TFS_DICB_TPB * 32) prefetch_l1(A.rowinfo + i);
    if (MODE != 2)
        for (int i = r0 + tid * (128 / (int)sizeof(T)); i < r1; i += TFS_DICB_TPB * (128 / (int)sizeof(T))) {
            prefetch_l1(d + i);
            if (MODE == 0) prefetch_l1(b + i);
        }
}

// MODE 0: z = M^-1 b (forward sweep, scaling, backward sweep) with the
// factor d; MODE 2: the DIC factor d from the matrix (binary64 only; b and z
// unused).  One block of TFS_DICB_TPB threads; dynamic shared memory holds
// lvl_begin[n_levels] values of T.  Rows past lvl_begin[n_levels] (the
// layout's final padding) are never touched.
template <typename T, int MODE>
__global__ void __launch_bounds__(TFS_DICB_TPB, 1)
k_dic_block(SellDev A, const T *__restrict__ val, T *d, const T *b, T *z, const int *__restrict__ lvl_begin,
            int n_levels, DevState *st)
{
    extern __shared__ __align__(16) unsigned char dicb_smem[];
    T *s = reinterpret_cast<T *>(dicb_smem);
    const int tid = threadIdx.x;
    cudaGridDependencySynchronize();   // PDL secondary: a no-op when launched plainly
    if (st->done) return;
    if (MODE == 0 && tid == 0) st->t_sweep0 = gtimer();
    const int n_rows = __ldg(lvl_begin + n_levels);
    for (int q = 0; q < DICB_AHEAD && q < n_levels; q++) prefetch_level<T, MODE>(A, val, d, b, lvl_begin, q);
    // Forward sweep (or the recurrence), levels ascending.
    for (int l = 0; l < n_levels; l++) {
        if (l + DICB_AHEAD < n_levels) prefetch_level<T, MODE>(A, val, d, b, lvl_begin, l + DICB_AHEAD);
        const int r1 = __ldg(lvl_begin + l + 1);
        for (int i = __ldg(lvl_begin + l) + tid; i < r1; i += TFS_DICB_TPB) {
            const RowGeom g = row_geom(A, i);
            if (g.len == 0) {
                s[i] = MODE == 2 ? (T)1 : (T)0;
                continue;
            }
            if (MODE == 2) {
                T acc = __ldg(val + g.off + (g.dpos << 5));
                for (int j = 0; j < g.dpos; j++) {
                    const int ee = g.off + (j << 5);
                    const T a = __ldg(val + ee);
                    acc = acc - s[__ldg(A.col + ee)] * a * a;
                }
                s[i] = (T)1 / acc;
            } else {
                T acc = __ldg(b + i);
                for (int j = 0; j < g.dpos; j++) {
                    const int ee = g.off + (j << 5);
                    acc = acc - __ldg(val + ee) * s[__ldg(A.col + ee)];
                }
                s[i] = acc * __ldg(d + i);
            }
        }
        __syncthreads();
    }
    if (MODE == 2) {
        for (int i = tid; i < n_rows; i += TFS_DICB_TPB) d[i] = s[i];
        return;
    }
    // Every row's backward start value y_i / (D_i + TINY) (Prec_Solve.f90:55-57).
    for (int i = tid; i < n_rows; i += TFS_DICB_TPB)
        if (__ldg(A.rowinfo + i) & 0xffffu) s[i] = s[i] / (__ldg(d + i) + (T)TINY);
    for (int q = 0; q < DICB_AHEAD && q < n_levels; q++)
        prefetch_level<T, 1>(A, val, d, b, lvl_begin, n_levels - 1 - q);
    __syncthreads();
    // Backward sweep, levels descending (Prec_Solve.f90:60-67).
    for (int l = n_levels - 1; l >= 0; l--) {
        if (l - DICB_AHEAD >= 0) prefetch_level<T, 1>(A, val, d, b, lvl_begin, l - DICB_AHEAD);
        const int r1 = __ldg(lvl_begin + l + 1);
        for (int i = __ldg(lvl_begin + l) + tid; i < r1; i += TFS_DICB_TPB) {
            const RowGeom g = row_geom(A, i);
            if (g.len == 0) continue;   // s[i] = 0 since the forward sweep
            T acc = s[i];
            for (int j = g.dpos + 1; j < g.len; j++) {
                const int ee = g.off + (j << 5);
                acc = acc - __ldg(val + ee) * s[__ldg(A.col + ee)];
            }
            s[i] = acc * __ldg(d + i);
        }
        __syncthreads();
    }
    for (int i = tid; i < n_rows; i += TFS_DICB_TPB) z[i] = s[i];
}

}  // namespace tfs
