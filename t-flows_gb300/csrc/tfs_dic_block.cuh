// tfs_dic_block.cuh -- a whole DIC preconditioner application (or the DIC
// recurrence of Prec_Form) in one thread block, for systems with deep level
// schedules of narrow levels whose vector fits in shared memory.
//
// The meshes T-FlowS ships are small and, in their own cell numbering, have
// deep level schedules (the 14,490-cell plain_50 mesh: 148 levels of at most
// 149 rows).  Launched level by level, or level-looped through global memory
// in one block, each of the ~300 dependent level steps of an application
// costs three L2 round trips (row geometry, entries, gathers of rows written
// one step earlier by other threads): about 1.7 us.  Here:
//   - the swept vector lives in shared memory (one value per row, in place:
//     y, then y / (D + TINY), then z), so a step's gathers are shared-memory
//     loads;
//   - each level's rows -- their SELL slices of column indices and values
//     (uniform or per-slice widths), geometry, diagonal and (forward)
//     right-hand side, contiguous in global memory because levels start on
//     slice boundaries -- are staged into a ring of R shared-memory slots by
//     16-byte cp.async copies issued R - 1 levels before the level runs, so
//     a step waits for no global load;
//   - the block's threads are split: the first half sweeps the level's
//     rows, the second half issues the copies (and waits for them), so the
//     row threads' dependent chain per step holds no copy instructions; the
//     level and slice-offset tables are copied into shared memory once;
//   - a step is then one cp.async group wait (copy threads), one
//     __syncthreads, the row's shared-memory loads and arithmetic.
// L1 prefetches in place of the ring measured slower than no prefetch at all
// (plain_50 binary64: 529 against 402 us per application).
//
// Every row does exactly sweep_row's arithmetic (the reference's order of
// terms: Prec_Solve.f90:46-67, Prec_Form.f90:32-40), so the results are
// bitwise those of the per-level schedule.  Every copy is a 16-byte aligned
// cp.async of the block's own, in-bounds data and every wait is on the
// thread's own copies: no wait depends on another block.
#pragma once
#include "tfs_kernels.cuh"

namespace tfs {

#define TFS_DICB_TPB 512
#define TFS_DICB_ROWS (TFS_DICB_TPB / 2)     // threads sweeping rows; the others stage levels
#define TFS_DICB_MAX_SLOTS 8
#define TFS_DICB_MAX_LEVELS 4096

// Byte offsets inside one ring slot of `rm` rows and `ents` SELL entries
// (rm and ents multiples of 32, so every part starts on a 16-byte boundary):
// geometry, diagonal, right-hand side, column indices and values of one
// level.
struct DicbSlot {
    int rm, ents, off_d, off_b, off_col, off_val, bytes;
};

template <typename T>
__host__ __device__ inline DicbSlot dicb_slot(int rm, int ents)
{
    DicbSlot s;
    s.rm = rm;
    s.ents = ents;
    s.off_d = rm * 4;
    s.off_b = s.off_d + rm * (int)sizeof(T);
    s.off_col = s.off_b + rm * (int)sizeof(T);
    s.off_val = s.off_col + ents * 4;
    s.bytes = s.off_val + ents * (int)sizeof(T);
    return s;
}

// Shared memory of the vector (n_rows values of T), rounded to 128 bytes.
template <typename T>
__host__ __device__ inline int dicb_vec_bytes(int n_rows)
{
    return (n_rows * (int)sizeof(T) + 127) & ~127;
}

// Shared memory of the level table (n_levels + 1 ints, padded to 4) and the
// slice-offset table (n_rows / 32 + 1 ints), rounded to 16 bytes.
__host__ __device__ inline int dicb_table_bytes(int n_levels, int n_rows)
{
    return ((((n_levels + 4) & ~3) + (n_rows >> 5) + 1) * 4 + 15) & ~15;
}

__device__ __forceinline__ uint32_t dicb_smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void dicb_cp16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" : : "r"(dicb_smem_addr(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void dicb_commit()
{
    asm volatile("cp.async.commit_group;" : : : "memory");
}

// Wait until at most n of the thread's committed copy groups are pending.
__device__ __forceinline__ void dicb_wait(int n)
{
    switch (n) {
    case 0: asm volatile("cp.async.wait_group 0;" : : : "memory"); break;
    case 1: asm volatile("cp.async.wait_group 1;" : : : "memory"); break;
    case 2: asm volatile("cp.async.wait_group 2;" : : : "memory"); break;
    case 3: asm volatile("cp.async.wait_group 3;" : : : "memory"); break;
    case 4: asm volatile("cp.async.wait_group 4;" : : : "memory"); break;
    case 5: asm volatile("cp.async.wait_group 5;" : : : "memory"); break;
    case 6: asm volatile("cp.async.wait_group 6;" : : : "memory"); break;
    default: asm volatile("cp.async.wait_group 7;" : : : "memory"); break;
    }
}

// Stage level l's rows into `slot` (each copy thread, ct = 0 ..
// TFS_DICB_TPB - TFS_DICB_ROWS - 1, its share of 16-byte chunks).  PART 0:
// forward (geometry, d, b, entries); 1: backward (no b); 2: the recurrence
// (geometry and entries only).  lv: the level table, so: the slice-offset
// table, both in shared memory.
template <typename T, int PART>
__device__ __forceinline__ void dicb_stage(unsigned char *slot, const DicbSlot &L, const SellDev &A,
                                           const T *val, const T *d, const T *b, const int *lv, const int *so,
                                           int l, int ct)
{
    const int r0 = lv[l], nr = lv[l + 1] - r0;
    const int e0 = so[r0 >> 5], ne = so[(r0 + nr) >> 5] - e0;
    constexpr int NC = TFS_DICB_TPB - TFS_DICB_ROWS;
    auto copy = [&](unsigned char *dst, const void *src, int bytes) {
        for (int o = ct * 16; o < bytes; o += NC * 16)
            dicb_cp16(dst + o, (const unsigned char *)src + o);
    };
    copy(slot, A.rowinfo + r0, nr * 4);
    if (PART != 2) copy(slot + L.off_d, d + r0, nr * (int)sizeof(T));
    if (PART == 0) copy(slot + L.off_b, b + r0, nr * (int)sizeof(T));
    copy(slot + L.off_col, A.col + e0, ne * 4);
    copy(slot + L.off_val, val + e0, ne * (int)sizeof(T));
}

// One sweep of k_dic_block over all levels, ascending (DIR > 0) or
// descending, through the ring of R slots.
template <typename T, int PART, int DIR>
__device__ __forceinline__ void dicb_sweep(T *s, unsigned char *ring, const DicbSlot &L, int R, const SellDev &A,
                                           const T *val, const T *d, const T *b, const int *lv, const int *so,
                                           int n_levels)
{
    const int tid = threadIdx.x;
    const bool copier = tid >= TFS_DICB_ROWS;
    const int ct = tid - TFS_DICB_ROWS;
    auto level_at = [&](int q) { return DIR > 0 ? q : n_levels - 1 - q; };
    int staged = 0;   // levels staged (= copy groups committed) by a copy thread
    for (; staged < R - 1 && staged < n_levels; staged++) {
        if (copier) {
            dicb_stage<T, PART>(ring + (size_t)(staged % R) * L.bytes, L, A, val, d, b, lv, so, level_at(staged), ct);
            dicb_commit();
        }
    }
    for (int q = 0; q < n_levels; q++) {
        if (copier) dicb_wait(staged - q - 1);   // this thread's copies of level q
        __syncthreads();             // everyone's copies; level q - 1 done, its slot free
        if (copier) {
            if (staged < n_levels) {
                dicb_stage<T, PART>(ring + (size_t)(staged % R) * L.bytes, L, A, val, d, b, lv, so,
                                    level_at(staged), ct);
                dicb_commit();
                staged++;
            }
            continue;
        }
        const unsigned char *slot = ring + (size_t)(q % R) * L.bytes;
        const uint32_t *sinfo = reinterpret_cast<const uint32_t *>(slot);
        const T *sd = reinterpret_cast<const T *>(slot + L.off_d);
        const T *sb = reinterpret_cast<const T *>(slot + L.off_b);
        const int *scol = reinterpret_cast<const int *>(slot + L.off_col);
        const T *sval = reinterpret_cast<const T *>(slot + L.off_val);
        const int l = level_at(q);
        const int r0 = lv[l], nr = lv[l + 1] - r0, sb0 = so[r0 >> 5];
        for (int k = tid; k < nr; k += TFS_DICB_ROWS) {
            const uint32_t info = sinfo[k];
            const int len = (int)(info & 0xffffu), dpos = (int)(info >> 16);
            const int e0 = so[(r0 + k) >> 5] - sb0 + (k & 31);   // entry j at e0 + 32 j
            const int i = r0 + k;
            if (PART == 2) {
                if (len == 0) { s[i] = (T)1; continue; }
                T acc = sval[e0 + (dpos << 5)];
                for (int j = 0; j < dpos; j++) {
                    const T a = sval[e0 + (j << 5)];
                    acc = acc - s[scol[e0 + (j << 5)]] * a * a;
                }
                s[i] = (T)1 / acc;
            } else if (PART == 0) {
                if (len == 0) { s[i] = (T)0; continue; }
                T acc = sb[k];
                for (int j = 0; j < dpos; j++) acc = acc - sval[e0 + (j << 5)] * s[scol[e0 + (j << 5)]];
                s[i] = acc * sd[k];
            } else {
                if (len == 0) continue;   // 0 since the forward sweep
                T acc = s[i];
                for (int j = dpos + 1; j < len; j++) acc = acc - sval[e0 + (j << 5)] * s[scol[e0 + (j << 5)]];
                s[i] = acc * sd[k];
            }
        }
    }
    if (copier) dicb_wait(0);
    __syncthreads();
}

// MODE 0: z = M^-1 b (forward sweep, scaling, backward sweep) with the
// factor d; MODE 2: the DIC factor d from the matrix (binary64; b and z
// unused).  One block of TFS_DICB_TPB threads; dynamic shared memory: the
// vector (dicb_vec_bytes), R slots of L.bytes and the level and slice-offset
// tables (dicb_table_bytes; at most TFS_DICB_MAX_LEVELS levels).  Rows past
// lvl_begin[n_levels] (the layout's final padding) are never touched.
template <typename T, int MODE>
__global__ void __launch_bounds__(TFS_DICB_TPB, 1)
k_dic_block(SellDev A, const T *__restrict__ val, T *d, const T *b, T *z, const int *__restrict__ lvl_begin,
            int n_levels, DicbSlot L, int R, DevState *st)
{
    extern __shared__ __align__(128) unsigned char dicb_smem[];
    const int n_rows = __ldg(lvl_begin + n_levels);
    T *s = reinterpret_cast<T *>(dicb_smem);
    unsigned char *ring = dicb_smem + dicb_vec_bytes<T>(n_rows);
    int *lv = reinterpret_cast<int *>(ring + (size_t)R * L.bytes);
    int *so = lv + ((n_levels + 4) & ~3);
    const int tid = threadIdx.x;
    cudaGridDependencySynchronize();   // PDL secondary: a no-op when launched plainly
    if (st->done) return;
    if (MODE == 0 && tid == 0) st->t_sweep0 = gtimer();
    for (int l = tid; l <= n_levels; l += TFS_DICB_TPB) lv[l] = __ldg(lvl_begin + l);
    for (int q = tid; q <= (n_rows >> 5); q += TFS_DICB_TPB)
        so[q] = A.width ? q * 32 * A.width : __ldg(A.slice_off + q);
    __syncthreads();
    if (MODE == 2) {
        dicb_sweep<T, 2, 1>(s, ring, L, R, A, val, d, b, lv, so, n_levels);
        for (int i = tid; i < n_rows; i += TFS_DICB_TPB) d[i] = s[i];
        return;
    }
    dicb_sweep<T, 0, 1>(s, ring, L, R, A, val, d, b, lv, so, n_levels);
    // Every row's backward start value y_i / (D_i + TINY) (Prec_Solve.f90:55-57).
#pragma unroll 4
    for (int i = tid; i < n_rows; i += TFS_DICB_TPB)
        if (__ldg(A.rowinfo + i) & 0xffffu) s[i] = s[i] / (__ldg(d + i) + (T)TINY);
    __syncthreads();
    dicb_sweep<T, 1, -1>(s, ring, L, R, A, val, d, b, lv, so, n_levels);
    for (int i = tid; i < n_rows; i += TFS_DICB_TPB) z[i] = s[i];
}

}  // namespace tfs
