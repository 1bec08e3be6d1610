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
//     y, then z; the backward start values y / (D + TINY) go through z in
//     global memory), so a step's gathers are shared-memory loads;
//   - consecutive levels are grouped (host side) so that a group's rows and
//     SELL entries fit one of R ring slots; a group's rows -- geometry,
//     diagonal, (forward) right-hand side, column indices and values, one
//     contiguous range of each array because levels start on slice
//     boundaries -- are staged into its slot by five bulk asynchronous copies
//     (cp.async.bulk, completion counted in bytes on the slot's "full"
//     mbarrier) that one lane of a copy warp issues as soon as the slot's
//     previous group is done;
//   - the 256 row threads sweep a group level by level with one named
//     barrier (bar.sync) per level, test the slot's "full" barrier once per
//     group and release the slot with one arrival on its "empty" barrier;
//   - the level records (first row, rows, first entry, entries), the group
//     table and the slice-offset table are built in shared memory once.
// Measured on plain_50 per binary32 / binary64 application: one 16-byte
// cp.async per thread and level with every copy thread's and row thread's
// arrival on per-level barriers 189 / 245 us (the copies' 256 + 256 barrier
// arrivals per level were the bound: 133 / 208 us with no row arithmetic at
// all); one bulk copy set and one arrival per level 139 / 232 us (issuing a
// level's five bulk copies takes the copy lane about 500 cycles, testing the
// barrier and releasing the slot the row threads about 400); levels grouped
// into two slots 113 / 228 us (3 or 4 slots: 116 / 239, 119 / 242), of
// which the scaling pass between the sweeps (global loads of the geometry
// and D, one division per row) took 24 / 48 us.  With the scaling in the
// forward sweep, right after each row's value (the backward sweep staging
// the start values from z like the right-hand side): 106 / 245 us (a
// division per row inside the sweep holds each level back on the narrow
// binary64 pipe).  Split into a forward kernel, a scaling grid over every
// SM and a backward kernel (MODE 3, k_dic_scale, MODE 4): 98 / 186 us, the
// default for binary64 and for deep binary32 schedules (dicb_split).
// Loading each row thread's next-level operands from the slot during the
// current level measured slower (129 / 252 us; 146 / 248 with the gathers
// kept ahead of those loads).
//
// Every row does exactly sweep_row's arithmetic (the reference's order of
// terms: Prec_Solve.f90:46-67, Prec_Form.f90:32-40), so the results are
// bitwise those of the per-level schedule.  Every bulk copy is of the
// block's own, in-bounds data, 16-byte aligned at both ends (the host checks
// the base addresses; the copy lane checks each group's and stops on a
// misaligned one).  No wait depends on another block: the mbarrier waits
// are on this block's own copies and row threads, and each is bounded
// (TFS_DICB_WAIT_NS of global time); a wait that runs out raises the
// block's abort flag, after which no thread waits on an mbarrier again, no
// copy is issued and no row is read from a slot (a slot may then hold
// another group's rows; the results are garbage), every row thread still
// passes the same named barriers, the copy lane waits (bounded, regardless
// of the flag) for the copies it issued to land before it leaves, and the
// solve ends with TFS_ERR_TIMEOUT.
#pragma once
#include "tfs_kernels.cuh"
#include "tfs_dicb_plan.h"

namespace tfs {

#define TFS_DICB_ROWS 256                    // threads sweeping rows
#define TFS_DICB_TPB (TFS_DICB_ROWS + 32)    // + one copy warp (its lane 0 issues the copies)
#ifndef TFS_DICB_SLOTS
#define TFS_DICB_SLOTS 2                     // ring slots (each holds one group of levels)
#endif
#define TFS_DICB_MAX_LEVELS 4096
#define TFS_DICB_ROW_BAR 1                   // named barrier of the row threads
#ifndef TFS_DICB_WAIT_NS
#define TFS_DICB_WAIT_NS 500000000ull        // 0.5 s
#endif

// Whether an application in arithmetic T over n_levels levels runs as three
// kernels (forward sweep, scaling grid, backward sweep) instead of one:
// always in binary64; in binary32 for deep schedules (measured per DIC-CG
// solve, split against one kernel: plain_50 8.66 / 9.31 ms, a 23x19x17
// lexicographic system 3.75 / 3.88 ms, chan 0.974 / 0.990 ms; a randomly
// numbered 16^3 system, 15 levels, 2.60 / 2.46 ms).
#define TFS_DICB_SPLIT32_LEVELS 24
template <typename T>
__host__ __device__ inline bool dicb_split(int n_levels)
{
    return sizeof(T) == 8 || n_levels >= TFS_DICB_SPLIT32_LEVELS;
}

__device__ __forceinline__ uint32_t dicb_smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void dicb_mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" : : "r"(dicb_smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void dicb_mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" : : "r"(dicb_smem_addr(bar)) : "memory");
}

// Arrive on bar and raise its pending transaction count by `bytes`, the
// bytes the bulk copies issued next will deliver.
__device__ __forceinline__ void dicb_mbar_expect(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 : : "r"(dicb_smem_addr(bar)), "r"(bytes) : "memory");
}

// Bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned)
// from global to this block's shared memory, counted on bar when it lands.
__device__ __forceinline__ void dicb_bulk(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 : : "r"(dicb_smem_addr(dst)), "l"(src), "r"(bytes), "r"(dicb_smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool dicb_mbar_test(uint64_t *bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(ok) : "r"(dicb_smem_addr(bar)), "r"(parity) : "memory");
    return ok != 0;
}

// Wait for the phase of the given parity to complete, at most wait_ns;
// false (and the abort flag raised) when it did not, or at once when the
// flag is already up.
__device__ __forceinline__ bool dicb_mbar_wait(uint64_t *bar, unsigned parity, volatile int *abort,
                                               unsigned long long wait_ns)
{
    if (dicb_mbar_test(bar, parity)) return true;
    if (*abort) return false;
    const unsigned long long t0 = gtimer();
    for (unsigned k = 1;; k++) {
        if (dicb_mbar_test(bar, parity)) return true;
        if ((k & 255u) == 0u) {
            if (*abort) return false;
            if (gtimer() - t0 > wait_ns) {
                *abort = 1;
                return false;
            }
        }
    }
}

__device__ __forceinline__ void dicb_row_sync()
{
    asm volatile("bar.sync %0, %1;" : : "n"(TFS_DICB_ROW_BAR), "n"(TFS_DICB_ROWS) : "memory");
}

// The ring's per-slot barriers, the block's abort flag and the wait limit
// (TFS_DICB_WAIT_NS, or the diagnostic limit under which the copy lane
// stages nothing: tfs_diag_dic_timeout).
struct DicbSync {
    uint64_t *full, *empty;   // R each
    volatile int *abort;
    unsigned long long wait_ns;
    bool starve;
};

// Row i's new value from its staged entries j0 <= j < j1 (at e0 + 32 j of
// the slot): acc - sum a_j s[col_j] in ascending j (PART 0 and 1), or
// acc - sum s[col_j] a_j a_j (PART 2); up to 8 entries have every column
// index, value and gather issued before the in-order chain of updates.
// Measured on plain_50 (ungrouped ring): binary32 219 -> 189 us per
// application; with the binary64 updates predicated like the binary32
// ones, 286 -> 367 us.
template <typename T, int PART>
__device__ __forceinline__ T dicb_row(T acc, const T *s, const int *scol, const T *sval, int e0, int j0, int j1)
{
    int c[8];
    T a[8], x[8];
#pragma unroll
    for (int u = 0; u < 8; u++)
        if (j0 + u < j1) {
            c[u] = scol[e0 + ((j0 + u) << 5)];
            a[u] = sval[e0 + ((j0 + u) << 5)];
        }
#pragma unroll
    for (int u = 0; u < 8; u++)
        if (j0 + u < j1) x[u] = s[c[u]];
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (j0 + u < j1) acc = PART == 2 ? acc - x[u] * a[u] * a[u] : acc - a[u] * x[u];
    } else {
        // binary64: leave the chain at the row's last entry (GB300's narrow
        // binary64 pipe would otherwise also run the absent entries' updates)
#pragma unroll
        for (int u = 0; u < 8; u++) {
            if (j0 + u >= j1) break;
            acc = PART == 2 ? acc - x[u] * a[u] * a[u] : acc - a[u] * x[u];
        }
    }
    for (int j = j0 + 8; j < j1; j++) {
        const T v = sval[e0 + (j << 5)];
        acc = PART == 2 ? acc - s[scol[e0 + (j << 5)]] * v * v : acc - v * s[scol[e0 + (j << 5)]];
    }
    return acc;
}

// One sweep of k_dic_block over all groups of levels, ascending (DIR > 0)
// or descending, through the ring of R slots.  g0: the number of groups
// staged by the sweeps before this one (slot and barrier phase of the q-th
// group of this sweep: (g0 + q) % R and (g0 + q) / R).  PART 0: forward
// (geometry, d, the right-hand side b and entries staged; every row's
// backward start value y_i / (D_i + TINY) (Prec_Solve.f90:55-57) also
// written to t); 1: backward (geometry, d, the start values b and entries
// staged); 2: the recurrence (geometry and entries only).  START = false:
// the forward sweep leaves the start values to k_dic_scale.  lr: level
// records, gs: group table, so: slice offsets, all in shared memory.
template <typename T, int PART, int DIR, bool START = true>
__device__ __forceinline__ void dicb_sweep(T *s, unsigned char *ring, const DicbSlot &L, int R, const SellDev &A,
                                           const T *val, const T *d, const T *b, T *t, const int4 *lr,
                                           const int *gs, const int *so, int n_groups, int g0, const DicbSync &y)
{
    const int tid = threadIdx.x, W = A.width;
    int slot = g0 % R;
    unsigned ph = (unsigned)((g0 / R) & 1);   // phase parity of the slot's current use
    if (tid >= TFS_DICB_ROWS) {
        if (tid != TFS_DICB_ROWS || y.starve) return;
        // the copy lane
        int issued = 0;
        // the backward sweep stages the start values the forward sweep wrote:
        // its first group is the forward sweep's last, so wait for the
        // forward sweep's last release (use g0 - 1 of the ring)
        if (PART == 1 && g0 > 0 && !dicb_mbar_wait(y.empty + (g0 - 1) % R, (unsigned)(((g0 - 1) / R) & 1), y.abort, y.wait_ns))
            return;
        for (int q = 0; q < n_groups; q++) {
            const int g = DIR > 0 ? q : n_groups - 1 - q;
            // the slot's previous group must be done by the row threads;
            // after an abort no more copies
            if ((g0 + q >= R && !dicb_mbar_wait(y.empty + slot, ph ^ 1u, y.abort, y.wait_ns)) || *y.abort) break;
            const int4 first = lr[gs[g]], last = lr[gs[g + 1] - 1];
            const int r0 = first.x, nr = last.x + last.y - first.x;
            const int e0 = first.z, ne = last.z + last.w - first.z;
            const unsigned bytes = (unsigned)nr * (4u + (PART != 2 ? 2u * (unsigned)sizeof(T) : 0u)) +
                                   (unsigned)ne * (4u + (unsigned)sizeof(T));
            const unsigned long long chk =
                (unsigned long long)(A.rowinfo + r0) | (unsigned long long)(A.col + e0) |
                (unsigned long long)(val + e0) | (PART != 2 ? (unsigned long long)(d + r0) : 0ull) |
                (PART != 2 ? (unsigned long long)(b + r0) : 0ull) | (unsigned long long)(nr * 4) |
                (unsigned long long)(ne * 4);
            if ((chk & 15ull) || nr > L.rm || ne > L.ents) {
                *y.abort = 1;
                break;
            }
            unsigned char *sl = ring + (size_t)slot * L.bytes;
            dicb_mbar_expect(y.full + slot, bytes);
            dicb_bulk(sl, A.rowinfo + r0, nr * 4, y.full + slot);
            if (PART != 2) dicb_bulk(sl + L.off_d, d + r0, nr * (int)sizeof(T), y.full + slot);
            if (PART != 2) dicb_bulk(sl + L.off_b, b + r0, nr * (int)sizeof(T), y.full + slot);
            if (ne) {
                dicb_bulk(sl + L.off_col, A.col + e0, ne * 4, y.full + slot);
                dicb_bulk(sl + L.off_val, val + e0, ne * (int)sizeof(T), y.full + slot);
            }
            issued++;
            if (++slot == R) { slot = 0; ph ^= 1u; }
        }
        if (*y.abort) {
            // the copies of the last min(R, issued) groups may still be in
            // flight: wait for them to land (bounded; the flag is not asked)
            for (int k = 0; k < R && k < issued; k++) {
                if (--slot < 0) { slot = R - 1; ph ^= 1u; }
                const unsigned long long t0 = gtimer();
                while (!dicb_mbar_test(y.full + slot, ph) && gtimer() - t0 < y.wait_ns) {
                }
            }
        }
        return;
    }
    for (int q = 0; q < n_groups; q++) {
        const int g = DIR > 0 ? q : n_groups - 1 - q;
        const int la = gs[g], lb = gs[g + 1];
        // after an abort the slot may hold another group's rows: no row reads it
        const bool ok = dicb_mbar_wait(y.full + slot, ph, y.abort, y.wait_ns);
        const int4 first = lr[la];
        const int rg = first.x, sg = first.z;   // the group's first row and entry
        const unsigned char *sl = ring + (size_t)slot * L.bytes;
        const uint32_t *sinfo = reinterpret_cast<const uint32_t *>(sl);
        const T *sd = reinterpret_cast<const T *>(sl + L.off_d);
        const T *sb = reinterpret_cast<const T *>(sl + L.off_b);
        const int *scol = reinterpret_cast<const int *>(sl + L.off_col);
        const T *sval = reinterpret_cast<const T *>(sl + L.off_val);
        for (int lq = 0; lq < lb - la; lq++) {
            const int4 rec = lr[DIR > 0 ? la + lq : lb - 1 - lq];
            const int nr = ok ? rec.y : 0;
            for (int k = tid; k < nr; k += TFS_DICB_ROWS) {
                const int i = rec.x + k, kk = i - rg;   // row in the vector and in the slot
                const uint32_t info = sinfo[kk];
                const int len = (int)(info & 0xffffu), dpos = (int)(info >> 16);
                // entry j of the row at e0 + 32 j of the slot
                const int e0 = (W ? (kk & ~31) * W : so[i >> 5] - sg) + (kk & 31);
                if (PART == 2) {
                    if (len == 0) { s[i] = (T)1; continue; }
                    s[i] = (T)1 / dicb_row<T, 2>(sval[e0 + (dpos << 5)], s, scol, sval, e0, 0, dpos);
                } else if (PART == 0) {
                    if (len == 0) { s[i] = (T)0; continue; }
                    const T yi = dicb_row<T, 0>(sb[kk], s, scol, sval, e0, 0, dpos) * sd[kk];
                    s[i] = yi;
                    if (START) t[i] = yi / (sd[kk] + (T)TINY);   // not read by this sweep
                } else {
                    if (len == 0) { s[i] = (T)0; continue; }
                    s[i] = dicb_row<T, 1>(sb[kk], s, scol, sval, e0, dpos + 1, len) * sd[kk];
                }
            }
            // the start values written to t must be visible to the bulk
            // copies that stage them for the backward sweep
            if (PART == 0 && START && lq == lb - la - 1) asm volatile("fence.proxy.async.global;" : : : "memory");
            dicb_row_sync();   // this level's rows visible to the next
        }
        if (tid == TFS_DICB_ROWS - 32) dicb_mbar_arrive(y.empty + slot);   // done with the slot
        if (++slot == R) { slot = 0; ph ^= 1u; }
    }
}

// MODE 0: z = M^-1 b (forward sweep, scaling, backward sweep) with the
// factor d; MODE 2: the DIC factor d from the matrix (binary64; b and z
// unused); MODE 3: the forward sweep alone, z = y; MODE 4: the backward
// sweep alone from the start values in z (MODE 3, k_dic_scale, MODE 4 is
// the binary64 application: the divisions of the scaling then run on every
// SM instead of taking this block's narrow binary64 pipe).  One block of TFS_DICB_TPB threads; dynamic shared memory: the
// vector (dicb_vec_bytes), R slots of L.bytes, the level records, the group
// table (groups[0 .. n_groups]: first level of every group, then n_levels)
// and the slice-offset table (dicb_table_bytes; at most TFS_DICB_MAX_LEVELS
// levels), the ring's 2 R mbarriers and the abort flag (dicb_sync_bytes).
// Rows past lvl_begin[n_levels] (the layout's final padding) are never
// touched.
template <typename T, int MODE>
__global__ void __launch_bounds__(TFS_DICB_TPB, 1)
k_dic_block(SellDev A, const T *__restrict__ val, T *d, const T *b, T *z, const int *__restrict__ lvl_begin,
            int n_levels, const int *__restrict__ groups, int n_groups, DicbSlot L, int R, DevState *st)
{
    extern __shared__ __align__(128) unsigned char dicb_smem[];
    const int n_rows = __ldg(lvl_begin + n_levels);
    T *s = reinterpret_cast<T *>(dicb_smem);
    unsigned char *ring = dicb_smem + dicb_vec_bytes<T>(n_rows);
    int4 *lr = reinterpret_cast<int4 *>(ring + (size_t)R * L.bytes);
    int *gs = reinterpret_cast<int *>(lr + n_levels);
    int *so = gs + n_groups + 1;
    uint64_t *bars = reinterpret_cast<uint64_t *>(reinterpret_cast<unsigned char *>(lr) +
                                                  dicb_table_bytes(n_levels, n_groups, n_rows));
    const int tid = threadIdx.x;
    cudaGridDependencySynchronize();   // PDL secondary: a no-op when launched plainly
    if (st->done) return;
    const unsigned long long diag_ns = st->dicb_wait_ns;
    DicbSync y{bars, bars + R, reinterpret_cast<volatile int *>(bars + 2 * R),
               diag_ns ? diag_ns : TFS_DICB_WAIT_NS, diag_ns != 0};
    if ((MODE == 0 || MODE == 3) && tid == 0) st->t_sweep0 = gtimer();
    for (int q = tid; q <= (n_rows >> 5); q += TFS_DICB_TPB)
        so[q] = A.width ? q * 32 * A.width : __ldg(A.slice_off + q);
    for (int q = tid; q <= n_groups; q += TFS_DICB_TPB) gs[q] = __ldg(groups + q);
    __syncthreads();
    for (int l = tid; l < n_levels; l += TFS_DICB_TPB) {
        const int r0 = __ldg(lvl_begin + l), r1 = __ldg(lvl_begin + l + 1);
        lr[l] = make_int4(r0, r1 - r0, so[r0 >> 5], so[r1 >> 5] - so[r0 >> 5]);
    }
    if (tid == 0) {
        for (int k = 0; k < R; k++) {
            dicb_mbar_init(y.full + k, 1);    // the copy lane's arrival (+ the copies' bytes)
            dicb_mbar_init(y.empty + k, 1);   // one row thread's arrival
        }
        *y.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" : : : "memory");
    }
    __syncthreads();
    const bool row = tid < TFS_DICB_ROWS;
    if (MODE == 2) {
        dicb_sweep<T, 2, 1>(s, ring, L, R, A, val, d, b, nullptr, lr, gs, so, n_groups, 0, y);
        if (row)
            for (int i = tid; i < n_rows; i += TFS_DICB_ROWS) d[i] = s[i];
    } else if (MODE == 0) {
        // z holds the backward start values between the sweeps
        dicb_sweep<T, 0, 1>(s, ring, L, R, A, val, d, b, z, lr, gs, so, n_groups, 0, y);
        dicb_sweep<T, 1, -1>(s, ring, L, R, A, val, d, z, nullptr, lr, gs, so, n_groups, n_groups, y);
        if (row)
            for (int i = tid; i < n_rows; i += TFS_DICB_ROWS) z[i] = s[i];
    } else {
        if (MODE == 3)
            dicb_sweep<T, 0, 1, false>(s, ring, L, R, A, val, d, b, nullptr, lr, gs, so, n_groups, 0, y);
        else
            dicb_sweep<T, 1, -1>(s, ring, L, R, A, val, d, z, nullptr, lr, gs, so, n_groups, 0, y);
        if (row)
            for (int i = tid; i < n_rows; i += TFS_DICB_ROWS) z[i] = s[i];
    }
    __syncthreads();
    if (tid == 0 && *y.abort) {
        st->status = TFS_ERR_TIMEOUT;
        st->done = 1;
        st->niter_out = st->iter + 1;
    }
}

// The scaling between the sweeps of a split application (MODE 3 and 4 of
// k_dic_block): z_i = y_i / (D_i + TINY) for every row with entries
// (Prec_Solve.f90:55-57).
template <typename T>
__global__ void k_dic_scale(const uint32_t *__restrict__ rowinfo, const T *__restrict__ d, T *z, int n_rows,
                            const DevState *st)
{
    cudaGridDependencySynchronize();   // z is the forward sweep's
    if (st->done) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_rows; i += gridDim.x * blockDim.x)
        if (__ldg(rowinfo + i) & 0xffffu) z[i] = z[i] / (__ldg(d + i) + (T)TINY);
}

}  // namespace tfs
