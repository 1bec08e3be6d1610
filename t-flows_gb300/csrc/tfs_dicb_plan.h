// tfs_dicb_plan.h -- the shared-memory layout of the one-block DIC
// (k_dic_block, tfs_dic_block.cuh) and its host-side plan: how large a ring
// slot is and which consecutive levels share one.  No CUDA calls: the engine
// includes it, and the host compiler builds it on its own for the tests.
//
// Dynamic shared memory of one launch, in order: the swept vector (one value
// per row of the levels), R ring slots, the level records (one int4 per
// level), the group table (first level of every group, then the level
// count), the slice-offset table, the ring's 2 R mbarriers and the abort
// flag.  The slots share what the vector and the tables leave, rows and
// entries in the widest level's proportion; a slot must hold the widest
// level (else the one-block DIC does not run: the level kernels do).  Groups
// are filled greedily in level order.
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

#ifdef __CUDACC__
#define TFS_DICB_HD __host__ __device__
#else
#define TFS_DICB_HD
#endif

namespace tfs {

// Byte offsets inside one ring slot of `rm` rows and `ents` SELL entries
// (rm and ents multiples of 32, so every part starts on a 128-byte
// boundary): geometry, diagonal, right-hand side, column indices and values
// of one group of levels.
struct DicbSlot {
    int rm, ents, off_d, off_b, off_col, off_val, bytes;
};

template <typename T>
TFS_DICB_HD inline DicbSlot dicb_slot(int rm, int ents)
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
TFS_DICB_HD inline int dicb_vec_bytes(int n_rows)
{
    return (n_rows * (int)sizeof(T) + 127) & ~127;
}

// Shared memory of the level records (one int4 per level: first row, rows,
// first SELL entry, entries), the group table (first level of every group,
// n_groups + 1 ints) and the slice-offset table (n_rows / 32 + 1 ints),
// rounded to 16 bytes.
TFS_DICB_HD inline int dicb_table_bytes(int n_levels, int n_groups, int n_rows)
{
    return n_levels * 16 + (((n_groups + 1) + (n_rows >> 5) + 1) * 4 + 15) / 16 * 16;
}

// Shared memory of the ring's R full and R empty mbarriers and the abort
// flag.
TFS_DICB_HD inline int dicb_sync_bytes(int R)
{
    return 2 * R * 8 + 16;
}

// The plan for one arithmetic: dynamic shared memory of a launch (0: the
// one-block DIC does not run), slot capacity in rows and entries, and the
// group table (first level of every group, then n_levels).
struct DicbPlanResult {
    int bytes = 0, rm = 0, ents = 0;
    std::vector<int> groups;
};

// lvl_begin: n_levels + 1 internal row offsets (levels start on slice
// boundaries); slice_off: SELL-32 slice starts (entry offsets); optin: the
// device's shared memory per block; R: ring slots; max_levels: the kernel's
// level limit.
template <typename T>
inline DicbPlanResult dicb_plan(const std::vector<int> &lvl_begin, const std::vector<int> &slice_off, int optin,
                                int R, int max_levels)
{
    DicbPlanResult P;
    const int nl = (int)lvl_begin.size() - 1;
    if (nl < 1 || nl > max_levels || lvl_begin[nl] > (1 << 24)) return P;
    const int rows = lvl_begin[nl];
    auto lvl_ents = [&](int l) { return slice_off[lvl_begin[l + 1] >> 5] - slice_off[lvl_begin[l] >> 5]; };
    int rm = 32, ents = 32;
    for (int l = 0; l < nl; l++) {
        rm = std::max(rm, lvl_begin[l + 1] - lvl_begin[l]);
        ents = std::max(ents, lvl_ents(l));
    }
    const int64_t room =
        (int64_t)optin - dicb_vec_bytes<T>(rows) - dicb_table_bytes(nl, nl, rows) - dicb_sync_bytes(R);
    const int64_t widest = dicb_slot<T>(rm, ents).bytes;
    if (room < R * widest) return P;
    const double k = (double)(room / R) / (double)widest;   // >= 1
    const int rm_c = std::max(rm, (int)(rm * k) & ~31), ents_c = std::max(ents, (int)(ents * k) & ~31);
    const int slot = dicb_slot<T>(rm_c, ents_c).bytes;
    if (slot > room / R) return P;
    P.groups.push_back(0);
    int gr = 0, ge = 0;
    for (int l = 0; l < nl; l++) {
        const int lrows = lvl_begin[l + 1] - lvl_begin[l], lents = lvl_ents(l);
        if (l > 0 && (gr + lrows > rm_c || ge + lents > ents_c)) {
            P.groups.push_back(l);
            gr = ge = 0;
        }
        gr += lrows;
        ge += lents;
    }
    P.groups.push_back(nl);
    const int ng = (int)P.groups.size() - 1;
    P.rm = rm_c;
    P.ents = ents_c;
    P.bytes = dicb_vec_bytes<T>(rows) + R * slot + dicb_table_bytes(nl, ng, rows) + dicb_sync_bytes(R);
    return P;
}

}  // namespace tfs
