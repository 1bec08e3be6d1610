// Host check of the one-block DIC plan (tfs_dicb_plan.h): slot capacity and
// the grouping of levels into ring slots on synthetic level structures.
// Prints "ok" when every invariant holds.
#include <cstdio>
#include <random>
#include <vector>

#include "tfs_dicb_plan.h"

using namespace tfs;

static int fails = 0;
#define EXPECT(c)                                                        \
    do {                                                                 \
        if (!(c)) {                                                      \
            std::printf("line %d: %s\n", __LINE__, #c);                  \
            fails++;                                                     \
        }                                                                \
    } while (0)

static const int OPTIN = 232448;   // 227 KB of shared memory per block

// Levels of the given row counts, each padded to a multiple of 32 rows;
// slice widths from width(slice).
template <class Width>
static void layout(const std::vector<int> &level_rows, Width width, std::vector<int> &lvl_begin,
                   std::vector<int> &slice_off)
{
    lvl_begin.assign(1, 0);
    for (int r : level_rows) lvl_begin.push_back(lvl_begin.back() + (r + 31) / 32 * 32);
    const int slices = lvl_begin.back() / 32;
    slice_off.assign(1, 0);
    for (int s = 0; s < slices; s++) slice_off.push_back(slice_off.back() + 32 * width(s));
}

template <typename T>
static void check_plan(const std::vector<int> &lb, const std::vector<int> &so, bool want_fit)
{
    const DicbPlanResult P = dicb_plan<T>(lb, so, OPTIN, 2, 4096);
    const int nl = (int)lb.size() - 1;
    EXPECT((P.bytes > 0) == want_fit);
    if (!P.bytes) return;
    EXPECT(P.bytes <= OPTIN);
    EXPECT(P.rm % 32 == 0 && P.ents % 32 == 0);
    EXPECT(P.groups.front() == 0 && P.groups.back() == nl);
    const int ng = (int)P.groups.size() - 1;
    // the layout adds up to the plan's byte count
    EXPECT(P.bytes == dicb_vec_bytes<T>(lb[nl]) + 2 * dicb_slot<T>(P.rm, P.ents).bytes +
                          dicb_table_bytes(nl, ng, lb[nl]) + dicb_sync_bytes(2));
    for (int g = 0; g < ng; g++) {
        const int a = P.groups[g], b = P.groups[g + 1];
        EXPECT(a < b);
        const int rows = lb[b] - lb[a], ents = so[lb[b] >> 5] - so[lb[a] >> 5];
        EXPECT(rows <= P.rm && ents <= P.ents);
        // greedy: the next level would not have fitted
        if (b < nl) {
            const int rows2 = lb[b + 1] - lb[a], ents2 = so[lb[b + 1] >> 5] - so[lb[a] >> 5];
            EXPECT(rows2 > P.rm || ents2 > P.ents);
        }
    }
}

int main()
{
    std::vector<int> lb, so;
    std::mt19937 rng(7);
    // deep schedule of narrow levels (a 14,490-cell mesh in its own
    // numbering: 148 levels of at most 149 rows), uniform width 7
    std::vector<int> deep;
    for (int l = 0; l < 148; l++) deep.push_back(1 + (int)(rng() % 149));
    layout(deep, [](int) { return 7; }, lb, so);
    check_plan<double>(lb, so, true);
    check_plan<float>(lb, so, true);
    // per-slice widths 4..8
    layout(deep, [&](int s) { return 4 + (s * 7919) % 5; }, lb, so);
    check_plan<double>(lb, so, true);
    check_plan<float>(lb, so, true);
    // wide levels (a randomly numbered 24^3 system: 15 levels of up to 2074
    // rows): two slots of the widest level do not fit beside the vector
    layout({2074, 1900, 1800, 1500, 1200, 1000, 900, 800, 700, 600, 500, 400, 300, 200, 100},
           [](int) { return 7; }, lb, so);
    check_plan<double>(lb, so, false);
    // a vector that does not fit at all (40^3 rows in binary64)
    layout(std::vector<int>(100, 640), [](int) { return 7; }, lb, so);
    check_plan<double>(lb, so, false);
    // more levels than the kernel takes
    layout(std::vector<int>(4097, 1), [](int) { return 7; }, lb, so);
    check_plan<float>(lb, so, false);
    // one level
    layout({96}, [](int) { return 7; }, lb, so);
    check_plan<double>(lb, so, true);
    if (fails) return 1;
    std::printf("ok\n");
    return 0;
}
