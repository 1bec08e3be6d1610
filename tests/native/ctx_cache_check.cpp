// Host-only check of tfs::CtxAddrCache (t-flows_gb300/csrc/tfs_ctx_cache.h),
// the per-context cache of the no-allocation entry point's scratch address.
// Contexts are simulated by ids; prints "ok" or the first failed check.
#include <cstdio>

#include "tfs_ctx_cache.h"

static int fails = 0;
#define CHECK(c)                                                  \
    do {                                                          \
        if (!(c)) { std::printf("failed: %s\n", #c); fails++; }   \
    } while (0)

int main()
{
    tfs::CtxAddrCache<int, 4> cache;
    int a = 0, b = 0;
    int *next = &a;             // what the next lookup returns
    uint64_t current = 7;       // the "current context" id after a lookup
    int *got = nullptr;
    auto lookup = [&](int **p) { *p = next; return 0; };
    auto after = [&] { return current; };

    CHECK(cache.get(0, 7, lookup, after, &got) == 0 && got == &a && cache.lookups() == 1);
    // same device, same context: cached
    next = &b;
    CHECK(cache.get(0, 7, lookup, after, &got) == 0 && got == &a && cache.lookups() == 1);
    // another context on the same device (reset, re-retained primary, or a
    // caller's own context): looked up again
    current = 9;
    CHECK(cache.get(0, 9, lookup, after, &got) == 0 && got == &b && cache.lookups() == 2);
    CHECK(cache.get(0, 9, lookup, after, &got) == 0 && got == &b && cache.lookups() == 2);
    // the old context comes back (its id differs from the cached one)
    next = &a;
    current = 7;
    CHECK(cache.get(0, 7, lookup, after, &got) == 0 && got == &a && cache.lookups() == 3);
    // no current context known (id 0): never trusted, always looked up
    current = 0;
    CHECK(cache.get(0, 0, lookup, after, &got) == 0 && cache.lookups() == 4);
    CHECK(cache.get(0, 0, lookup, after, &got) == 0 && cache.lookups() == 5);
    // a first call with no context yet: the lookup creates one, whose id is
    // what gets cached
    current = 11;
    CHECK(cache.get(1, 0, lookup, after, &got) == 0 && cache.lookups() == 6);
    CHECK(cache.get(1, 11, lookup, after, &got) == 0 && cache.lookups() == 6);
    // devices are cached independently
    CHECK(cache.get(0, 11, lookup, after, &got) == 0 && cache.lookups() == 7);
    // a failing lookup is reported and caches nothing
    auto bad = [&](int **p) { *p = nullptr; return 5; };
    CHECK(cache.get(2, 3, bad, after, &got) == 5);
    CHECK(cache.get(2, 3, lookup, after, &got) == 0 && cache.lookups() == 8);
    // ordinal out of range
    CHECK(cache.get(4, 3, lookup, after, &got) == -1 && cache.get(-1, 3, lookup, after, &got) == -1);
    if (!fails) std::printf("ok\n");
    return fails ? 1 : 0;
}
