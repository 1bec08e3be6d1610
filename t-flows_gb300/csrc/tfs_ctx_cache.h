// tfs_ctx_cache.h -- a device address cached per CUDA context.
//
// The address of a __device__ variable belongs to the CUDA context the
// module was loaded into, not to the device ordinal: after cudaDeviceReset,
// after the primary context was released and retained again, or under a
// context the caller created itself, the same ordinal has another context
// and the old address is stale.  CtxAddrCache keeps, per device ordinal, the
// address together with the unique id of the context it was looked up in,
// and looks the address up again whenever the current context's id differs
// (or is unknown, reported as 0).  Host code only; no CUDA calls here -- the
// caller passes the current context id and a lookup function.
#pragma once
#include <cstdint>
#include <mutex>

namespace tfs {

template <typename T, int MAX_DEVICES = 64>
class CtxAddrCache {
public:
    // *out = the address for (dev, ctx_id).  `lookup(T **)` returns 0 on
    // success; `ctx_after()` gives the current context id once the lookup ran
    // (a lookup may itself create the device's primary context).  Returns
    // lookup's status, or -1 for a device ordinal out of range.
    template <class Lookup, class CtxAfter>
    int get(int dev, uint64_t ctx_id, Lookup lookup, CtxAfter ctx_after, T **out)
    {
        if (dev < 0 || dev >= MAX_DEVICES) return -1;
        std::lock_guard<std::mutex> lk(mu_);
        Entry &e = e_[dev];
        if (ctx_id != 0 && e.addr && e.ctx == ctx_id) {
            *out = e.addr;
            return 0;
        }
        T *p = nullptr;
        int rc = lookup(&p);
        if (rc) return rc;
        e.addr = p;
        e.ctx = ctx_after();
        lookups_++;
        *out = p;
        return 0;
    }
    long lookups() const { return lookups_; }

private:
    struct Entry {
        uint64_t ctx = 0;
        T *addr = nullptr;
    };
    std::mutex mu_;
    Entry e_[MAX_DEVICES];
    long lookups_ = 0;
};

}  // namespace tfs
