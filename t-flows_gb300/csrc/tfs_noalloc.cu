// tfs_noalloc.cu -- residual and its norm without any device allocation.
//
// Some callers of this library cannot allocate device memory when they call
// it: a flow solver that runs inside a host framework which hands it a fixed
// device arena, code that issues work while another thread is capturing a
// CUDA graph (cudaMalloc is not allowed there), or a real-time coupling loop
// that must never block in the allocator.  tfs_residual_norm_noalloc serves
// them: it computes r1 <- r1 - A x with the reference's per-row arithmetic
// (Residual.f90:22-27) and ||r1||_2 from arrays the caller already holds on
// the device, and it allocates nothing.  Its only scratch is the file-scope
// array below (one partial sum per 256-row block plus an arrival counter),
// which every GPU that loads the library keeps until the process exits.
//
// Host code cannot hand the array's name to a kernel (on the host it is a
// stand-in, not a device address), so the address is looked up with
// cudaGetSymbolAddress and cached per CUDA context (tfs_ctx_cache.h): a
// call under another context than the cached one -- after cudaDeviceReset,
// after the primary context was released and retained again, or in a
// context the caller created -- looks it up again in that context.  The
// lookup of a context's first call is the only set-up; it should come
// before any stream capture.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "tfs_ctx_cache.h"
#include "tfs_internal.h"

namespace {

constexpr int kRows = 256;                         // rows per block
constexpr int kMaxBlocks = TFS_NOALLOC_MAX_ROWS / kRows;

struct NoallocScratch {
    double part[kMaxBlocks];   // one partial of ||r||^2 per block
    unsigned int counter;      // blocks that have published their partial
};

static __device__ __align__(256) NoallocScratch g_scratch;

// Device address of g_scratch per device ordinal and context.
tfs::CtxAddrCache<NoallocScratch> g_cache;

// Unique id + 1 of the calling thread's current CUDA context, 0 when there
// is none or the driver cannot say.  The driver entry points come through
// the runtime, so the library does not link the driver library.
uint64_t current_context_id()
{
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static GetCurrent get_cur = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = (GetCurrent)p;
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (GetId)p;
        cudaGetLastError();
    });
    if (!get_cur || !get_id) return 0;
    CUcontext c = nullptr;
    if (get_cur(&c) != CUDA_SUCCESS || !c) return 0;
    unsigned long long id = 0;
    if (get_id(c, &id) != CUDA_SUCCESS) return 0;
    return (uint64_t)id + 1;
}

// r1 <- r1 - A x for 1-based CSR, one row per thread, and the norm.
__global__ void __launch_bounds__(kRows)
k_residual_norm_noalloc(int n, const int32_t *__restrict__ row1, const int32_t *__restrict__ col1,
                        const double *__restrict__ val, const double *__restrict__ x,
                        double *__restrict__ r1, double *__restrict__ norm, NoallocScratch *scr)
{
    const int i = blockIdx.x * kRows + threadIdx.x;
    double e2 = 0.0;
    if (i < n) {
        double r = r1[i];
        for (int j = row1[i] - 1; j < row1[i + 1] - 1; j++) r = r - val[j] * x[col1[j] - 1];
        r1[i] = r;
        e2 = r * r;
    }
    __shared__ double sm[kRows / 32];
    __shared__ unsigned int is_last;
    for (int o = 16; o > 0; o >>= 1) e2 = e2 + __shfl_down_sync(0xffffffffu, e2, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = e2;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = sm[0];
        for (int w = 1; w < kRows / 32; w++) s = s + sm[w];
        scr->part[blockIdx.x] = s;
        __threadfence();
        is_last = (atomicAdd(&scr->counter, 1u) == gridDim.x - 1) ? 1u : 0u;
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    // The last block sums the partials in block order.
    double a = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kRows) a = a + __ldcg(scr->part + b);
    __syncthreads();
    for (int o = 16; o > 0; o >>= 1) a = a + __shfl_down_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = sm[0];
        for (int w = 1; w < kRows / 32; w++) s = s + sm[w];
        *norm = sqrt(s);
        scr->counter = 0u;
    }
}

}  // namespace

extern "C" int tfs_residual_norm_noalloc(int32_t n, const int32_t *d_row1, const int32_t *d_col1,
                                         const double *d_val, const double *d_x, double *d_r1,
                                         double *d_norm, void *stream)
{
    if (n <= 0) {
        tfs_set_error_text("tfs_residual_norm_noalloc: n must be positive");
        return TFS_ERR_ARG;
    }
    if (!d_row1 || !d_col1 || !d_val || !d_x || !d_r1 || !d_norm) {
        tfs_set_error_text("tfs_residual_norm_noalloc: a device array is NULL");
        return TFS_ERR_ARG;
    }
    if (n > TFS_NOALLOC_MAX_ROWS) {
        tfs_set_error_text("tfs_residual_norm_noalloc: n exceeds TFS_NOALLOC_MAX_ROWS (4,194,304 rows)");
        return TFS_ERR_ARG;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return tfs_engine_error(e, "cudaGetDevice");
    NoallocScratch *scr = nullptr;
    cudaError_t le = cudaSuccess;
    const int rc = g_cache.get(
        dev, current_context_id(),
        [&](NoallocScratch **p) {
            void *a = nullptr;
            le = cudaGetSymbolAddress(&a, g_scratch);
            *p = (NoallocScratch *)a;
            return le == cudaSuccess ? 0 : 1;
        },
        [] { return current_context_id(); }, &scr);
    if (rc == -1) {
        tfs_set_error_text("tfs_residual_norm_noalloc: device ordinal beyond 63");
        return TFS_ERR_ARG;
    }
    if (rc) return tfs_engine_error(le, "cudaGetSymbolAddress");
    cudaStream_t s = (cudaStream_t)stream;
    // The counter starts at zero for every call (a failed earlier call may
    // have left it elsewhere); the partials are all rewritten before use.
    e = cudaMemsetAsync(&scr->counter, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return tfs_engine_error(e, "cudaMemsetAsync");
    const int blocks = (n + kRows - 1) / kRows;
    k_residual_norm_noalloc<<<blocks, kRows, 0, s>>>(n, d_row1, d_col1, d_val, d_x, d_r1, d_norm, scr);
    e = cudaGetLastError();
    if (e != cudaSuccess) return tfs_engine_error(e, "k_residual_norm_noalloc launch");
    return TFS_OK;
}
