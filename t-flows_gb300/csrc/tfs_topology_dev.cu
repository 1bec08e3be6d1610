// tfs_topology_dev.cu -- Matrix_Mod_Topology on the device.
//
// The reference builds the compressed-row topology of its matrix once per
// mesh on the host (Matrix_Mod/Topology.f90:2-127): stencil widths from the
// faces (:33-41), row starts with the diagonal first (:54-59), off-diagonal
// columns in face order (:62-71), every row sorted ascending and its
// diagonal located (:75-82), the mirror position of every entry (:85-103)
// and the two entry positions of every interior face (:106-121).  The same
// arrays come out of this file, bit for bit, built on the device:
//
//   k_topo_width/count  stencil widths (integer atomics: the counts, not
//                       their order, are the result)
//   k_scan_*            row starts: exclusive prefix sum of the widths (a
//                       three-pass scan: per block, block totals, add back)
//   k_topo_fill         the diagonal, then each face's two off-diagonal
//                       entries in slots taken with integer atomics
//   k_topo_sort         each row sorted ascending by one thread (a row holds
//                       distinct cell numbers, so the sorted row is unique
//                       whatever order the slots were filled in) and its
//                       diagonal located
//   k_topo_mir          mir(p) by a search of the mirrored row
//   k_topo_pos          pos(1:2,s) by searches of the rows of c1 and c2
//
// The faces must join distinct pairs of distinct cells (each stored entry
// then belongs to exactly one face side), as meshes from the reference's
// generators do; every array is 1-based, as in the reference.
#include <cuda_runtime.h>

#include <cstdint>

#include "tfs_internal.h"

namespace {

constexpr int kTB = 256;

__global__ void k_topo_width(int n_cells, int *width)
{
    for (int c = blockIdx.x * kTB + threadIdx.x; c < n_cells; c += gridDim.x * kTB) width[c] = 1;
}

__global__ void k_topo_count(int n_faces, const int *__restrict__ fc, int *width)
{
    for (int s = blockIdx.x * kTB + threadIdx.x; s < n_faces; s += gridDim.x * kTB) {
        const int c1 = fc[2 * s], c2 = fc[2 * s + 1];
        if (c2 > 0) {
            atomicAdd(width + c1 - 1, 1);
            atomicAdd(width + c2 - 1, 1);
        }
    }
}

// Exclusive scan, pass 1: each block scans kTB * 4 elements and writes its
// total.
__global__ void k_scan_block(int n, const int *__restrict__ in, int *out, int *block_sum)
{
    __shared__ int sm[kTB];
    const int base = blockIdx.x * kTB * 4;
    int v[4], t = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int i = base + threadIdx.x * 4 + q;
        v[q] = i < n ? in[i] : 0;
        t += v[q];
    }
    sm[threadIdx.x] = t;
    __syncthreads();
    for (int o = 1; o < kTB; o <<= 1) {   // inclusive scan of the thread totals
        const int a = threadIdx.x >= o ? sm[threadIdx.x - o] : 0;
        __syncthreads();
        sm[threadIdx.x] += a;
        __syncthreads();
    }
    int run = sm[threadIdx.x] - t;        // exclusive prefix of this thread
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int i = base + threadIdx.x * 4 + q;
        if (i < n) out[i] = run;
        run += v[q];
    }
    if (threadIdx.x == kTB - 1) block_sum[blockIdx.x] = sm[kTB - 1];
}

// Pass 2 (one block, chunk after chunk): exclusive scan of the block totals
// in place; *total receives the grand total.
__global__ void k_scan_totals(int nb, int *block_sum, int *total)
{
    __shared__ int sm[kTB];
    int carry = 0;
    for (int b0 = 0; b0 < nb; b0 += kTB) {
        const int b = b0 + threadIdx.x;
        const int v = b < nb ? block_sum[b] : 0;
        sm[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kTB; o <<= 1) {
            const int a = threadIdx.x >= o ? sm[threadIdx.x - o] : 0;
            __syncthreads();
            sm[threadIdx.x] += a;
            __syncthreads();
        }
        if (b < nb) block_sum[b] = carry + sm[threadIdx.x] - v;
        const int chunk = sm[kTB - 1];
        __syncthreads();
        carry += chunk;
    }
    if (threadIdx.x == 0) *total = carry;
}

// Pass 3: row(c) = 1 + exclusive prefix; row(n+1) = 1 + total.  The slot
// counters restart at 1 (the diagonal takes slot 0).
__global__ void k_scan_add(int n, const int *__restrict__ excl, const int *__restrict__ block_sum,
                           const int *__restrict__ total, int *row1, int *slot)
{
    for (int i = blockIdx.x * kTB + threadIdx.x; i <= n; i += gridDim.x * kTB) {
        if (i < n) {
            row1[i] = 1 + excl[i] + block_sum[i / (kTB * 4)];
            slot[i] = 1;
        } else {
            row1[n] = 1 + *total;
        }
    }
}

__global__ void k_topo_fill(int n_cells, int n_faces, const int *__restrict__ fc,
                            const int *__restrict__ row1, int *slot, int *col1)
{
    const int tid = blockIdx.x * kTB + threadIdx.x, stride = gridDim.x * kTB;
    for (int c = tid; c < n_cells; c += stride) col1[row1[c] - 1] = c + 1;
    for (int s = tid; s < n_faces; s += stride) {
        const int c1 = fc[2 * s], c2 = fc[2 * s + 1];
        if (c2 > 0) {
            col1[row1[c1 - 1] - 1 + atomicAdd(slot + c1 - 1, 1)] = c2;
            col1[row1[c2 - 1] - 1 + atomicAdd(slot + c2 - 1, 1)] = c1;
        }
    }
}

__global__ void k_topo_sort(int n_cells, const int *__restrict__ row1, int *col1, int *dia1)
{
    for (int c = blockIdx.x * kTB + threadIdx.x; c < n_cells; c += gridDim.x * kTB) {
        const int b = row1[c] - 1, e = row1[c + 1] - 1;
        for (int a = b + 1; a < e; a++) {
            const int v = col1[a];
            int k = a - 1;
            while (k >= b && col1[k] > v) { col1[k + 1] = col1[k]; k--; }
            col1[k + 1] = v;
        }
        for (int p = b; p < e; p++)
            if (col1[p] == c + 1) dia1[c] = p + 1;
    }
}

__global__ void k_topo_mir(int n_cells, const int *__restrict__ row1, const int *__restrict__ col1, int *mir1)
{
    for (int c = blockIdx.x * kTB + threadIdx.x; c < n_cells; c += gridDim.x * kTB) {
        for (int p1 = row1[c] - 1; p1 < row1[c + 1] - 1; p1++) {
            const int c2 = col1[p1] - 1;
            int m = 0;
            for (int p2 = row1[c2] - 1; p2 < row1[c2 + 1] - 1; p2++)
                if (col1[p2] == c + 1) { m = p2 + 1; break; }
            mir1[p1] = m;
        }
    }
}

__global__ void k_topo_pos(int n_faces, const int *__restrict__ fc, const int *__restrict__ row1,
                           const int *__restrict__ col1, int *pos1)
{
    for (int s = blockIdx.x * kTB + threadIdx.x; s < n_faces; s += gridDim.x * kTB) {
        const int c1 = fc[2 * s], c2 = fc[2 * s + 1];
        int a = 0, b = 0;
        if (c2 > 0) {
            for (int p = row1[c1 - 1] - 1; p < row1[c1] - 1; p++)
                if (col1[p] == c2) a = p + 1;
            for (int p = row1[c2 - 1] - 1; p < row1[c2] - 1; p++)
                if (col1[p] == c1) b = p + 1;
        }
        pos1[2 * s] = a;
        pos1[2 * s + 1] = b;
    }
}

// Faces are checked before anything is built: 1 <= c1 <= n_cells,
// c2 <= n_cells, c1 != c2.  Any violation sets *bad.
__global__ void k_topo_check(int n_cells, int n_faces, const int *__restrict__ fc, int *bad)
{
    for (int s = blockIdx.x * kTB + threadIdx.x; s < n_faces; s += gridDim.x * kTB) {
        const int c1 = fc[2 * s], c2 = fc[2 * s + 1];
        if (c1 < 1 || c1 > n_cells || c2 > n_cells || c2 == c1) atomicOr(bad, 1);
    }
}

}  // namespace

extern "C" int tfs_topology_build_device(int32_t n_cells, int32_t n_faces, const int32_t *d_faces_c,
                                         int32_t *d_row1, int32_t *d_col1, int32_t *d_dia1,
                                         int32_t *d_mir1, int32_t *d_pos1, int32_t *nnz_out)
{
    if (n_cells <= 0 || n_faces < 0 || !d_row1 || !d_col1 || !d_dia1 || !d_mir1 || !nnz_out ||
        (n_faces > 0 && (!d_faces_c || !d_pos1)))
        return TFS_ERR_ARG;
    if ((int64_t)n_cells + 2 * (int64_t)n_faces > INT32_MAX) return TFS_ERR_ARG;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return tfs_engine_error(e, "cudaGetDevice");
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return tfs_engine_error(e, "cudaDeviceGetAttribute");
    auto grid = [&](int64_t items) {
        int64_t b = (items + kTB - 1) / kTB;
        if (b > (int64_t)sms * 16) b = (int64_t)sms * 16;
        return (int)(b < 1 ? 1 : b);
    };
    const int nb = (n_cells + kTB * 4 - 1) / (kTB * 4);
    // scratch: widths then slots (n), exclusive prefixes (n), block totals
    // (nb), the grand total, the error flag
    int *scr = nullptr;
    const size_t words = 2 * (size_t)n_cells + (size_t)nb + 2;
    e = cudaMalloc((void **)&scr, sizeof(int) * words);
    if (e != cudaSuccess) return tfs_engine_error(e, "cudaMalloc (topology scratch)");
    int *width = scr, *excl = scr + n_cells, *bsum = excl + n_cells, *total = bsum + nb, *bad = total + 1;
    int h_bad = 0, h_total = 0;
    e = cudaMemset(bad, 0, sizeof(int));
    if (e == cudaSuccess && n_faces > 0) k_topo_check<<<grid(n_faces), kTB>>>(n_cells, n_faces, d_faces_c, bad);
    if (e == cudaSuccess) e = cudaMemcpy(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        cudaFree(scr);
        return tfs_engine_error(e, "topology check");
    }
    if (h_bad) {
        cudaFree(scr);
        tfs_set_error_text("tfs_topology_build_device: a face has a cell number out of range or c1 == c2");
        return TFS_ERR_TOPOLOGY;
    }
    k_topo_width<<<grid(n_cells), kTB>>>(n_cells, width);
    if (n_faces > 0) k_topo_count<<<grid(n_faces), kTB>>>(n_faces, d_faces_c, width);
    k_scan_block<<<nb, kTB>>>(n_cells, width, excl, bsum);
    k_scan_totals<<<1, kTB>>>(nb, bsum, total);
    k_scan_add<<<grid((int64_t)n_cells + 1), kTB>>>(n_cells, excl, bsum, total, d_row1, width);
    e = cudaMemcpy(&h_total, total, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) {
        k_topo_fill<<<grid(n_cells > n_faces ? n_cells : n_faces), kTB>>>(n_cells, n_faces, d_faces_c, d_row1,
                                                                        width, d_col1);
        k_topo_sort<<<grid(n_cells), kTB>>>(n_cells, d_row1, d_col1, d_dia1);
        k_topo_mir<<<grid(n_cells), kTB>>>(n_cells, d_row1, d_col1, d_mir1);
        if (n_faces > 0) k_topo_pos<<<grid(n_faces), kTB>>>(n_faces, d_faces_c, d_row1, d_col1, d_pos1);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    cudaFree(scr);
    if (e != cudaSuccess) return tfs_engine_error(e, "tfs_topology_build_device");
    *nnz_out = h_total;
    return TFS_OK;
}
