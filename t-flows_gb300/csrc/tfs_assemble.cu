// tfs_assemble.cu -- matrix values assembled on the device from per-face
// coefficients through the face -> entry map (Matrix_Type%pos).
//
// The reference fills A%val face by face (NewUVW.f90:366-384,
// Compute_Pressure_Simple.f90:100-113): an interior face s between cells c1
// and c2 updates the entries (c1,c2) and (c2,c1) found through pos(1,s) and
// pos(2,s) and the two diagonals found through dia; a boundary face of a
// contributing type adds to the diagonal of c1; a cell loop then adds the
// inertial term to every diagonal (NewUVW.f90:500-505).  Every stored entry
// except the diagonal is touched by one face; a diagonal receives one
// addition per face of its cell, in face order.
//
// Here one thread owns one cell (one matrix row): it walks the faces of its
// cell in ascending face order -- a list built once per mesh on the host --
// updates the off-diagonal entries of its own row and sums its diagonal in
// exactly the reference's order, so the values are bitwise those of the
// sequential loops, and no two threads write the same entry.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "tfs_internal.h"

namespace {

// One incidence of cell c on face s: code = s << 1 | side, side 0 when c is
// the face's c1 (its entry (c1,c2) sits at pos(1,s)), 1 when c is c2.
__global__ void __launch_bounds__(256)
k_assemble_faces(int n_cells, const int *__restrict__ inc_ptr, const int *__restrict__ inc,
                 const int *__restrict__ fc2, const int *__restrict__ pos1, const int *__restrict__ pos2,
                 const int *__restrict__ dia, const double *__restrict__ off12,
                 const double *__restrict__ off21, const double *__restrict__ dia12,
                 const double *__restrict__ dia21, const double *__restrict__ cell, double *val)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += gridDim.x * blockDim.x) {
        const int dpos = __ldg(dia + c);
        double dv = val[dpos];
        const int k1 = __ldg(inc_ptr + c + 1);
        for (int k = __ldg(inc_ptr + c); k < k1; k++) {
            const int code = __ldg(inc + k), s = code >> 1;
            if ((code & 1) == 0) {
                if (__ldg(fc2 + s) > 0) {
                    const int p = __ldg(pos1 + s);
                    val[p] = val[p] - __ldg(off12 + s);
                    dv = dv + __ldg(dia12 + s);
                } else {
                    const double a = __ldg(dia12 + s);
                    if (a != 0.0) dv = dv + a;
                }
            } else {
                const int p = __ldg(pos2 + s);
                val[p] = val[p] - __ldg(off21 + s);
                dv = dv + __ldg(dia21 + s);
            }
        }
        if (cell) dv = dv + __ldg(cell + c);
        val[dpos] = dv;
    }
}

}  // namespace

struct FaceMap {
    int n_faces = 0;
    int *inc_ptr = nullptr, *inc = nullptr;     // cell -> faces, ascending
    int *fc2 = nullptr, *pos1 = nullptr, *pos2 = nullptr, *dia = nullptr;  // 0-based
    int64_t bytes = 0;
};

void tfs_faces_free(tfs_handle *h)
{
    if (!h || !h->faces) return;
    FaceMap *F = h->faces;
    for (int *p : {F->inc_ptr, F->inc, F->fc2, F->pos1, F->pos2, F->dia})
        if (p) cudaFree(p);
    h->device_bytes -= F->bytes;
    delete F;
    h->faces = nullptr;
}

extern "C" int tfs_faces_register(tfs_handle *h, int32_t n_faces, const int32_t *faces_c,
                                  const int32_t *pos1)
{
    if (!h || n_faces < 0 || (n_faces > 0 && (!faces_c || !pos1))) return TFS_ERR_ARG;
    const int n = h->n;
    // Validate against the registered topology: cell numbers in range, the
    // positions of an interior face inside the rows of c1 and c2 and off the
    // diagonal, boundary faces with c2 <= 0.
    std::vector<int> cnt(n + 1, 0);
    for (int s = 0; s < n_faces; s++) {
        const int c1 = faces_c[2 * s], c2 = faces_c[2 * s + 1];
        if (c1 < 1 || c1 > n || c2 > n) {
            tfs_set_error_text("tfs_faces_register: cell number out of range");
            return TFS_ERR_ARG;
        }
        if (c2 > 0) {
            const int p1 = pos1[2 * s] - 1, p2 = pos1[2 * s + 1] - 1;
            if (p1 < h->row0[c1 - 1] || p1 >= h->row0[c1] || p1 == h->dia0[c1 - 1] ||
                p2 < h->row0[c2 - 1] || p2 >= h->row0[c2] || p2 == h->dia0[c2 - 1]) {
                tfs_set_error_text("tfs_faces_register: pos does not match the registered topology");
                return TFS_ERR_ARG;
            }
            cnt[c2]++;
        }
        cnt[c1]++;
    }
    std::vector<int> ptr(n + 1, 0);
    for (int c = 0; c < n; c++) ptr[c + 1] = ptr[c] + cnt[c + 1];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1), inc((size_t)ptr[n] + 1, 0);
    std::vector<int> fc2(n_faces + 1, 0), p1v(n_faces + 1, -1), p2v(n_faces + 1, -1), dia(n);
    for (int s = 0; s < n_faces; s++) {   // ascending s: each list ends up sorted
        const int c1 = faces_c[2 * s], c2 = faces_c[2 * s + 1];
        fc2[s] = c2;
        inc[fill[c1 - 1]++] = s << 1;
        if (c2 > 0) {
            inc[fill[c2 - 1]++] = (s << 1) | 1;
            p1v[s] = pos1[2 * s] - 1;
            p2v[s] = pos1[2 * s + 1] - 1;
        }
    }
    for (int c = 0; c < n; c++) dia[c] = h->dia0[c];
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return tfs_engine_error(e, "cudaSetDevice");
    tfs_faces_free(h);
    FaceMap *F = new FaceMap();
    F->n_faces = n_faces;
    h->faces = F;
    auto up = [&](int **dst, const std::vector<int> &src) -> cudaError_t {
        const size_t bytes = sizeof(int) * std::max<size_t>(src.size(), 1);
        cudaError_t err = cudaMalloc((void **)dst, bytes);
        if (err != cudaSuccess) return err;
        F->bytes += (int64_t)bytes;
        h->device_bytes += (int64_t)bytes;
        return cudaMemcpyAsync(*dst, src.data(), sizeof(int) * src.size(), cudaMemcpyHostToDevice, h->stream);
    };
    if ((e = up(&F->inc_ptr, ptr)) != cudaSuccess || (e = up(&F->inc, inc)) != cudaSuccess ||
        (e = up(&F->fc2, fc2)) != cudaSuccess || (e = up(&F->pos1, p1v)) != cudaSuccess ||
        (e = up(&F->pos2, p2v)) != cudaSuccess || (e = up(&F->dia, dia)) != cudaSuccess) {
        cudaStreamSynchronize(h->stream);
        tfs_faces_free(h);
        return tfs_engine_error(e, "tfs_faces_register upload");
    }
    // The host vectors go out of scope: wait for the copies.
    e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return tfs_engine_error(e, "tfs_faces_register");
    return TFS_OK;
}

extern "C" int tfs_assemble_faces_device(tfs_handle *h, const double *d_off12, const double *d_off21,
                                         const double *d_dia12, const double *d_dia21,
                                         const double *d_cell, double *d_val)
{
    if (!h || !h->faces || !d_val) return TFS_ERR_ARG;
    FaceMap *F = h->faces;
    if (F->n_faces > 0 && (!d_off12 || !d_off21 || !d_dia12 || !d_dia21)) return TFS_ERR_ARG;
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return tfs_engine_error(e, "cudaSetDevice");
    const int n = h->n;
    int blocks = (n + 255) / 256;
    if (blocks > h->sm_count * 16) blocks = h->sm_count * 16;
    if (blocks < 1) blocks = 1;
    k_assemble_faces<<<blocks, 256, 0, h->stream>>>(n, F->inc_ptr, F->inc, F->fc2, F->pos1, F->pos2, F->dia,
                                                     d_off12, d_off21, d_dia12, d_dia21, d_cell, d_val);
    e = cudaGetLastError();
    if (e != cudaSuccess) return tfs_engine_error(e, "k_assemble_faces launch");
    return TFS_OK;
}
