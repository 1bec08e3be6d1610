// tfs_topology.cpp -- host construction of the T-FlowS compressed-row topology.
//
// Produces the arrays of Matrix_Mod_Topology (Sources/Process/Matrix_Mod/
// Topology.f90:2-127): row starts, ascending column numbers per row, the
// diagonal position, the mirror (transpose) position of every entry and the
// face -> entry map pos(1:2, s).  All outputs are 1-based like the Fortran.
//
// The reference fills each row in face order, sorts it with a quicksort and
// finds the mirror entry by a linear search of the neighbour's row
// (O(nnz * row length)).  Here each row is a short insertion sort (the keys
// of a row are distinct, so any ascending sort gives the same row) and mirror
// and face positions are binary searches in the sorted rows.  The result is
// identical entry for entry.
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "../../include/tfs_solver.h"

namespace {

// Position (1-based) of column c in the sorted row r, or 0 if absent.
inline int32_t find_in_row(const int32_t *row1, const int32_t *col1, int32_t r,
                           int32_t c)
{
    int32_t lo = row1[r - 1], hi = row1[r] - 1;  // 1-based positions
    while (lo <= hi) {
        int32_t mid = lo + (hi - lo) / 2;
        int32_t v = col1[mid - 1];
        if (v == c) return mid;
        if (v < c) lo = mid + 1; else hi = mid - 1;
    }
    return 0;
}

}  // namespace

extern "C" int32_t tfs_topology_count(int32_t n_cells, int32_t n_faces,
                                      const int32_t *faces_c)
{
    if (n_cells < 0 || n_faces < 0 || (n_faces > 0 && !faces_c)) return -1;
    int64_t n = n_cells;
    for (int32_t s = 0; s < n_faces; s++)
        if (faces_c[2 * s + 1] > 0) n += 2;
    if (n > INT32_MAX - 1) return -1;
    return (int32_t)n;
}

extern "C" int tfs_topology_build(int32_t n_cells, int32_t n_faces,
                                  const int32_t *faces_c, int32_t *row1,
                                  int32_t *col1, int32_t *dia1, int32_t *mir1,
                                  int32_t *pos1)
{
    if (n_cells <= 0 || n_faces < 0 || !row1 || !col1 || !dia1) return TFS_ERR_ARG;
    if (n_faces > 0 && !faces_c) return TFS_ERR_ARG;
    // Stencil width per cell (Topology.f90:33-41), validating cell numbers.
    std::vector<int32_t> fill((size_t)n_cells, 1);
    for (int32_t s = 0; s < n_faces; s++) {
        int32_t c1 = faces_c[2 * s], c2 = faces_c[2 * s + 1];
        if (c1 < 1 || c1 > n_cells || c2 > n_cells) return TFS_ERR_MATRIX;
        if (c2 > 0) { fill[c1 - 1]++; fill[c2 - 1]++; }
    }
    row1[0] = 1;
    for (int32_t c = 0; c < n_cells; c++) row1[c + 1] = row1[c] + fill[c];
    // Diagonal first, then neighbours in face order (Topology.f90:54-71).
    for (int32_t c = 0; c < n_cells; c++) {
        col1[row1[c] - 1] = c + 1;
        fill[c] = 1;
    }
    for (int32_t s = 0; s < n_faces; s++) {
        int32_t c1 = faces_c[2 * s], c2 = faces_c[2 * s + 1];
        if (c2 > 0) {
            col1[row1[c1 - 1] - 1 + fill[c1 - 1]++] = c2;
            col1[row1[c2 - 1] - 1 + fill[c2 - 1]++] = c1;
        }
    }
    // Sort rows, locate the diagonal (Topology.f90:75-82).
    for (int32_t c = 0; c < n_cells; c++) {
        int32_t *x = col1 + (row1[c] - 1);
        int32_t len = row1[c + 1] - row1[c];
        for (int32_t a = 1; a < len; a++) {
            int32_t v = x[a], b = a - 1;
            while (b >= 0 && x[b] > v) { x[b + 1] = x[b]; b--; }
            x[b + 1] = v;
        }
        for (int32_t p = 0; p < len; p++)
            if (x[p] == c + 1) dia1[c] = row1[c] + p;
    }
    // Mirror positions (Topology.f90:85-103).
    if (mir1) {
        for (int32_t c = 0; c < n_cells; c++)
            for (int32_t p = row1[c]; p < row1[c + 1]; p++)
                mir1[p - 1] = find_in_row(row1, col1, col1[p - 1], c + 1);
    }
    // Face -> entry positions (Topology.f90:106-121).
    if (pos1) {
        for (int32_t s = 0; s < n_faces; s++) {
            int32_t c1 = faces_c[2 * s], c2 = faces_c[2 * s + 1];
            if (c2 > 0) {
                pos1[2 * s] = find_in_row(row1, col1, c1, c2);
                pos1[2 * s + 1] = find_in_row(row1, col1, c2, c1);
            } else {
                pos1[2 * s] = 0;
                pos1[2 * s + 1] = 0;
            }
        }
    }
    return TFS_OK;
}
