/*
 * tfs_synth.h -- seeded synthetic finite-volume systems used by the benchmark
 * and the parity tests.  Host code only, in its own library libtfs_synth.so
 * (tfs_synth.cpp with the host topology builder it calls), so that a process
 * that only needs the inputs never loads the GPU solver library.
 *
 * A system is an nx*ny*nz hexahedral mesh of cell size h = 1/nx on
 * [0,1]x[0,ny/nx]x[0,nz/nx], interior nodes jittered by U(-j*h, j*h) per
 * coordinate, cells renumbered by a seeded random permutation.  Geometry
 * follows the reference generator's formulas: face area vector by the polygon
 * formula (Sources/Generate/Compute_Grid_Geometry.f90:189-213), face centre
 * = node average (:240-245), cell centre = node average (:134-139); cell
 * volume by the divergence theorem V = 1/3 sum_f x_f . S_f.  The CSR topology
 * is built by tfs_topology_build (Matrix_Mod/Topology.f90 semantics) and the
 * values are assembled face by face through pos/dia as the reference does
 * (Compute_Pressure_Simple.f90:100-107, NewUVW.f90:361-370).
 *
 * Kinds:
 *   TFS_SYNTH_POISSON   a_f = |S_f|/|x_c2 - x_c1| off-diagonal -a_f, diagonal
 *                       sum a_f; Dirichlet on x = 0 adds |S_b|/|x_fb - x_c|.
 *   TFS_SYNTH_CONVDIFF  diffusion nu*a_f (nu = 1e-3) plus first-order upwind
 *                       convection by the Taylor-Green field
 *                       u = U0 sin(2 pi x) cos(2 pi y) cos(2 pi z),
 *                       v = -U0 cos(2 pi x) sin(2 pi y) cos(2 pi z), w = 0,
 *                       U0 = 10 nu / h (cell Peclet <= 10), plus V/dt on the
 *                       diagonal with dt = 0.5 h / U0 (CFL 0.5).  Zero flux on
 *                       every wall (the field is tangential there).
 * RHS: U(-1, 1) per cell.  All random numbers come from a counter-based
 * generator (seed, stream, index), so a system is identical on every host.
 */
#ifndef TFS_SYNTH_H
#define TFS_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TFS_SYNTH_POISSON  0
#define TFS_SYNTH_CONVDIFF 1

typedef struct tfs_synth tfs_synth;

/* Build a system.  jitter is the fraction of h (0.2 = +-20%).  permute != 0
 * applies the seeded random cell renumbering. */
int tfs_synth_create(int kind, int32_t nx, int32_t ny, int32_t nz,
                     double jitter, uint64_t seed, int permute,
                     tfs_synth **out);

/* n = cells, nnz = stored entries, n_faces = interior faces. */
int tfs_synth_dims(const tfs_synth *s, int32_t *n, int32_t *nnz,
                   int32_t *n_faces);

/* Copy out the system.  Any pointer may be NULL to skip that array.
 * faces_c: 2*n_faces; row1: n+1; col1, val: nnz; dia1, b: n. */
int tfs_synth_export(const tfs_synth *s, int32_t *faces_c, int32_t *row1,
                     int32_t *col1, int32_t *dia1, double *val, double *b);

void tfs_synth_free(tfs_synth *s);

/* Deterministic log-uniform integer in [lo, hi] for (seed, index), the size
 * draw of the batched and serving workloads. */
int64_t tfs_synth_loguniform(int64_t lo, int64_t hi, uint64_t seed,
                             uint64_t index);

/* Deterministic uniform double in [0, 1) for (seed, stream, index). */
double tfs_synth_uniform(uint64_t seed, uint64_t stream, uint64_t index);

#ifdef __cplusplus
}
#endif
#endif /* TFS_SYNTH_H */
