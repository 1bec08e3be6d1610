// tfs_synth.cpp -- seeded synthetic finite-volume systems (see tfs_synth.h).
//
// Every floating-point operation here is a separately rounded IEEE add, mul,
// div or sqrt (the library is compiled with -ffp-contract=off), and the
// trigonometric/exponential functions are the series below rather than the
// platform libm, so the same (kind, sizes, jitter, seed) gives bit-identical
// systems on x86-64 and AArch64 hosts.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/tfs_solver.h"
#include "../../include/tfs_synth.h"

struct tfs_synth {
    int32_t n = 0, nnz = 0, n_faces = 0;
    std::vector<int32_t> faces_c, row1, col1, dia1;
    std::vector<double> val, b;
};

namespace {

// ---- counter-based random numbers (SplitMix64 finaliser) -----------------
inline uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t rng64(uint64_t seed, uint64_t stream, uint64_t idx)
{
    return mix64(mix64(mix64(seed) ^ (stream * 0xD1B54A32D192ED03ull)) ^ idx);
}
inline double unit(uint64_t seed, uint64_t stream, uint64_t idx)
{
    return (double)(rng64(seed, stream, idx) >> 11) * (1.0 / 9007199254740992.0);
}
enum : uint64_t { S_JITTER = 1, S_PERM = 2, S_RHS = 3 };

// ---- deterministic elementary functions ------------------------------------
const double TWO_PI_HI = 6.283185307179586;       // nearest double to 2*pi
const double TWO_PI_LO = 2.4492935982947064e-16;  // 2*pi - TWO_PI_HI
const double LN2 = 0.6931471805599453;

// Reduce x to r in [-pi, pi] with x = r + k*2pi.
double reduce_2pi(double x)
{
    double k = std::floor(x / TWO_PI_HI + 0.5);
    return (x - k * TWO_PI_HI) - k * TWO_PI_LO;
}
// Taylor series sum_{m>=0} (-1)^m r^(2m+1)/(2m+1)!, Horner from the 27th power.
double det_sin(double x)
{
    double r = reduce_2pi(x), r2 = r * r, s = 1.0;
    for (int m = 13; m >= 1; m--) s = 1.0 - s * r2 / (double)((2 * m) * (2 * m + 1));
    return r * s;
}
double det_cos(double x)
{
    double r = reduce_2pi(x), r2 = r * r, s = 1.0;
    for (int m = 13; m >= 1; m--) s = 1.0 - s * r2 / (double)((2 * m - 1) * (2 * m));
    return s;
}
// exp(x) = 2^k exp(r), |r| <= ln2/2, Taylor to r^20.
double det_exp(double x)
{
    double k = std::floor(x / LN2 + 0.5);
    double r = x - k * LN2, s = 1.0;
    for (int m = 20; m >= 1; m--) s = 1.0 + s * r / (double)m;
    return std::ldexp(s, (int)k);
}
// log(x) = e ln2 + 2 atanh((m-1)/(m+1)), m in [1,2).
double det_log(double x)
{
    int e = 0;
    double m = std::frexp(x, &e);  // x = m 2^e, m in [0.5, 1)
    m = m * 2.0;
    e -= 1;
    double t = (m - 1.0) / (m + 1.0), t2 = t * t, s = 0.0;
    for (int j = 30; j >= 0; j--) s = 1.0 / (double)(2 * j + 1) + t2 * s;
    return (double)e * LN2 + 2.0 * t * s;
}

struct V3 { double x, y, z; };
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }

// Area vector of the quadrilateral n1..n4 by the polygon (shoelace) formula.
V3 quad_area(const V3 p[4])
{
    V3 s{0.0, 0.0, 0.0};
    for (int a = 0; a < 4; a++) {
        const V3 &u = p[a], &w = p[(a + 1) & 3];
        s.x = s.x + (w.y - u.y) * (w.z + u.z);
        s.y = s.y + (w.z - u.z) * (w.x + u.x);
        s.z = s.z + (w.x - u.x) * (w.y + u.y);
    }
    return {0.5 * s.x, 0.5 * s.y, 0.5 * s.z};
}
V3 quad_centre(const V3 p[4])
{
    return {(p[0].x + p[1].x + p[2].x + p[3].x) / 4.0,
            (p[0].y + p[1].y + p[2].y + p[3].y) / 4.0,
            (p[0].z + p[1].z + p[2].z + p[3].z) / 4.0};
}

}  // namespace

extern "C" double tfs_synth_uniform(uint64_t seed, uint64_t stream, uint64_t index)
{
    return unit(seed, stream, index);
}

extern "C" int64_t tfs_synth_loguniform(int64_t lo, int64_t hi, uint64_t seed,
                                        uint64_t index)
{
    if (lo <= 0 || hi < lo) return -1;
    double a = det_log((double)lo), b = det_log((double)hi);
    double u = unit(seed, 17, index);
    int64_t v = (int64_t)std::floor(det_exp(a + u * (b - a)) + 0.5);
    return v < lo ? lo : (v > hi ? hi : v);
}

extern "C" int tfs_synth_create(int kind, int32_t nx, int32_t ny, int32_t nz,
                                double jitter, uint64_t seed, int permute,
                                tfs_synth **out)
{
    if (!out || nx < 1 || ny < 1 || nz < 1 || jitter < 0.0 || jitter >= 0.5) return TFS_ERR_ARG;
    if (kind != TFS_SYNTH_POISSON && kind != TFS_SYNTH_CONVDIFF) return TFS_ERR_ARG;
    int64_t ncell64 = (int64_t)nx * ny * nz;
    if (ncell64 > (int64_t)200000000) return TFS_ERR_ARG;
    *out = nullptr;
    tfs_synth *S = new (std::nothrow) tfs_synth;
    if (!S) return TFS_ERR_ARG;
    const int32_t n = (int32_t)ncell64;
    const double h = 1.0 / (double)nx;
    const int64_t NX = nx + 1, NY = ny + 1, NZ = nz + 1;

    // Nodes, interior ones jittered.
    std::vector<V3> node((size_t)(NX * NY * NZ));
    for (int64_t k = 0; k < NZ; k++)
        for (int64_t j = 0; j < NY; j++)
            for (int64_t i = 0; i < NX; i++) {
                int64_t id = i + NX * (j + NY * k);
                V3 p{(double)i * h, (double)j * h, (double)k * h};
                if (i > 0 && i < nx && j > 0 && j < ny && k > 0 && k < nz && jitter > 0.0) {
                    p.x = p.x + (2.0 * unit(seed, S_JITTER, 3 * id + 0) - 1.0) * jitter * h;
                    p.y = p.y + (2.0 * unit(seed, S_JITTER, 3 * id + 1) - 1.0) * jitter * h;
                    p.z = p.z + (2.0 * unit(seed, S_JITTER, 3 * id + 2) - 1.0) * jitter * h;
                }
                node[(size_t)id] = p;
            }
    auto nid = [&](int64_t i, int64_t j, int64_t k) { return (size_t)(i + NX * (j + NY * k)); };

    // Cell renumbering: natural id -> 1-based cell number.
    std::vector<int32_t> num((size_t)n);
    for (int32_t c = 0; c < n; c++) num[(size_t)c] = c + 1;
    if (permute) {
        for (int64_t i = n - 1; i >= 1; i--) {  // Fisher-Yates
            uint64_t r = rng64(seed, S_PERM, (uint64_t)i);
            int64_t j = (int64_t)(((unsigned __int128)r * (unsigned __int128)(i + 1)) >> 64);
            int32_t t = num[(size_t)i]; num[(size_t)i] = num[(size_t)j]; num[(size_t)j] = t;
        }
    }

    // Cell centres (node average, summed node by node as the reference does).
    std::vector<V3> xc((size_t)n);
    for (int64_t k = 0; k < nz; k++)
        for (int64_t j = 0; j < ny; j++)
            for (int64_t i = 0; i < nx; i++) {
                V3 c{0.0, 0.0, 0.0};
                for (int q = 0; q < 8; q++) {
                    const V3 &p = node[nid(i + (q & 1), j + ((q >> 1) & 1), k + ((q >> 2) & 1))];
                    c.x = c.x + p.x / 8.0; c.y = c.y + p.y / 8.0; c.z = c.z + p.z / 8.0;
                }
                xc[(size_t)(i + nx * (j + ny * k))] = c;
            }

    // The quad of the face of cell (i,j,k) normal to direction d on side hi.
    auto face_nodes = [&](int64_t i, int64_t j, int64_t k, int d, int side, V3 p[4]) {
        if (d == 0) {
            int64_t a = i + side;
            p[0] = node[nid(a, j, k)]; p[1] = node[nid(a, j + 1, k)];
            p[2] = node[nid(a, j + 1, k + 1)]; p[3] = node[nid(a, j, k + 1)];
        } else if (d == 1) {
            int64_t a = j + side;
            p[0] = node[nid(i, a, k)]; p[1] = node[nid(i, a, k + 1)];
            p[2] = node[nid(i + 1, a, k + 1)]; p[3] = node[nid(i + 1, a, k)];
        } else {
            int64_t a = k + side;
            p[0] = node[nid(i, j, a)]; p[1] = node[nid(i + 1, j, a)];
            p[2] = node[nid(i + 1, j + 1, a)]; p[3] = node[nid(i, j + 1, a)];
        }
    };

    // Volumes by the divergence theorem (outward area vectors).
    std::vector<double> vol((size_t)n, 0.0);
    if (kind == TFS_SYNTH_CONVDIFF) {
        for (int64_t k = 0; k < nz; k++)
            for (int64_t j = 0; j < ny; j++)
                for (int64_t i = 0; i < nx; i++) {
                    size_t c = (size_t)(i + nx * (j + ny * k));
                    double v = 0.0;
                    for (int d = 0; d < 3; d++)
                        for (int side = 0; side < 2; side++) {
                            V3 p[4];
                            face_nodes(i, j, k, d, side, p);
                            V3 S = quad_area(p), xf = quad_centre(p);
                            if (dot(S, sub(xf, xc[c])) < 0.0) S = {-S.x, -S.y, -S.z};
                            v = v + dot(xf, S);
                        }
                    vol[c] = v / 3.0;
                }
    }

    // Interior faces in natural order: for each cell its +x, +y, +z face.
    struct Face { int32_t c1, c2; double a12, a21; };
    std::vector<Face> faces;
    faces.reserve((size_t)(3 * (int64_t)n));
    const double nu = 1e-3, pe_max = 10.0;
    const double U0 = pe_max * nu / h;
    for (int64_t k = 0; k < nz; k++)
        for (int64_t j = 0; j < ny; j++)
            for (int64_t i = 0; i < nx; i++) {
                size_t c = (size_t)(i + nx * (j + ny * k));
                for (int d = 0; d < 3; d++) {
                    int64_t i2 = i + (d == 0), j2 = j + (d == 1), k2 = k + (d == 2);
                    if (i2 >= nx || j2 >= ny || k2 >= nz) continue;
                    size_t c2 = (size_t)(i2 + nx * (j2 + ny * k2));
                    V3 p[4];
                    face_nodes(i, j, k, d, 1, p);
                    V3 S = quad_area(p);
                    V3 dvec = sub(xc[c2], xc[c]);
                    if (dot(S, dvec) < 0.0) S = {-S.x, -S.y, -S.z};  // point c1 -> c2
                    double af = norm(S) / norm(dvec);
                    Face f{num[c], num[c2], af, af};
                    if (kind == TFS_SYNTH_CONVDIFF) {
                        V3 xf = quad_centre(p);
                        double X = TWO_PI_HI * xf.x, Y = TWO_PI_HI * xf.y, Z = TWO_PI_HI * xf.z;
                        double u = U0 * det_sin(X) * det_cos(Y) * det_cos(Z);
                        double v = -U0 * det_cos(X) * det_sin(Y) * det_cos(Z);
                        double F = u * S.x + v * S.y;
                        double A0 = nu * af;
                        // NewUVW.f90:361-362 first-order upwind
                        f.a12 = A0 - (F < 0.0 ? F : 0.0);
                        f.a21 = A0 + (F > 0.0 ? F : 0.0);
                    }
                    faces.push_back(f);
                }
            }

    S->n = n;
    S->n_faces = (int32_t)faces.size();
    S->faces_c.resize(2 * faces.size());
    for (size_t s = 0; s < faces.size(); s++) {
        S->faces_c[2 * s] = faces[s].c1;
        S->faces_c[2 * s + 1] = faces[s].c2;
    }
    int32_t nnz = tfs_topology_count(n, S->n_faces, S->faces_c.data());
    if (nnz < 0) { delete S; return TFS_ERR_ARG; }
    S->nnz = nnz;
    S->row1.resize((size_t)n + 1);
    S->col1.resize((size_t)nnz);
    S->dia1.resize((size_t)n);
    std::vector<int32_t> pos(2 * faces.size());
    int st = tfs_topology_build(n, S->n_faces, S->faces_c.data(), S->row1.data(),
                                S->col1.data(), S->dia1.data(), nullptr, pos.data());
    if (st != TFS_OK) { delete S; return st; }

    // Assembly through pos/dia, face by face (Compute_Pressure_Simple.f90:100-107,
    // NewUVW.f90:365-368).
    S->val.assign((size_t)nnz, 0.0);
    double *val = S->val.data();
    const int32_t *dia = S->dia1.data();
    for (size_t s = 0; s < faces.size(); s++) {
        const Face &f = faces[s];
        val[pos[2 * s] - 1] = val[pos[2 * s] - 1] - f.a12;
        val[dia[f.c1 - 1] - 1] = val[dia[f.c1 - 1] - 1] + f.a12;
        val[pos[2 * s + 1] - 1] = val[pos[2 * s + 1] - 1] - f.a21;
        val[dia[f.c2 - 1] - 1] = val[dia[f.c2 - 1] - 1] + f.a21;
    }
    if (kind == TFS_SYNTH_POISSON) {
        // Dirichlet on x = 0: diagonal gets |S_b| / |x_fb - x_c|.
        for (int64_t k = 0; k < nz; k++)
            for (int64_t j = 0; j < ny; j++) {
                size_t c = (size_t)(nx * (j + ny * k));
                V3 p[4];
                face_nodes(0, j, k, 0, 0, p);
                V3 S = quad_area(p), xf = quad_centre(p);
                double ab = norm(S) / norm(sub(xf, xc[c]));
                int32_t d = dia[num[c] - 1] - 1;
                val[d] = val[d] + ab;
            }
    } else {
        // Time term V/dt on the diagonal (NewUVW.f90:500-505, rho = 1).
        const double dt = 0.5 * h / U0;
        for (int32_t c = 0; c < n; c++) {
            int32_t d = dia[num[(size_t)c] - 1] - 1;
            val[d] = val[d] + vol[(size_t)c] / dt;
        }
    }
    // Right-hand side per (renumbered) cell.
    S->b.resize((size_t)n);
    for (int32_t r = 0; r < n; r++) S->b[(size_t)r] = 2.0 * unit(seed, S_RHS, (uint64_t)r) - 1.0;
    *out = S;
    return TFS_OK;
}

extern "C" int tfs_synth_dims(const tfs_synth *s, int32_t *n, int32_t *nnz, int32_t *n_faces)
{
    if (!s) return TFS_ERR_ARG;
    if (n) *n = s->n;
    if (nnz) *nnz = s->nnz;
    if (n_faces) *n_faces = s->n_faces;
    return TFS_OK;
}

extern "C" int tfs_synth_export(const tfs_synth *s, int32_t *faces_c, int32_t *row1,
                                int32_t *col1, int32_t *dia1, double *val, double *b)
{
    if (!s) return TFS_ERR_ARG;
    if (faces_c) std::memcpy(faces_c, s->faces_c.data(), s->faces_c.size() * sizeof(int32_t));
    if (row1) std::memcpy(row1, s->row1.data(), s->row1.size() * sizeof(int32_t));
    if (col1) std::memcpy(col1, s->col1.data(), s->col1.size() * sizeof(int32_t));
    if (dia1) std::memcpy(dia1, s->dia1.data(), s->dia1.size() * sizeof(int32_t));
    if (val) std::memcpy(val, s->val.data(), s->val.size() * sizeof(double));
    if (b) std::memcpy(b, s->b.data(), s->b.size() * sizeof(double));
    return TFS_OK;
}

extern "C" void tfs_synth_free(tfs_synth *s) { delete s; }
