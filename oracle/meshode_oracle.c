/*
 * meshode_oracle.c -- CPU restatement of MeshODE's per-iteration deformation
 * hot path.  TEST INFRASTRUCTURE ONLY: this file is the oracle the CUDA
 * library in meshode_gb300/csrc is tested against.  It is loaded by the tests,
 * by smoke() and by the CPU-baseline leg of bench.py, never by the product
 * path.
 *
 * Every function below is a line-by-line restatement of the cited reference
 * loop, in the same arithmetic type and the same operation order, so that it
 * reproduces the reference's results bit for bit on an IEEE-754 machine
 * without FMA contraction (the reference builds with g++ -O2 for x86-64,
 * which has no FMA by default).  The file must therefore be compiled with
 * -ffp-contract=off (aarch64 gcc contracts by default).
 *
 * Parity status: pinned.  oracle/build_ref.py compiles the reference's own
 * source files (mesh.cc, uniformgrid.cc, the interface layers) unchanged
 * against small stand-in headers for Eigen, ceres::Jet, torch and libigl into
 * oracle/_ref, and tests/test_ref_pin.py checks this file against it bit for
 * bit on the reference's demo meshes and on probes at every branch;
 * tests/golden/gen_ref_fixtures.py keeps fixtures from it for machines
 * without the reference.  Still unpinned: libigl's own point-mesh distance
 * (its stand-in is the exact FP64 distance below) and the published
 * arithmetic of Ceres and Eigen, which the stand-ins restate.
 *
 * Third-party arithmetic restated here:
 *   - ceres::Jet<float,3> (forward-mode dual numbers, version not pinned by the
 *     reference's .gitmodules): a*b = (a.a*b.a, a.a*b.v + a.v*b.a),
 *     a+b = (a.a+b.a, a.v+b.v), a-b, -a, constants carry a zero derivative.
 *   - igl::point_mesh_squared_distance (libigl, not pinned): exact squared
 *     Euclidean distance from a point to the closest point of a triangle set.
 *     Restated as an FP64 closest-point computation (segment distances plus
 *     the interior plane distance), brute force and through an AABB tree.
 */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------ */
/* Float -> int truncation with x86-64 semantics.                           */
/* uniformgrid.cc:87-89 does `int px = *(float*)&p[0] * grid_dimension_`. */
/* On x86-64 (cvttss2si) NaN and out-of-range values give INT_MIN.          */
/* ------------------------------------------------------------------------ */
static int trunc_i32(float f) {
    if (f >= -2147483648.0f && f < 2147483648.0f) return (int)f;
    return INT_MIN;
}

EXPORT int orc_trunc_i32(float f) { return trunc_i32(f); }

/* ------------------------------------------------------------------------ */
/* UniformGrid::DistanceFloat<float>  (src/lib/uniformgrid.cc:85-150)       */
/* Grid storage is voxel_distance_[z][y][x] (uniformgrid.h:33), flattened    */
/* here to grid[(z*N + y)*N + x], values already cast to float.              */
/* ------------------------------------------------------------------------ */
static inline float G(const float* g, int N, int z, int y, int x) {
    return g[((int64_t)z * N + y) * N + x];
}

EXPORT float orc_distance_float(const float* grid, int N, const float* p) {
    const float Nf = (float)N;
    int px = trunc_i32(p[0] * Nf);
    int py = trunc_i32(p[1] * Nf);
    int pz = trunc_i32(p[2] * Nf);
    if (px < 0 || py < 0 || pz < 0 || px >= N - 1 || py >= N - 1 || pz >= N - 1) {
        const float C = (float)((double)(N - 1) - 1e-3);
        float l = 0.0f;
        if (px < 0) l = l + -p[0] * Nf;
        else if (px >= N) l = l + (p[0] * Nf - C);
        if (py < 0) l = l + -p[1] * Nf;
        else if (py >= N) l = l + (p[1] * Nf - C);
        if (pz < 0) l = l + -p[2] * Nf;
        else if (pz >= N) l = l + (p[2] * Nf - C);
        return l;
    }
    float wx = p[0] * Nf - (float)px;
    float wy = p[1] * Nf - (float)py;
    float wz = p[2] * Nf - (float)pz;
    float w0 = (1.0f - wx) * (1.0f - wy) * (1.0f - wz) * G(grid, N, pz, py, px);
    float w1 = wx * (1.0f - wy) * (1.0f - wz) * G(grid, N, pz, py, px + 1);
    float w2 = (1.0f - wx) * wy * (1.0f - wz) * G(grid, N, pz, py + 1, px);
    float w3 = wx * wy * (1.0f - wz) * G(grid, N, pz, py + 1, px + 1);
    float w4 = (1.0f - wx) * (1.0f - wy) * wz * G(grid, N, pz + 1, py, px);
    float w5 = wx * (1.0f - wy) * wz * G(grid, N, pz + 1, py, px + 1);
    float w6 = (1.0f - wx) * wy * wz * G(grid, N, pz + 1, py + 1, px);
    float w7 = wx * wy * wz * G(grid, N, pz + 1, py + 1, px + 1);
    float res = w0 + w1 + w2 + w3 + w4 + w5 + w6 + w7;
    if (res > 0.2f) return 0.0f;
    return res;
}

/* ------------------------------------------------------------------------ */
/* ceres::Jet<float,3> arithmetic, restated.                                 */
/* ------------------------------------------------------------------------ */
typedef struct { float a; float v[3]; } jet3;

static inline jet3 jc(float x) { jet3 r = {x, {0.0f, 0.0f, 0.0f}}; return r; }
static inline jet3 jadd(jet3 f, jet3 g) {
    jet3 r; r.a = f.a + g.a;
    for (int i = 0; i < 3; ++i) r.v[i] = f.v[i] + g.v[i];
    return r;
}
static inline jet3 jsub(jet3 f, jet3 g) {
    jet3 r; r.a = f.a - g.a;
    for (int i = 0; i < 3; ++i) r.v[i] = f.v[i] - g.v[i];
    return r;
}
static inline jet3 jneg(jet3 f) {
    jet3 r; r.a = -f.a;
    for (int i = 0; i < 3; ++i) r.v[i] = -f.v[i];
    return r;
}
static inline jet3 jmul(jet3 f, jet3 g) {
    jet3 r; r.a = f.a * g.a;
    for (int i = 0; i < 3; ++i) r.v[i] = f.a * g.v[i] + f.v[i] * g.a;
    return r;
}

/* UniformGrid::DistanceFloat<ceres::Jet<float,3>> (uniformgrid.cc:85-150),
 * written against the jet operations exactly as the template expands.
 * out[0] = value, out[1..3] = d value / d p. */
EXPORT void orc_distance_jet(const float* grid, int N, const float* pv, float* out) {
    jet3 p[3];
    for (int k = 0; k < 3; ++k) { p[k] = jc(pv[k]); p[k].v[k] = 1.0f; }
    const jet3 NJ = jc((float)N);
    const float Nf = (float)N;
    int px = trunc_i32(p[0].a * Nf);
    int py = trunc_i32(p[1].a * Nf);
    int pz = trunc_i32(p[2].a * Nf);
    jet3 res;
    if (px < 0 || py < 0 || pz < 0 || px >= N - 1 || py >= N - 1 || pz >= N - 1) {
        const jet3 C = jc((float)((double)(N - 1) - 1e-3));
        jet3 l = jc(0.0f);
        if (px < 0) l = jadd(l, jmul(jneg(p[0]), NJ));
        else if (px >= N) l = jadd(l, jsub(jmul(p[0], NJ), C));
        if (py < 0) l = jadd(l, jmul(jneg(p[1]), NJ));
        else if (py >= N) l = jadd(l, jsub(jmul(p[1], NJ), C));
        if (pz < 0) l = jadd(l, jmul(jneg(p[2]), NJ));
        else if (pz >= N) l = jadd(l, jsub(jmul(p[2], NJ), C));
        res = l;
    } else {
        jet3 wx = jsub(jmul(p[0], NJ), jc((float)px));
        jet3 wy = jsub(jmul(p[1], NJ), jc((float)py));
        jet3 wz = jsub(jmul(p[2], NJ), jc((float)pz));
        jet3 one = jc(1.0f);
        jet3 ox = jsub(one, wx), oy = jsub(one, wy), oz = jsub(one, wz);
        jet3 w0 = jmul(jmul(jmul(ox, oy), oz), jc(G(grid, N, pz, py, px)));
        jet3 w1 = jmul(jmul(jmul(wx, oy), oz), jc(G(grid, N, pz, py, px + 1)));
        jet3 w2 = jmul(jmul(jmul(ox, wy), oz), jc(G(grid, N, pz, py + 1, px)));
        jet3 w3 = jmul(jmul(jmul(wx, wy), oz), jc(G(grid, N, pz, py + 1, px + 1)));
        jet3 w4 = jmul(jmul(jmul(ox, oy), wz), jc(G(grid, N, pz + 1, py, px)));
        jet3 w5 = jmul(jmul(jmul(wx, oy), wz), jc(G(grid, N, pz + 1, py, px + 1)));
        jet3 w6 = jmul(jmul(jmul(ox, wy), wz), jc(G(grid, N, pz + 1, py + 1, px)));
        jet3 w7 = jmul(jmul(jmul(wx, wy), wz), jc(G(grid, N, pz + 1, py + 1, px + 1)));
        res = jadd(jadd(jadd(jadd(jadd(jadd(jadd(w0, w1), w2), w3), w4), w5), w6), w7);
        if (res.a > 0.2f) res = jc(0.0f);
    }
    out[0] = res.a;
    out[1] = res.v[0]; out[2] = res.v[1]; out[3] = res.v[2];
}

/* ------------------------------------------------------------------------ */
/* DistanceFieldLoss_forward / _backward (src/interface/distance_layer.cc)   */
/* ------------------------------------------------------------------------ */

/* distance_layer.cc:27-34: L[i] = d(v_i)^2 */
EXPORT void orc_dfloss_forward(const float* V, int64_t n, const float* grid, int N,
                               float* L) {
#pragma omp parallel for schedule(static) if (n > 4096)
    for (int64_t i = 0; i < n; ++i) {
        float d = orc_distance_float(grid, N, V + 3 * i);
        L[i] = d * d;
    }
}

/* distance_layer.cc:58-78: vd = d(p) as a Jet, vd *= vd, l = vd.v * 0.5
 * (the 0.5 is a double literal: float -> double -> float). */
EXPORT void orc_dfloss_backward(const float* V, int64_t n, const float* grid, int N,
                                float* Gout) {
#pragma omp parallel for schedule(static) if (n > 4096)
    for (int64_t i = 0; i < n; ++i) {
        float o[4];
        orc_distance_jet(grid, N, V + 3 * i, o);
        jet3 vd = {o[0], {o[1], o[2], o[3]}};
        vd = jmul(vd, vd);
        for (int k = 0; k < 3; ++k) Gout[3 * i + k] = (float)((double)vd.v[k] * 0.5);
    }
}

/* ------------------------------------------------------------------------ */
/* Edge losses.  A "half-edge" list is given as pairs (v0, v1).              */
/* For faces (rigid_layer.cc:29-45) half-edge 3f+j is (F[f][j], F[f][(j+1)%3]).*/
/* For graphs (graph_layer.cc:18-32) edge k is (E[k][0], E[k][1]).           */
/* ------------------------------------------------------------------------ */
static inline void he_ends(const int* idx, int kind, int64_t h, int* v0, int* v1) {
    if (kind == 0) {
        int64_t f = h / 3; int j = (int)(h % 3);
        *v0 = idx[f * 3 + j];
        *v1 = idx[f * 3 + (j + 1) % 3];
    } else {
        *v0 = idx[2 * h];
        *v1 = idx[2 * h + 1];
    }
}

/* StoreRigidityInformation (rigid_layer.cc:29-45) and StoreGraphInformation
 * (graph_layer.cc:18-32): off[h] = v1 - v0 from the (normalised) source. */
EXPORT void orc_edge_offsets(const float* V, const int* idx, int64_t nh, int kind,
                             float* off) {
    for (int64_t h = 0; h < nh; ++h) {
        int v0, v1; he_ends(idx, kind, h, &v0, &v1);
        for (int c = 0; c < 3; ++c) off[3 * h + c] = V[3 * (int64_t)v1 + c] - V[3 * (int64_t)v0 + c];
    }
}

/* RigidEdgeLoss_forward (rigid_layer.cc:72-86) / GraphEdgeLoss_forward
 * (graph_layer.cc:74-88): R[h][c] = (v1 - v0 - off)_c ^ 2 */
EXPORT void orc_edge_forward(const float* V, const int* idx, int64_t nh, int kind,
                             const float* off, float* L) {
    for (int64_t h = 0; h < nh; ++h) {
        int v0, v1; he_ends(idx, kind, h, &v0, &v1);
        for (int c = 0; c < 3; ++c) {
            float r = V[3 * (int64_t)v1 + c] - V[3 * (int64_t)v0 + c] - off[3 * h + c];
            L[3 * h + c] = r * r;
        }
    }
}

/* RigidEdgeLoss_backward (rigid_layer.cc:113-130) / GraphEdgeLoss_backward
 * (graph_layer.cc:116-132): serial scatter in half-edge order,
 * g[v0] -= r, g[v1] += r. */
EXPORT void orc_edge_backward(const float* V, int64_t nv, const int* idx, int64_t nh,
                              int kind, const float* off, float* Gout) {
    memset(Gout, 0, sizeof(float) * 3 * (size_t)nv);
    for (int64_t h = 0; h < nh; ++h) {
        int v0, v1; he_ends(idx, kind, h, &v0, &v1);
        for (int c = 0; c < 3; ++c) {
            Gout[3 * (int64_t)v0 + c] -= (V[3 * (int64_t)v1 + c] - V[3 * (int64_t)v0 + c] - off[3 * h + c]);
            Gout[3 * (int64_t)v1 + c] += (V[3 * (int64_t)v1 + c] - V[3 * (int64_t)v0 + c] - off[3 * h + c]);
        }
    }
}

/* StoreCadInformation (cad_layer.cc:11-77): the CAD loss's edge set is E's
 * edges, then F's half-edges (list [ne + 3nf][2]); each edge's weight is
 * lambda = 2e-2 / (|off| + 1e-8) with |off| Eigen's float norm (sqrt of
 * x*x + (y*y + z*z)) and the sum and quotient in double (:48-49, :71-72). */
EXPORT void orc_edge_cad_list(const int* E, int64_t ne, const int* F, int64_t nf, int* list) {
    for (int64_t h = 0; h < ne; ++h) { list[2 * h] = E[2 * h]; list[2 * h + 1] = E[2 * h + 1]; }
    for (int64_t h = 0; h < 3 * nf; ++h) {
        int v0, v1; he_ends(F, 0, h, &v0, &v1);
        list[2 * (ne + h)] = v0; list[2 * (ne + h) + 1] = v1;
    }
}

EXPORT void orc_edge_cad_weights(const float* off, int64_t nh, float* lam) {
    for (int64_t h = 0; h < nh; ++h) {
        float x = off[3 * h], y = off[3 * h + 1], z = off[3 * h + 2];
        float n = sqrtf(x * x + (y * y + z * z));
        lam[h] = (float)(2e-2 / ((double)n + 1e-8));
    }
}

/* CadEdgeLoss_forward (cad_layer.cc:108-143): ((v1 - v0 - off) * w)^2. */
EXPORT void orc_edge_forward_w(const float* V, const int* idx, int64_t nh, int kind,
                               const float* off, const float* w, float* L) {
    for (int64_t h = 0; h < nh; ++h) {
        int v0, v1; he_ends(idx, kind, h, &v0, &v1);
        for (int c = 0; c < 3; ++c) {
            float r = (V[3 * (int64_t)v1 + c] - V[3 * (int64_t)v0 + c] - off[3 * h + c]) * w[h];
            L[3 * h + c] = r * r;
        }
    }
}

/* CadEdgeLoss_backward (cad_layer.cc:178-219): serial scatter of
 * (v1 - v0 - off) * (w * w). */
EXPORT void orc_edge_backward_w(const float* V, int64_t nv, const int* idx, int64_t nh, int kind,
                                const float* off, const float* w, float* Gout) {
    memset(Gout, 0, sizeof(float) * 3 * (size_t)nv);
    for (int64_t h = 0; h < nh; ++h) {
        int v0, v1; he_ends(idx, kind, h, &v0, &v1);
        float l2 = w[h] * w[h];
        for (int c = 0; c < 3; ++c) {
            Gout[3 * (int64_t)v0 + c] -= (V[3 * (int64_t)v1 + c] - V[3 * (int64_t)v0 + c] - off[3 * h + c]) * l2;
            Gout[3 * (int64_t)v1 + c] += (V[3 * (int64_t)v1 + c] - V[3 * (int64_t)v0 + c] - off[3 * h + c]) * l2;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Normalisation.                                                            */
/* Mesh::Normalize (src/lib/mesh.cc:66-96) on float input promoted to double, */
/* NormalizeByTemplate / DenormalizeByTemplate (src/interface/normalize.cc).  */
/* ------------------------------------------------------------------------ */
EXPORT void orc_normalize_params(const float* V, int64_t n, double* scale, double* trans) {
    double mn[3], mx[3];
    for (int j = 0; j < 3; ++j) {
        mn[j] = 1e30; mx[j] = -1e30;
        for (int64_t i = 0; i < n; ++i) {
            double x = (double)V[3 * i + j];
            if (x < mn[j]) mn[j] = x;
            if (x > mx[j]) mx[j] = x;
        }
    }
    double e0 = mx[0] - mn[0], e1 = mx[1] - mn[1], e2 = mx[2] - mn[2];
    double m12 = (e1 < e2) ? e2 : e1;  /* std::max(e1, e2) */
    double m = (e0 < m12) ? m12 : e0;  /* std::max(e0, m12), mesh.cc:79-80 */
    *scale = m * 1.1;
    for (int j = 0; j < 3; ++j) trans[j] = mn[j] - 0.05 * (*scale);
}

/* Normalised target vertices in double, as Mesh::Normalize leaves them
 * (mesh.cc:83-85): v = (v - pos) / scale. */
EXPORT void orc_normalize_double(const float* V, int64_t n, double scale, const double* trans,
                                 double* out) {
    for (int64_t i = 0; i < n; ++i)
        for (int j = 0; j < 3; ++j) out[3 * i + j] = ((double)V[3 * i + j] - trans[j]) / scale;
}

/* normalize.cc:13-23 */
EXPORT void orc_normalize_by_template(float* V, int64_t n, double scale, const double* trans) {
    for (int64_t i = 0; i < n; ++i)
        for (int j = 0; j < 3; ++j) V[3 * i + j] = (float)(((double)V[3 * i + j] - trans[j]) / scale);
}

/* normalize.cc:34-44 */
EXPORT void orc_denormalize_by_template(float* V, int64_t n, double scale, const double* trans) {
    for (int64_t i = 0; i < n; ++i)
        for (int j = 0; j < 3; ++j) V[3 * i + j] = (float)((double)V[3 * i + j] * scale + trans[j]);
}

/* ------------------------------------------------------------------------ */
/* FP64 point-triangle squared distance (the exact quantity libigl's          */
/* point_mesh_squared_distance returns).  Closest point = the interior        */
/* projection when it lies inside the triangle, else the nearest of the       */
/* three edge segments; degenerate triangles reduce to their segments.        */
/* ------------------------------------------------------------------------ */
static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline void sub3(const double* a, const double* b, double* r) { r[0] = a[0] - b[0]; r[1] = a[1] - b[1]; r[2] = a[2] - b[2]; }
static inline void cross3(const double* a, const double* b, double* r) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

static double seg_dist2(const double* p, const double* a, const double* b) {
    double ab[3], ap[3];
    sub3(b, a, ab); sub3(p, a, ap);
    double l2 = dot3(ab, ab);
    double t = 0.0;
    if (l2 > 0.0) {
        t = dot3(ap, ab) / l2;
        if (t < 0.0) t = 0.0;
        if (t > 1.0) t = 1.0;
    }
    double q[3] = {ap[0] - t * ab[0], ap[1] - t * ab[1], ap[2] - t * ab[2]};
    return dot3(q, q);
}

EXPORT double orc_point_tri_dist2(const double* p, const double* a, const double* b, const double* c) {
    double d = seg_dist2(p, a, b);
    double d1 = seg_dist2(p, b, c); if (d1 < d) d = d1;
    double d2 = seg_dist2(p, c, a); if (d2 < d) d = d2;
    double ab[3], ac[3], n[3];
    sub3(b, a, ab); sub3(c, a, ac); cross3(ab, ac, n);
    double nn = dot3(n, n);
    if (nn > 0.0) {
        double ap[3], bp[3], cp[3], bc[3], ca[3], t[3];
        sub3(p, a, ap); sub3(p, b, bp); sub3(p, c, cp);
        sub3(c, b, bc); sub3(a, c, ca);
        cross3(ab, ap, t); double s0 = dot3(t, n);
        cross3(bc, bp, t); double s1 = dot3(t, n);
        cross3(ca, cp, t); double s2 = dot3(t, n);
        if (s0 >= 0.0 && s1 >= 0.0 && s2 >= 0.0) {
            double h = dot3(ap, n);
            double dp = h * h / nn;
            if (dp < d) d = dp;
        }
    }
    return d;
}

/* Voxel sample position (mesh.cc:112-120): (k/N, j/N, i/N) for voxel
 * index (i*N + j)*N + k, i = z, j = y, k = x. */
static inline void voxel_pos(int64_t idx, int N, double* p) {
    int64_t k = idx % N, j = (idx / N) % N, i = idx / ((int64_t)N * N);
    p[0] = (double)k / N; p[1] = (double)j / N; p[2] = (double)i / N;
}

/* Brute-force FP64 DF over a list of voxel indices (all voxels when
 * vox == NULL).  Vn are the normalised target vertices in double.
 * out[q] = sqrt(min sqrD) in double (mesh.cc:140-150). */
EXPORT void orc_df_bruteforce(const double* Vn, const int* F, int64_t nf, int N,
                              const int64_t* vox, int64_t nvox, double* out) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t q = 0; q < nvox; ++q) {
        int64_t idx = vox ? vox[q] : q;
        double p[3]; voxel_pos(idx, N, p);
        double best = DBL_MAX;
        for (int64_t f = 0; f < nf; ++f) {
            double d = orc_point_tri_dist2(p, Vn + 3 * (int64_t)F[3 * f], Vn + 3 * (int64_t)F[3 * f + 1],
                                           Vn + 3 * (int64_t)F[3 * f + 2]);
            if (d < best) best = d;
        }
        out[q] = sqrt(best);
    }
}

/* ------------------------------------------------------------------------ */
/* FP64 AABB tree (top-down, longest-axis median split), the CPU analogue of */
/* libigl's AABB used by point_mesh_squared_distance.  Used for the timed CPU */
/* baseline of the DF build and for large-size DF checks.                    */
/* ------------------------------------------------------------------------ */
typedef struct { double lo[3], hi[3]; int left, right, start, count; } bnode;
typedef struct {
    const double* V; const int* F; int* order; double* cen; bnode* nodes; int nn;
} btree;

static void tri_box(const btree* t, int f, double* lo, double* hi) {
    for (int c = 0; c < 3; ++c) { lo[c] = DBL_MAX; hi[c] = -DBL_MAX; }
    for (int k = 0; k < 3; ++k) {
        const double* v = t->V + 3 * (int64_t)t->F[3 * (int64_t)f + k];
        for (int c = 0; c < 3; ++c) { if (v[c] < lo[c]) lo[c] = v[c]; if (v[c] > hi[c]) hi[c] = v[c]; }
    }
}

static int g_sort_axis;
static const double* g_sort_cen;
static int cmp_cen(const void* a, const void* b) {
    double x = g_sort_cen[3 * (int64_t)*(const int*)a + g_sort_axis];
    double y = g_sort_cen[3 * (int64_t)*(const int*)b + g_sort_axis];
    if (x < y) return -1;
    if (x > y) return 1;
    return (*(const int*)a) - (*(const int*)b);
}

static int btree_build(btree* t, int start, int count) {
    int id = t->nn++;
    bnode* nd = &t->nodes[id];
    for (int c = 0; c < 3; ++c) { nd->lo[c] = DBL_MAX; nd->hi[c] = -DBL_MAX; }
    for (int i = start; i < start + count; ++i) {
        double lo[3], hi[3]; tri_box(t, t->order[i], lo, hi);
        for (int c = 0; c < 3; ++c) {
            if (lo[c] < nd->lo[c]) nd->lo[c] = lo[c];
            if (hi[c] > nd->hi[c]) nd->hi[c] = hi[c];
        }
    }
    nd->start = start; nd->count = count; nd->left = nd->right = -1;
    if (count <= 4) return id;
    int axis = 0; double ext = -1;
    for (int c = 0; c < 3; ++c) if (nd->hi[c] - nd->lo[c] > ext) { ext = nd->hi[c] - nd->lo[c]; axis = c; }
    g_sort_axis = axis; g_sort_cen = t->cen;
    qsort(t->order + start, (size_t)count, sizeof(int), cmp_cen);
    int half = count / 2;
    int l = btree_build(t, start, half);
    int r = btree_build(t, start + half, count - half);
    t->nodes[id].left = l; t->nodes[id].right = r;
    return id;
}

static inline double box_dist2(const double* p, const double* lo, const double* hi) {
    double d = 0;
    for (int c = 0; c < 3; ++c) {
        double e = 0;
        if (p[c] < lo[c]) e = lo[c] - p[c];
        else if (p[c] > hi[c]) e = p[c] - hi[c];
        d += e * e;
    }
    return d;
}

static double btree_query(const btree* t, const double* p, double best) {
    int stack[128]; int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const bnode* nd = &t->nodes[stack[--sp]];
        /* prune with a relative margin far above the rounding of box_dist2
         * and orc_point_tri_dist2, so the result is the exact minimum of the
         * computed distances over every triangle (what brute force returns) */
        if (box_dist2(p, nd->lo, nd->hi) > best * (1.0 + 1e-9)) continue;
        if (nd->left < 0) {
            for (int i = nd->start; i < nd->start + nd->count; ++i) {
                int f = t->order[i];
                double d = orc_point_tri_dist2(p, t->V + 3 * (int64_t)t->F[3 * (int64_t)f],
                                               t->V + 3 * (int64_t)t->F[3 * (int64_t)f + 1],
                                               t->V + 3 * (int64_t)t->F[3 * (int64_t)f + 2]);
                if (d < best) best = d;
            }
        } else {
            const bnode* L = &t->nodes[nd->left];
            const bnode* R = &t->nodes[nd->right];
            double dl = box_dist2(p, L->lo, L->hi), dr = box_dist2(p, R->lo, R->hi);
            if (dl < dr) { stack[sp++] = nd->right; stack[sp++] = nd->left; }
            else { stack[sp++] = nd->left; stack[sp++] = nd->right; }
        }
    }
    return best;
}

/* Nearest triangle of every point of P through the AABB tree: the squared
 * distance and the face index (the lowest index among exact ties found first
 * in the tree's order).  The libigl stand-in of oracle/_ref calls this in
 * place of igl::point_mesh_squared_distance; C (np x 3) is filled with NaN.
 * nthreads <= 0 uses every OpenMP thread.  Returns 0 on success. */
static double btree_query_idx(const btree* t, const double* p, int* best_f) {
    double best = DBL_MAX;
    int bf = -1;
    int stack[128]; int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const bnode* nd = &t->nodes[stack[--sp]];
        if (box_dist2(p, nd->lo, nd->hi) > best * (1.0 + 1e-9)) continue;  /* as btree_query */
        if (nd->left < 0) {
            for (int i = nd->start; i < nd->start + nd->count; ++i) {
                int f = t->order[i];
                double d = orc_point_tri_dist2(p, t->V + 3 * (int64_t)t->F[3 * (int64_t)f],
                                               t->V + 3 * (int64_t)t->F[3 * (int64_t)f + 1],
                                               t->V + 3 * (int64_t)t->F[3 * (int64_t)f + 2]);
                if (d < best || (d == best && f < bf)) { best = d; bf = f; }
            }
        } else {
            const bnode* L = &t->nodes[nd->left];
            const bnode* R = &t->nodes[nd->right];
            double dl = box_dist2(p, L->lo, L->hi), dr = box_dist2(p, R->lo, R->hi);
            if (dl < dr) { stack[sp++] = nd->right; stack[sp++] = nd->left; }
            else { stack[sp++] = nd->left; stack[sp++] = nd->right; }
        }
    }
    *best_f = bf;
    return best;
}

EXPORT int orc_point_mesh_sqdist(const double* P, int64_t np, const double* V, int64_t nv, const int* F,
                                 int64_t nf, double* sqrD, int* I, double* C, int nthreads) {
    (void)nthreads;
    if (nf <= 0 || nv <= 0) return -1;
    for (int64_t k = 0; k < 3 * nf; ++k)
        if (F[k] < 0 || F[k] >= nv) return -3;
    btree t;
    t.V = V; t.F = F; t.nn = 0;
    t.order = (int*)malloc(sizeof(int) * (size_t)nf);
    t.cen = (double*)malloc(sizeof(double) * 3 * (size_t)nf);
    t.nodes = (bnode*)malloc(sizeof(bnode) * 2 * (size_t)nf);
    if (!t.order || !t.cen || !t.nodes) { free(t.order); free(t.cen); free(t.nodes); return -2; }
    for (int64_t f = 0; f < nf; ++f) {
        t.order[f] = (int)f;
        for (int c = 0; c < 3; ++c)
            t.cen[3 * f + c] = (V[3 * (int64_t)F[3 * f] + c] + V[3 * (int64_t)F[3 * f + 1] + c] +
                                V[3 * (int64_t)F[3 * f + 2] + c]) / 3.0;
    }
    btree_build(&t, 0, (int)nf);
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
#endif
    for (int64_t q = 0; q < np; ++q) {
        int f;
        sqrD[q] = btree_query_idx(&t, P + 3 * q, &f);
        I[q] = f;
        for (int c = 0; c < 3; ++c) C[3 * q + c] = NAN;
    }
    free(t.order); free(t.cen); free(t.nodes);
    return 0;
}

/* DF through the AABB tree over a list of voxels (all when vox == NULL).
 * nthreads <= 0 uses every OpenMP thread. Returns 0 on success. */
static double wall_seconds(void) {
    struct timespec ts;
    timespec_get(&ts, TIME_UTC);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* orc_df_bvh with its two phases timed: the serial tree build (t[0]) and the
 * voxel queries (t[1]), in seconds (for bounded CPU timings that scale only
 * the queries to a full grid). */
static int df_bvh_impl(const double* Vn, const int* F, int64_t nf, int N, const int64_t* vox, int64_t nvox,
                       double* out, int nthreads, double* t);

EXPORT int orc_df_bvh(const double* Vn, const int* F, int64_t nf, int N,
                      const int64_t* vox, int64_t nvox, double* out, int nthreads) {
    return df_bvh_impl(Vn, F, nf, N, vox, nvox, out, nthreads, NULL);
}

EXPORT int orc_df_bvh_timed(const double* Vn, const int* F, int64_t nf, int N, const int64_t* vox, int64_t nvox,
                            double* out, int nthreads, double* t2) {
    return df_bvh_impl(Vn, F, nf, N, vox, nvox, out, nthreads, t2);
}

static int df_bvh_impl(const double* Vn, const int* F, int64_t nf, int N, const int64_t* vox, int64_t nvox,
                       double* out, int nthreads, double* t) {
    if (nf <= 0) return -1;
    const double t0 = t ? wall_seconds() : 0.0;
    btree bt;
    bt.V = Vn; bt.F = F; bt.nn = 0;
    bt.order = (int*)malloc(sizeof(int) * (size_t)nf);
    bt.cen = (double*)malloc(sizeof(double) * 3 * (size_t)nf);
    bt.nodes = (bnode*)malloc(sizeof(bnode) * 2 * (size_t)nf);
    if (!bt.order || !bt.cen || !bt.nodes) { free(bt.order); free(bt.cen); free(bt.nodes); return -2; }
    for (int64_t f = 0; f < nf; ++f) {
        bt.order[f] = (int)f;
        for (int c = 0; c < 3; ++c)
            bt.cen[3 * f + c] = (Vn[3 * (int64_t)F[3 * f] + c] + Vn[3 * (int64_t)F[3 * f + 1] + c] +
                                Vn[3 * (int64_t)F[3 * f + 2] + c]) / 3.0;
    }
    btree_build(&bt, 0, (int)nf);
    const double t1 = t ? wall_seconds() : 0.0;
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
#endif
    for (int64_t q = 0; q < nvox; ++q) {
        int64_t idx = vox ? vox[q] : q;
        double p[3]; voxel_pos(idx, N, p);
        out[q] = sqrt(btree_query(&bt, p, DBL_MAX));
    }
    if (t) {
        t[0] = t1 - t0;
        t[1] = wall_seconds() - t1;
    }
    free(bt.order); free(bt.cen); free(bt.nodes);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* LBVH restatement for bit-exact checks of the GPU build.                   */
/* Morton codes of triangle centroids in the normalised unit cube, a stable  */
/* sort by code, and the Karras (HPG 2012) binary radix tree over the sorted */
/* codes.  The float operations match the CUDA kernels one for one.          */
/* ------------------------------------------------------------------------ */
static uint32_t spread10(uint32_t x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

static uint32_t quant10(float c) {
    float q = c * 1024.0f;
    q = fmaxf(q, 0.0f);
    q = fminf(q, 1023.0f);
    return (uint32_t)q;
}

/* Vn32: normalised target vertices as float (the GPU input). */
EXPORT void orc_morton_codes(const float* Vn32, const int* F, int64_t nf, uint32_t* codes) {
    for (int64_t f = 0; f < nf; ++f) {
        float c[3];
        for (int k = 0; k < 3; ++k) {
            float s = Vn32[3 * (int64_t)F[3 * f] + k] + Vn32[3 * (int64_t)F[3 * f + 1] + k];
            s = s + Vn32[3 * (int64_t)F[3 * f + 2] + k];
            c[k] = s / 3.0f;
        }
        codes[f] = (spread10(quant10(c[0])) << 2) | (spread10(quant10(c[1])) << 1) | spread10(quant10(c[2]));
    }
}

static const uint32_t* g_codes;
static int cmp_code(const void* a, const void* b) {
    uint32_t x = g_codes[*(const int*)a], y = g_codes[*(const int*)b];
    if (x < y) return -1;
    if (x > y) return 1;
    return (*(const int*)a) - (*(const int*)b);
}

/* Stable sort of triangle ids by Morton code. */
EXPORT void orc_sort_codes(const uint32_t* codes, int64_t n, uint32_t* sorted_codes, int* perm) {
    for (int64_t i = 0; i < n; ++i) perm[i] = (int)i;
    g_codes = codes;
    qsort(perm, (size_t)n, sizeof(int), cmp_code);
    for (int64_t i = 0; i < n; ++i) sorted_codes[i] = codes[perm[i]];
}

static int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

static int karras_delta(const uint32_t* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint32_t a = k[i], b = k[j];
    if (a != b) return clz32(a ^ b);
    return 32 + clz32((uint32_t)i ^ (uint32_t)j);
}

/* Internal node i of n-1: child indices encoded as >= 0 internal, or
 * ~leaf (negative) for leaves.  Matches the CUDA hierarchy kernel. */
EXPORT void orc_karras(const uint32_t* k, int n, int* left, int* right) {
    for (int i = 0; i < n - 1; ++i) {
        int d = (karras_delta(k, n, i, i + 1) - karras_delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
        int dmin = karras_delta(k, n, i, i - d);
        int lmax = 2;
        while (karras_delta(k, n, i, i + lmax * d) > dmin) lmax *= 2;
        int l = 0;
        for (int t = lmax / 2; t >= 1; t /= 2)
            if (karras_delta(k, n, i, i + (l + t) * d) > dmin) l += t;
        int j = i + l * d;
        int dnode = karras_delta(k, n, i, j);
        int s = 0;
        int t = l;
        do {
            t = (t + 1) / 2;
            if (karras_delta(k, n, i, i + (s + t) * d) > dnode) s += t;
        } while (t > 1);
        int gamma = i + s * d + (d < 0 ? -1 : 0);
        int lo = i < j ? i : j, hi = i < j ? j : i;
        left[i] = (lo == gamma) ? ~gamma : gamma;
        right[i] = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    }
}

/* ------------------------------------------------------------------------ */
/* torch.optim.Adam, one step of one parameter tensor (torch/optim/adam.py   */
/* _single_tensor_adam, the loop of rigid_deform.py:32,39), restated with   */
/* one IEEE rounding per tensor operation:                                   */
/*   exp_avg.lerp_(grad, 1-b1)        m = fma(1-b1, g - m, m)                */
/*   exp_avg_sq.mul_(b2).addcmul_(grad, grad, value=1-b2)                     */
/*                                    v = v*b2 + ((1-b2)*g)*g                */
/*   denom = exp_avg_sq.sqrt() / bc2_sqrt + eps                               */
/*   param.addcdiv_(exp_avg, denom, value=-step_size)                         */
/*                                    p = fma(-step_size, m/denom, p)        */
/* step_size = lr/(1-b1^t) and bc2_sqrt = sqrt(1-b2^t) come from the caller, */
/* computed in double like adam.py's host arithmetic.  lerp and addcdiv are  */
/* single fused multiply-adds as in ATen's lerp for weights below 0.5; the   */
/* torch CPU kernels may round their vectorised and tail lanes differently, */
/* so this restatement agrees with torch CPU to about an ulp per step.       */
/* ------------------------------------------------------------------------ */
EXPORT void orc_adam_step(float* p, const float* g, float* m, float* v, int64_t n, float omb1, float b2,
                          float omb2, float eps, float step_size, float bc2s) {
    for (int64_t i = 0; i < n; ++i) {
        const float gi = g[i];
        m[i] = fmaf(omb1, gi - m[i], m[i]);
        v[i] = v[i] * b2 + (omb2 * gi) * gi;
        const float denom = sqrtf(v[i]) / bc2s + eps;
        p[i] = fmaf(-step_size, m[i] / denom, p[i]);
    }
}
