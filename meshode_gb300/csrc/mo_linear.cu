// SolveLinear (src/interface/linear_layer.cc:5-79): the sparse linear
// propagation after a graph or flow deformation.
//
// LinearEstimation (src/lib/linear.cc:10-112), in double:
//   minimise  sum_g (w_g * sum_{j in cell g} x_j - w_g * G_g)^2      w_g = 1/|cell g|
//           + 1e-6 * sum_i |x_i - G_{ref(i)}|^2
//           + sum_edges reg_e |(x_a - x_b) - (V_a - V_b)|^2          reg_e = (0.02 r / (|V_a - V_b| + 1e-8))^2
// over the three coordinates, edges = the faces' half-edges then E; cell g
// holds the vertices i with ref(i) = g.
// LinearEstimationWithRot (linear.cc:114-230): per vertex the rotation
// R_i = U V^T of the SVD of sum_{j in N(i)} (G_j - G_i)(V_j - V_i)^T and the
// scale s_i = sum |G_j - G_i| / (sum |V_j - V_i| + 1e-8), then
//   minimise  sum_i |x_i - G_i|^2 + sum over face half-edges (a, b), both
//   directions, reg_ab |(x_b - x_a) - s_a R_a (V_b - V_a)|^2,   reg_ab = 0.02 r / |V_b - V_a|.
//
// The reference assembles A and factorises it with SimplicialLDLT.  Here the
// normal equations A x = B are solved matrix-free with Jacobi-preconditioned
// conjugate gradients in double: A x is gathered per vertex over the
// deterministic vertex -> edge CSR (and, for the cell term, a cell -> vertex
// CSR), every dot product is a fixed-order reduction, and one CG iteration
// is a captured CUDA graph of five launches.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "mo_common.cuh"

namespace mo {
namespace {

constexpr int LT = 256;        // threads per block
constexpr int LBLOCKS = 512;   // blocks of the dot-product partials

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

struct LinScratch {
    int32_t* edges;    // [nh, 2]
    void* csr;         // vertex -> half-edge CSR (mo_edge_csr_build layout)
    size_t csr_bytes;
    double* w;         // per half-edge weight
    double* G;         // [ng, 3] graph positions (LE) or [nv, 3] targets (rot)
    double* V0;        // [nv, 3] input positions
    double* diag;      // [nv]
    double* cellw;     // [ng] 1/|cell|
    int32_t* cell_ptr; // [ng + 1]
    int32_t* cell_mem; // [nv] vertices by cell, increasing
    double* cellsum;   // [ng, 3]
    double* rot;       // [nv, 9] s_i * R_i (row-major)
    double* x;         // [nv, 3]
    double* r;
    double* z;
    double* p;
    double* Ap;
    double* partial;   // [LBLOCKS, 3]
    double* scal;      // rz[3], pAp[3], alpha[3], beta[3], rz0[3], bb[3]
    int* status;
    uint32_t* keys_a;  // cell sort
    uint32_t* keys_b;
    int* vals_a;
    int* vals_b;
    int* hist;
    size_t bytes;
};

LinScratch plan(char* base, int64_t nv, int64_t nf, int64_t ne, int64_t ng, int with_rot) {
    LinScratch s;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + o : nullptr;
        o += a256(bytes ? bytes : 1);
        return p;
    };
    const int64_t nh = 3 * nf + (with_rot ? 0 : ne);
    s.edges = reinterpret_cast<int32_t*>(take(8 * (size_t)nh));
    s.csr_bytes = mo_edge_csr_bytes(nv, nh, MO_EDGES_LIST);
    s.csr = take(s.csr_bytes);
    s.w = reinterpret_cast<double*>(take(8 * (size_t)nh));
    s.G = reinterpret_cast<double*>(take(24 * (size_t)(with_rot ? nv : ng)));
    s.V0 = reinterpret_cast<double*>(take(24 * (size_t)nv));
    s.diag = reinterpret_cast<double*>(take(8 * (size_t)nv));
    s.cellw = reinterpret_cast<double*>(take(8 * (size_t)ng));
    s.cell_ptr = reinterpret_cast<int32_t*>(take(4 * (size_t)(ng + 1)));
    s.cell_mem = reinterpret_cast<int32_t*>(take(4 * (size_t)nv));
    s.cellsum = reinterpret_cast<double*>(take(24 * (size_t)ng));
    s.rot = reinterpret_cast<double*>(take(with_rot ? 72 * (size_t)nv : 0));
    s.x = reinterpret_cast<double*>(take(24 * (size_t)nv));
    s.r = reinterpret_cast<double*>(take(24 * (size_t)nv));
    s.z = reinterpret_cast<double*>(take(24 * (size_t)nv));
    s.p = reinterpret_cast<double*>(take(24 * (size_t)nv));
    s.Ap = reinterpret_cast<double*>(take(24 * (size_t)nv));
    s.partial = reinterpret_cast<double*>(take(48 * (size_t)LBLOCKS));  // two sets of 3 per block
    s.scal = reinterpret_cast<double*>(take(8 * 18));
    s.status = reinterpret_cast<int*>(take(16));
    s.keys_a = reinterpret_cast<uint32_t*>(take(4 * (size_t)nv));
    s.keys_b = reinterpret_cast<uint32_t*>(take(4 * (size_t)nv));
    s.vals_a = reinterpret_cast<int*>(take(4 * (size_t)nv));
    s.vals_b = reinterpret_cast<int*>(take(4 * (size_t)nv));
    s.hist = reinterpret_cast<int*>(take(4 * radix_hist_ints((int)nv)));
    s.bytes = o;
    return s;
}

// ---- set-up ----------------------------------------------------------------
__global__ void k_lin_edges(const int32_t* __restrict__ F, int64_t nf, const int32_t* __restrict__ E, int64_t ne,
                            int32_t* __restrict__ out) {
    const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h < 3 * nf) {
        const int64_t f = h / 3;
        const int j = (int)(h - 3 * f);
        out[2 * h] = F[3 * f + j];
        out[2 * h + 1] = F[3 * f + (j == 2 ? 0 : j + 1)];
    } else if (h < 3 * nf + ne) {
        const int64_t k = h - 3 * nf;
        out[2 * h] = E[2 * k];
        out[2 * h + 1] = E[2 * k + 1];
    }
}

__global__ void k_lin_to_double(const float* __restrict__ a, int64_t n, double* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)a[i];
}

__device__ __forceinline__ double norm3(double x, double y, double z) { return sqrt(x * x + y * y + z * z); }

// Half-edge weights from the input positions (edges validated by the CSR).
__global__ void k_lin_weights(const int32_t* __restrict__ edges, int64_t nh, const double* __restrict__ V,
                              double rigidity, int with_rot, double* __restrict__ w) {
    const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nh) return;
    const int64_t a = edges[2 * h], b = edges[2 * h + 1];
    const double n = norm3(V[3 * a] - V[3 * b], V[3 * a + 1] - V[3 * b + 1], V[3 * a + 2] - V[3 * b + 2]);
    if (with_rot) {
        // linear.cc:206: regulation * 2e-2 / |off| * rigidity, both directions
        w[h] = 2.0 * (1.0 * 2e-2 / n * rigidity);
    } else {
        // linear.cc:62-63: (regular * 2e-2 / (|V0 - V1| + 1e-8))^2
        const double reg = rigidity * 2e-2 / (n + 1e-8);
        w[h] = reg * reg;
    }
}

__global__ void k_lin_cell_keys(const int32_t* __restrict__ ref, int64_t nv, int64_t ng, uint32_t* __restrict__ keys,
                                int* __restrict__ vals, int* __restrict__ status) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int g = ref[i];
    if (g < 0 || (int64_t)g >= ng) atomicOr(status, 1);
    keys[i] = (g < 0 || (int64_t)g >= ng) ? 0u : (uint32_t)g;
    vals[i] = (int)i;
}

__global__ void k_lin_cell_ptr(const uint32_t* __restrict__ keys, int64_t nv, int32_t* __restrict__ cell_ptr) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nv) return;
    const uint32_t key = keys[k];
    const uint32_t prev = k == 0 ? 0u : keys[k - 1];
    // cell_ptr[g] = first position of cell g; empty cells take the next start
    for (uint32_t g = (k == 0 ? 0u : prev + 1); g <= key; ++g) cell_ptr[g] = (int32_t)k;
}

__global__ void k_lin_cell_tail(const uint32_t* __restrict__ keys, int64_t nv, int64_t ng,
                                int32_t* __restrict__ cell_ptr) {
    const uint32_t last = nv > 0 ? keys[nv - 1] : 0u;
    for (int64_t g = (nv > 0 ? (int64_t)last + 1 : 0); g <= ng; ++g) cell_ptr[g] = (int32_t)nv;
}

__global__ void k_lin_cellw(const int32_t* __restrict__ cell_ptr, int64_t ng, double* __restrict__ cellw) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const int c = cell_ptr[g + 1] - cell_ptr[g];
    cellw[g] = c > 0 ? 1.0 / (double)c : 0.0;
}

// Jacobi diagonal and right-hand side (LinearEstimation).
__global__ void k_lin_rhs(int64_t nv, const int* __restrict__ row_ptr, const int* __restrict__ other,
                          const int* __restrict__ key, const double* __restrict__ w, const double* __restrict__ V,
                          const int32_t* __restrict__ ref, const double* __restrict__ G,
                          const double* __restrict__ cellw, double* __restrict__ diag, double* __restrict__ B) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int64_t g = ref[i];
    const double wg = cellw[g];
    double d = 1e-6 + wg * wg;
    double b[3];
    for (int c = 0; c < 3; ++c) b[c] = wg * G[3 * g + c] + 1e-6 * G[3 * g + c];
    for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
        const int64_t o = other[k];
        if (o == i) continue;  // a self-loop's four entries cancel
        const double we = w[key[k] >> 1];
        d += we;
        for (int c = 0; c < 3; ++c) b[c] += we * (V[3 * i + c] - V[3 * o + c]);
    }
    diag[i] = d;
    for (int c = 0; c < 3; ++c) B[3 * i + c] = b[c];
}

// ---- with rotations --------------------------------------------------------
// Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations (bounded
// sweeps): a = Q diag(e) Q^T, Q columns the eigenvectors.
__device__ void jacobi3(double a[3][3], double Q[3][3], double e[3]) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Q[r][c] = r == c ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 32; ++sweep) {
        const double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
        const double scale = fabs(a[0][0]) + fabs(a[1][1]) + fabs(a[2][2]);
        if (off <= 1e-300 || off <= 1e-18 * scale) break;
        for (int p = 0; p < 2; ++p) {
            for (int q = p + 1; q < 3; ++q) {
                if (a[p][q] == 0.0) continue;
                const double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; ++k) {  // a <- J^T a J
                    const double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    const double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    const double qkp = Q[k][p], qkq = Q[k][q];
                    Q[k][p] = c * qkp - s * qkq;
                    Q[k][q] = s * qkp + c * qkq;
                }
            }
        }
    }
    for (int k = 0; k < 3; ++k) e[k] = a[k][k];
}

__device__ __forceinline__ void cross3(const double a[3], const double b[3], double c[3]) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

__device__ __forceinline__ bool unit3(double v[3]) {
    const double n = norm3(v[0], v[1], v[2]);
    if (!(n > 0.0)) return false;
    v[0] /= n; v[1] /= n; v[2] /= n;
    return true;
}

// R = U V^T for M = U S V^T: the orthogonal polar factor of M (unique when M
// is nonsingular).  From M^T M = Q diag(l) Q^T: v_k = q_k, u_k = M v_k /
// sqrt(l_k) for the two largest; when the smallest singular value vanishes
// (neighbours in one plane: every vertex of a surface patch) the third pair
// is completed as u1 x u2, v1 x v2 -- the reference's own choice there is an
// arbitrary sign, and the completed column multiplies only the normal part
// of an edge, which is zero for those neighbourhoods.
__device__ void polar3(const double M[3][3], double R[3][3]) {
    double a[3][3], Q[3][3], e[3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) a[r][c] = M[0][r] * M[0][c] + M[1][r] * M[1][c] + M[2][r] * M[2][c];
    jacobi3(a, Q, e);
    int ord[3] = {0, 1, 2};  // descending eigenvalues
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (e[ord[j]] > e[ord[i]]) { const int t = ord[i]; ord[i] = ord[j]; ord[j] = t; }
    double u[3][3], v[3][3];
    const double smax = sqrt(fmax(e[ord[0]], 0.0));
    int rank = 0;
    for (int k = 0; k < 3; ++k) {
        for (int c = 0; c < 3; ++c) v[k][c] = Q[c][ord[k]];
        const double sk = sqrt(fmax(e[ord[k]], 0.0));
        if (sk > 1e-12 * smax && sk > 0.0) {
            for (int r = 0; r < 3; ++r) u[k][r] = (M[r][0] * v[k][0] + M[r][1] * v[k][1] + M[r][2] * v[k][2]) / sk;
            ++rank;
        }
    }
    if (rank == 0) {
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) R[r][c] = r == c ? 1.0 : 0.0;
        return;
    }
    if (rank == 1) {  // complete u2 orthogonal to u1 along v2's direction
        double t[3] = {v[1][0], v[1][1], v[1][2]};
        const double d = t[0] * u[0][0] + t[1] * u[0][1] + t[2] * u[0][2];
        for (int c = 0; c < 3; ++c) t[c] -= d * u[0][c];
        if (!unit3(t)) {  // v2 parallel to u1: any perpendicular
            double ax[3] = {fabs(u[0][0]) < 0.9 ? 1.0 : 0.0, fabs(u[0][0]) < 0.9 ? 0.0 : 1.0, 0.0};
            cross3(u[0], ax, t);
            unit3(t);
        }
        for (int c = 0; c < 3; ++c) u[1][c] = t[c];
        rank = 2;
    }
    if (rank == 2) {
        cross3(u[0], u[1], u[2]);
        cross3(v[0], v[1], v[2]);
    }
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R[r][c] = u[0][r] * v[0][c] + u[1][r] * v[1][c] + u[2][r] * v[2][c];
}

// s_i * R_i from the unique neighbours of i (linear.cc:131-163).
__global__ void k_lin_rotations(int64_t nv, const int* __restrict__ row_ptr, const int* __restrict__ other,
                                const double* __restrict__ V, const double* __restrict__ T, double* __restrict__ rot) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    double M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double lo = 0.0, lc = 0.0;
    const int b = row_ptr[i], e = row_ptr[i + 1];
    for (int k = b; k < e; ++k) {
        const int o = other[k];
        bool seen = false;  // links[] is a set: each neighbour once
        for (int j = b; j < k && !seen; ++j) seen = other[j] == o;
        if (seen) continue;
        const double d1[3] = {V[3 * o] - V[3 * i], V[3 * o + 1] - V[3 * i + 1], V[3 * o + 2] - V[3 * i + 2]};
        const double d2[3] = {T[3 * o] - T[3 * i], T[3 * o + 1] - T[3 * i + 1], T[3 * o + 2] - T[3 * i + 2]};
        lo += norm3(d1[0], d1[1], d1[2]);
        lc += norm3(d2[0], d2[1], d2[2]);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) M[r][c] += d2[r] * d1[c];
    }
    const double s = lc / (lo + 1e-8);
    double R[3][3];
    polar3(M, R);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) rot[9 * i + 3 * r + c] = s * R[r][c];
}

// Diagonal and right-hand side with rotations (linear.cc:190-216).
__global__ void k_lin_rhs_rot(int64_t nv, const int* __restrict__ row_ptr, const int* __restrict__ other,
                              const int* __restrict__ key, const double* __restrict__ w,
                              const double* __restrict__ V, const double* __restrict__ T,
                              const double* __restrict__ rot, double* __restrict__ diag, double* __restrict__ B) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    double d = 1.0;
    double b[3] = {T[3 * i], T[3 * i + 1], T[3 * i + 2]};
    for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
        const int64_t o = other[k];
        if (o == i) continue;
        const double we = w[key[k] >> 1];  // both directions: 2 * reg
        const double reg = 0.5 * we;
        d += we;
        // + reg * s_o R_o (V_i - V_o)  - reg * s_i R_i (V_o - V_i)
        const double e[3] = {V[3 * i] - V[3 * o], V[3 * i + 1] - V[3 * o + 1], V[3 * i + 2] - V[3 * o + 2]};
        for (int r = 0; r < 3; ++r) {
            const double* Ro = rot + 9 * o + 3 * r;
            const double* Ri = rot + 9 * i + 3 * r;
            b[r] += reg * (Ro[0] * e[0] + Ro[1] * e[1] + Ro[2] * e[2]) + reg * (Ri[0] * e[0] + Ri[1] * e[1] + Ri[2] * e[2]);
        }
    }
    diag[i] = d;
    for (int c = 0; c < 3; ++c) B[3 * i + c] = b[c];
}

// ---- CG --------------------------------------------------------------------
// Ap = A p for both systems; partial[block] = sum p.Ap per column.
__global__ void __launch_bounds__(LT) k_lin_apply(int64_t nv, const int* __restrict__ row_ptr,
                                                  const int* __restrict__ other, const int* __restrict__ key,
                                                  const double* __restrict__ w, const int32_t* __restrict__ ref,
                                                  const double* __restrict__ cellw, const double* __restrict__ cellsum,
                                                  double c0, const double* __restrict__ p, double* __restrict__ Ap,
                                                  double* __restrict__ partial) {
    __shared__ double sh[3][LT];
    double acc[3] = {0.0, 0.0, 0.0};
    for (int64_t i = (int64_t)blockIdx.x * LT + threadIdx.x; i < nv; i += (int64_t)gridDim.x * LT) {
        double y[3];
        for (int c = 0; c < 3; ++c) y[c] = c0 * p[3 * i + c];
        if (ref) {
            const int64_t g = ref[i];
            const double w2 = cellw[g] * cellw[g];
            for (int c = 0; c < 3; ++c) y[c] += w2 * cellsum[3 * g + c];
        }
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
            const int64_t o = other[k];
            const double we = w[key[k] >> 1];
            for (int c = 0; c < 3; ++c) y[c] += we * (p[3 * i + c] - p[3 * o + c]);
        }
        for (int c = 0; c < 3; ++c) {
            Ap[3 * i + c] = y[c];
            acc[c] += p[3 * i + c] * y[c];
        }
    }
    for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] = acc[c];
    __syncthreads();
    for (int o = LT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int c = 0; c < 3; ++c) partial[3 * blockIdx.x + c] = sh[c][0];
}

// cellsum[g] = sum of p over cell g's members, in vertex order.
__global__ void k_lin_cellsum(int64_t ng, const int32_t* __restrict__ cell_ptr, const int32_t* __restrict__ mem,
                              const double* __restrict__ p, double* __restrict__ cellsum) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    double s[3] = {0.0, 0.0, 0.0};
    for (int k = cell_ptr[g]; k < cell_ptr[g + 1]; ++k) {
        const int64_t j = mem[k];
        for (int c = 0; c < 3; ++c) s[c] += p[3 * j + c];
    }
    for (int c = 0; c < 3; ++c) cellsum[3 * g + c] = s[c];
}

// Fixed-order sum of the block partials into out[3].
__global__ void __launch_bounds__(LT) k_lin_reduce(const double* __restrict__ partial, int nblocks,
                                                   double* __restrict__ out) {
    __shared__ double sh[3][LT];
    for (int c = 0; c < 3; ++c) {
        double a = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += LT) a += partial[3 * b + c];
        sh[c][threadIdx.x] = a;
    }
    __syncthreads();
    for (int o = LT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int c = 0; c < 3; ++c) out[c] = sh[c][0];
}

// scal: rz[0..2] pAp[3..5] alpha[6..8] beta[9..11] rz_new[12..14] bb[15..17]
// x += alpha p, r -= alpha Ap, z = r / diag; partial = r.z per column.
__global__ void __launch_bounds__(LT) k_lin_update(int64_t nv, double* __restrict__ scal, double* __restrict__ x,
                                                   double* __restrict__ r, double* __restrict__ z,
                                                   const double* __restrict__ p, const double* __restrict__ Ap,
                                                   const double* __restrict__ diag, double* __restrict__ partial) {
    __shared__ double sh[3][LT];
    __shared__ double alpha[3];
    if (threadIdx.x < 3) {
        const double pap = scal[3 + threadIdx.x];
        alpha[threadIdx.x] = pap > 0.0 ? scal[threadIdx.x] / pap : 0.0;
    }
    __syncthreads();
    double acc[3] = {0.0, 0.0, 0.0};
    for (int64_t i = (int64_t)blockIdx.x * LT + threadIdx.x; i < nv; i += (int64_t)gridDim.x * LT) {
        const double di = diag[i];
        for (int c = 0; c < 3; ++c) {
            const int64_t k = 3 * i + c;
            x[k] += alpha[c] * p[k];
            const double rk = r[k] - alpha[c] * Ap[k];
            r[k] = rk;
            const double zk = rk / di;
            z[k] = zk;
            acc[c] += rk * zk;
        }
    }
    for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] = acc[c];
    __syncthreads();
    for (int o = LT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int c = 0; c < 3; ++c) partial[3 * blockIdx.x + c] = sh[c][0];
}

// p = z + beta p with beta = rz_new / rz; then rz = rz_new.  Block 0 thread c
// rolls the scalars after every block has read them (next launch).
__global__ void __launch_bounds__(LT) k_lin_direction(int64_t nv, const double* __restrict__ scal,
                                                      const double* __restrict__ z, double* __restrict__ p) {
    double beta[3];
    for (int c = 0; c < 3; ++c) beta[c] = scal[c] > 0.0 ? scal[12 + c] / scal[c] : 0.0;
    for (int64_t i = (int64_t)blockIdx.x * LT + threadIdx.x; i < nv; i += (int64_t)gridDim.x * LT)
        for (int c = 0; c < 3; ++c) p[3 * i + c] = z[3 * i + c] + beta[c] * p[3 * i + c];
}

__global__ void k_lin_roll(double* scal) {
    if (threadIdx.x < 3) scal[threadIdx.x] = scal[12 + threadIdx.x];
}

// r = B - A x (B in r), z = r / diag, p = z; partial = r.z and b.b per column.
__global__ void __launch_bounds__(LT) k_lin_start(int64_t nv, double* __restrict__ r, const double* __restrict__ Ax,
                                                  const double* __restrict__ diag, double* __restrict__ z,
                                                  double* __restrict__ p, double* __restrict__ partial) {
    __shared__ double sh[6][LT];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t i = (int64_t)blockIdx.x * LT + threadIdx.x; i < nv; i += (int64_t)gridDim.x * LT) {
        for (int c = 0; c < 3; ++c) {
            const int64_t k = 3 * i + c;
            const double b = r[k];
            const double rk = b - Ax[k];
            r[k] = rk;
            const double zk = rk / diag[i];
            z[k] = zk;
            p[k] = zk;
            acc[c] += rk * zk;
            acc[3 + c] += b * b;
        }
    }
    for (int c = 0; c < 6; ++c) sh[c][threadIdx.x] = acc[c];
    __syncthreads();
    for (int o = LT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int c = 0; c < 6; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int c = 0; c < 3; ++c) partial[3 * blockIdx.x + c] = sh[c][0];
        for (int c = 0; c < 3; ++c) partial[3 * (LBLOCKS + blockIdx.x) + c] = sh[3 + c][0];
    }
}

__global__ void k_lin_to_float(const double* __restrict__ x, int64_t n, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)x[i];
}

// ||r||^2 per column into out[3] (for the convergence check).
__global__ void __launch_bounds__(LT) k_lin_rr(int64_t nv, const double* __restrict__ r, double* __restrict__ partial) {
    __shared__ double sh[3][LT];
    double acc[3] = {0, 0, 0};
    for (int64_t i = (int64_t)blockIdx.x * LT + threadIdx.x; i < nv; i += (int64_t)gridDim.x * LT)
        for (int c = 0; c < 3; ++c) acc[c] += r[3 * i + c] * r[3 * i + c];
    for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] = acc[c];
    __syncthreads();
    for (int o = LT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int c = 0; c < 3; ++c) partial[3 * blockIdx.x + c] = sh[c][0];
}

}  // namespace
}  // namespace mo

using namespace mo;

namespace {
int solve_on(float* V, int64_t nv, const int32_t* F, int64_t nf, const int32_t* E, int64_t ne, const int32_t* ref,
             const float* G, int64_t ng, double rigidity, int with_rot, double tol, int max_iter, void* scratch,
             size_t scratch_bytes, int* iters_out, double* rel_residual_out, cudaStream_t s);
}  // namespace

extern "C" size_t mo_solve_linear_scratch_bytes(int64_t nv, int64_t nf, int64_t ne, int64_t ng, int with_rot) {
    if (nv < 0 || nf < 0 || ne < 0 || ng < 0) return 0;
    return plan(nullptr, nv, nf, ne, ng, with_rot ? 1 : 0).bytes;
}

extern "C" int mo_solve_linear(float* V, int64_t nv, const int32_t* F, int64_t nf, const int32_t* E, int64_t ne,
                               const int32_t* ref, const float* G, int64_t ng, double rigidity, int with_rot,
                               double tol, int max_iter, void* scratch, size_t scratch_bytes, int* iters_out,
                               double* rel_residual_out, void* stream) {
    with_rot = with_rot ? 1 : 0;
    MO_CHECK_ARG(nv > 0 && nf >= 0 && ne >= 0 && ng >= 0, "bad sizes");
    MO_CHECK_ARG(nv < ((int64_t)1 << 30) && 3 * nf + ne < ((int64_t)1 << 30), "system too large");
    MO_CHECK_ARG(V && G && (nf == 0 || F), "null pointer");
    MO_CHECK_ARG(with_rot || ((ne == 0 || E) && ref && ng > 0), "LinearEstimation needs references and a graph");
    MO_CHECK_ARG(!with_rot || ng == nv, "with_rot needs one target position per vertex (ng == nv)");
    MO_CHECK_ARG(tol > 0.0 && max_iter > 0, "bad tolerance or iteration limit");
    MO_CHECK_ARG(std::isfinite(rigidity), "bad rigidity");
    // The iterations are captured as a CUDA graph, which the caller's stream
    // (possibly the legacy default stream) may not allow: the solve runs on a
    // stream of its own that first waits for the caller's work.
    cudaStream_t caller = as_stream(stream);
    cudaStream_t s = nullptr;
    cudaEvent_t ready = nullptr;
    MO_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaError_t e0 = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
    if (e0 == cudaSuccess) e0 = cudaEventRecord(ready, caller);
    if (e0 == cudaSuccess) e0 = cudaStreamWaitEvent(s, ready, 0);
    if (ready) cudaEventDestroy(ready);
    if (e0 != cudaSuccess) {
        cudaStreamDestroy(s);
        return cuda_status(e0, "solver stream");
    }
    int rc0 = solve_on(V, nv, F, nf, E, ne, ref, G, ng, rigidity, with_rot, tol, max_iter, scratch, scratch_bytes,
                       iters_out, rel_residual_out, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return rc0;
}

namespace {
int solve_on(float* V, int64_t nv, const int32_t* F, int64_t nf, const int32_t* E, int64_t ne, const int32_t* ref,
             const float* G, int64_t ng, double rigidity, int with_rot, double tol, int max_iter, void* scratch,
             size_t scratch_bytes, int* iters_out, double* rel_residual_out, cudaStream_t s) {
    const LinScratch need = plan(nullptr, nv, nf, ne, ng, with_rot);
    void* owned = nullptr;
    if (!scratch) {
        MO_CUDA(cudaMallocAsync(&owned, need.bytes, s));
        scratch = owned;
    } else if (scratch_bytes < need.bytes) {
        set_error("SolveLinear scratch too small: %zu < %zu", scratch_bytes, need.bytes);
        return MO_ERR_SCRATCH;
    }
    LinScratch S = plan(reinterpret_cast<char*>(scratch), nv, nf, ne, ng, with_rot);
    const int64_t nh = 3 * nf + (with_rot ? 0 : ne);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(LBLOCKS, (nv + LT - 1) / LT));
    int rc = MO_OK;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    auto fail = [&](cudaError_t e, const char* where) { rc = cuda_status(e, where); };
    do {
        cudaError_t e = cudaMemsetAsync(S.status, 0, 16, s);
        if (e != cudaSuccess) { fail(e, "memset"); break; }
        if (nh > 0) {
            k_lin_edges<<<ceil_div(nh, 256), 256, 0, s>>>(F, nf, with_rot ? nullptr : E, with_rot ? 0 : ne, S.edges);
            ::mo::note_launch();
        }
        rc = mo_edge_csr_build(S.edges, nh, MO_EDGES_LIST, nv, S.csr, S.csr_bytes, S.status, s);
        if (rc) break;
        const int* row_ptr = reinterpret_cast<const int*>(S.csr);
        const int* key = row_ptr + (nv + 1);
        const int* other = key + 2 * nh;
        // the status must be clean before any kernel indexes by the edges
        int status = 0;
        e = cudaMemcpyAsync(&status, S.status, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { fail(e, "status"); break; }
        if (status) { set_error("edge or face index out of range [0, %lld)", (long long)nv); rc = MO_ERR_DEVICE; break; }
        k_lin_to_double<<<ceil_div(3 * nv, 256), 256, 0, s>>>(V, 3 * nv, S.V0); ::mo::note_launch();
        k_lin_to_double<<<ceil_div(3 * (with_rot ? nv : ng), 256), 256, 0, s>>>(G, 3 * (with_rot ? nv : ng), S.G);
        ::mo::note_launch();
        if (nh > 0) {
            k_lin_weights<<<ceil_div(nh, 256), 256, 0, s>>>(S.edges, nh, S.V0, rigidity, with_rot, S.w);
            ::mo::note_launch();
        }
        double c0;
        if (!with_rot) {
            k_lin_cell_keys<<<ceil_div(nv, 256), 256, 0, s>>>(ref, nv, ng, S.keys_a, S.vals_a, S.status);
            ::mo::note_launch();
            int bits = 1;
            while (bits < 32 && ((int64_t)1 << bits) < ng) ++bits;
            e = radix_sort_pairs(S.keys_a, S.vals_a, S.keys_b, S.vals_b, (int)nv, bits, S.hist, s);
            if (e != cudaSuccess) { fail(e, "radix_sort_pairs"); break; }
            e = cudaMemcpyAsync(&status, S.status, sizeof(int), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) { fail(e, "status"); break; }
            if (status) { set_error("reference index out of range [0, %lld)", (long long)ng); rc = MO_ERR_DEVICE; break; }
            k_lin_cell_ptr<<<ceil_div(nv, 256), 256, 0, s>>>(S.keys_a, nv, S.cell_ptr); ::mo::note_launch();
            k_lin_cell_tail<<<1, 1, 0, s>>>(S.keys_a, nv, ng, S.cell_ptr); ::mo::note_launch();
            e = cudaMemcpyAsync(S.cell_mem, S.vals_a, 4 * (size_t)nv, cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) { fail(e, "copy"); break; }
            k_lin_cellw<<<ceil_div(ng, 256), 256, 0, s>>>(S.cell_ptr, ng, S.cellw); ::mo::note_launch();
            k_lin_rhs<<<ceil_div(nv, 256), 256, 0, s>>>(nv, row_ptr, other, key, S.w, S.V0, ref, S.G, S.cellw,
                                                        S.diag, S.r);
            ::mo::note_launch();
            c0 = 1e-6;
        } else {
            k_lin_rotations<<<ceil_div(nv, 128), 128, 0, s>>>(nv, row_ptr, other, S.V0, S.G, S.rot); ::mo::note_launch();
            k_lin_rhs_rot<<<ceil_div(nv, 256), 256, 0, s>>>(nv, row_ptr, other, key, S.w, S.V0, S.G, S.rot, S.diag,
                                                            S.r);
            ::mo::note_launch();
            c0 = 1.0;
        }
        const int32_t* cref = with_rot ? nullptr : ref;
        // start from the input positions: r = B - A x0
        e = cudaMemcpyAsync(S.x, S.V0, 24 * (size_t)nv, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) { fail(e, "copy"); break; }
        if (cref) {
            k_lin_cellsum<<<ceil_div(ng, 256), 256, 0, s>>>(ng, S.cell_ptr, S.cell_mem, S.x, S.cellsum);
            ::mo::note_launch();
        }
        k_lin_apply<<<blocks, LT, 0, s>>>(nv, row_ptr, other, key, S.w, cref, S.cellw, S.cellsum, c0, S.x, S.Ap,
                                          S.partial);
        ::mo::note_launch();
        k_lin_start<<<blocks, LT, 0, s>>>(nv, S.r, S.Ap, S.diag, S.z, S.p, S.partial); ::mo::note_launch();
        k_lin_reduce<<<1, LT, 0, s>>>(S.partial, blocks, S.scal); ::mo::note_launch();                  // rz
        k_lin_reduce<<<1, LT, 0, s>>>(S.partial + 3 * LBLOCKS, blocks, S.scal + 15); ::mo::note_launch(); // bb
        e = cudaGetLastError();
        if (e != cudaSuccess) { fail(e, "cg start"); break; }
        // one iteration, captured once
        e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) { fail(e, "capture"); break; }
        if (cref) k_lin_cellsum<<<ceil_div(ng, 256), 256, 0, s>>>(ng, S.cell_ptr, S.cell_mem, S.p, S.cellsum);
        k_lin_apply<<<blocks, LT, 0, s>>>(nv, row_ptr, other, key, S.w, cref, S.cellw, S.cellsum, c0, S.p, S.Ap,
                                          S.partial);
        k_lin_reduce<<<1, LT, 0, s>>>(S.partial, blocks, S.scal + 3);  // pAp
        k_lin_update<<<blocks, LT, 0, s>>>(nv, S.scal, S.x, S.r, S.z, S.p, S.Ap, S.diag, S.partial);
        k_lin_reduce<<<1, LT, 0, s>>>(S.partial, blocks, S.scal + 12);  // rz_new
        k_lin_direction<<<blocks, LT, 0, s>>>(nv, S.scal, S.z, S.p);
        k_lin_roll<<<1, 32, 0, s>>>(S.scal);
        e = cudaStreamEndCapture(s, &graph);
        if (e != cudaSuccess) { fail(e, "capture"); break; }
        e = cudaGraphInstantiate(&exec, graph, 0);
        if (e != cudaSuccess) { fail(e, "instantiate"); break; }
        double bb[3];
        e = cudaMemcpyAsync(bb, S.scal + 15, sizeof(bb), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { fail(e, "read"); break; }
        // convergence: max over columns of ||r|| / ||b|| <= tol, checked every
        // `check` iterations; the iteration count is bounded by max_iter
        const int check = 32;
        int it = 0;
        double rel = INFINITY;
        while (it < max_iter) {
            const int n = std::min(check, max_iter - it);
            for (int k = 0; k < n; ++k) {
                e = cudaGraphLaunch(exec, s);
                if (e != cudaSuccess) break;
            }
            if (e != cudaSuccess) { fail(e, "cg iteration"); break; }
            it += n;
            k_lin_rr<<<blocks, LT, 0, s>>>(nv, S.r, S.partial); ::mo::note_launch();
            k_lin_reduce<<<1, LT, 0, s>>>(S.partial, blocks, S.scal + 6); ::mo::note_launch();
            double rr[3];
            e = cudaMemcpyAsync(rr, S.scal + 6, sizeof(rr), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) { fail(e, "residual"); break; }
            rel = 0.0;
            for (int c = 0; c < 3; ++c) rel = std::max(rel, bb[c] > 0.0 ? std::sqrt(rr[c] / bb[c]) : std::sqrt(rr[c]));
            if (!(rel > tol)) break;
        }
        if (rc) break;
        if (iters_out) *iters_out = it;
        if (rel_residual_out) *rel_residual_out = rel;
        k_lin_to_float<<<ceil_div(3 * nv, 256), 256, 0, s>>>(S.x, 3 * nv, V); ::mo::note_launch();
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { fail(e, "solve"); break; }
        if (!(rel <= tol)) {
            set_error("conjugate gradients did not reach %g in %d iterations (relative residual %g)", tol, it, rel);
            rc = MO_ERR_DEVICE;
        }
    } while (0);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (owned) cudaFreeAsync(owned, s);
    return rc;
}
}  // namespace
