// C entry points over the reference's own pyDeform functions, for
// oracle/_ref/libpydeform_ref.so (test infrastructure, never the product).
//
// The reference's sources (src/lib/uniformgrid.cc, src/lib/mesh.cc,
// src/interface/{deform_params,mesh_tensor,distance_layer,rigid_layer,
// graph_layer,cad_layer,normalize}.cc) are compiled unchanged from the
// reference tree by oracle/build_ref.py, against the stand-in headers under
// oracle/ref_shim (Eigen, ceres::Jet, torch::Tensor, libigl).  This file only
// moves plain arrays in and out of the reference's torch::Tensor arguments;
// every number comes from the reference's own loops.  Each wrapper returns 0,
// or -1 after storing a message for ref_last_error().
#include <cstdint>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <string>

#include "cad_layer.h"
#include "deform_params.h"
#include "distance_layer.h"
#include "graph_layer.h"
#include "mesh_tensor.h"
#include "normalize.h"
#include "rigid_layer.h"
#include "subdivision.h"

#define REF_EXPORT extern "C" __attribute__((visibility("default")))

namespace {
std::string g_err;

using torch::refshim::wrap;

torch::Tensor vtx(const float* V, int64_t n) { return wrap(V, {n, 3}, torch::kFloat32); }
torch::Tensor idx(const int* I, int64_t n, int64_t cols) { return wrap(I, {n, cols}, torch::kInt32); }

void copy_out(const torch::Tensor& t, void* out) {
    std::memcpy(out, t.storage().data(), (size_t)t.numel() * torch::element_size(t.dtype()));
}

template <class Fn>
int guarded(Fn fn) {
    try {
        fn();
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
    } catch (...) {
        g_err = "unknown exception";
    }
    return -1;
}
}  // namespace

// LoadCadMesh's remeshing (Subdivision, src/lib/subdivision.cc) needs CGAL,
// which the reference does not vendor; it is not part of oracle/_ref.
Subdivision::Subdivision() {}
void Subdivision::Subdivide(const Mesh&, double) { throw std::runtime_error("Subdivision needs CGAL (absent)"); }
void Subdivision::ComputeGeometryNeighbors(double) { throw std::runtime_error("Subdivision needs CGAL (absent)"); }
void Subdivision::ComputeRepresentativeGraph(double) { throw std::runtime_error("Subdivision needs CGAL (absent)"); }

REF_EXPORT const char* ref_last_error(void) { return g_err.c_str(); }

// LoadMesh (mesh_tensor.cc:87-100): counts, then the arrays.
REF_EXPORT int ref_load_mesh_counts(const char* path, int64_t* nv, int64_t* nf) {
    return guarded([&] {
        auto r = LoadMesh(path);
        *nv = r[0].size(0);
        *nf = r[1].size(0);
    });
}
REF_EXPORT int ref_load_mesh(const char* path, float* V, int* F) {
    return guarded([&] {
        auto r = LoadMesh(path);
        copy_out(r[0], V);
        copy_out(r[1], F);
    });
}
// SaveMesh (mesh_tensor.cc:180-186).
REF_EXPORT int ref_save_mesh(const char* path, const float* V, int64_t nv, const int* F, int64_t nf) {
    return guarded([&] { SaveMesh(path, vtx(V, nv), idx(F, nf, 3)); });
}
// Mesh::ReadOBJ + RemoveDegenerated + MergeDuplex, the first steps of
// LoadCadMesh (mesh_tensor.cc:105-107), without the CGAL remeshing.
REF_EXPORT int ref_cad_clean_counts(const char* path, int64_t* nv, int64_t* nf) {
    return guarded([&] {
        Mesh m;
        m.ReadOBJ(path);
        m.RemoveDegenerated();
        m.MergeDuplex();
        *nv = (int64_t)m.GetV().size();
        *nf = (int64_t)m.GetF().size();
    });
}
REF_EXPORT int ref_cad_clean(const char* path, double* V, int* F) {
    return guarded([&] {
        Mesh m;
        m.ReadOBJ(path);
        m.RemoveDegenerated();
        m.MergeDuplex();
        for (size_t i = 0; i < m.GetV().size(); ++i)
            for (int j = 0; j < 3; ++j) V[3 * i + j] = m.GetV()[i][j];
        for (size_t i = 0; i < m.GetF().size(); ++i)
            for (int j = 0; j < 3; ++j) F[3 * i + j] = m.GetF()[i][j];
    });
}

// InitializeDeformTemplate (deform_params.cc:16-40).
REF_EXPORT int ref_init_template(const float* V, int64_t nv, const int* F, int64_t nf, int symmetry, int N,
                                 int* id_out) {
    return guarded([&] { *id_out = InitializeDeformTemplate(vtx(V, nv), idx(F, nf, 3), symmetry, N); });
}
// A template whose grid is given (for probing UniformGrid::DistanceFloat
// on arbitrary grids): grid is [z][y][x] doubles, N^3 of them.
REF_EXPORT int ref_grid_template(const double* grid, int N, int* id_out) {
    return guarded([&] {
        const int id = CreateParams();
        auto& p = GetParams(id);
        p.grid = UniformGrid(N);
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
                for (int k = 0; k < N; ++k) p.grid.SetDistance(i, j, k, grid[((int64_t)i * N + j) * N + k]);
        *id_out = id;
    });
}
REF_EXPORT int ref_template_grid(int id, double* grid_out) {
    return guarded([&] {
        auto& g = GetParams(id).grid;
        const int N = g.Dimension();
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
                for (int k = 0; k < N; ++k) grid_out[((int64_t)i * N + j) * N + k] = g.GetDistance(i, j, k);
    });
}
REF_EXPORT int ref_template_transform(int id, double* scale_trans4) {
    return guarded([&] {
        auto& p = GetParams(id);
        scale_trans4[0] = p.scale;
        for (int j = 0; j < 3; ++j) scale_trans4[1 + j] = p.trans[j];
    });
}
// The rest offsets and weights stored by the Store*Information calls.
REF_EXPORT int ref_template_edges(int id, float* off_out, float* lambda_out) {
    return guarded([&] {
        auto& p = GetParams(id);
        for (size_t i = 0; i < p.edge_offset.size(); ++i)
            for (int j = 0; j < 3; ++j) off_out[3 * i + j] = p.edge_offset[i][j];
        if (lambda_out)
            for (size_t i = 0; i < p.edge_lambda.size(); ++i) lambda_out[i] = p.edge_lambda[i];
    });
}

// NormalizeByTemplate / DenormalizeByTemplate (normalize.cc:5-45), in place.
REF_EXPORT int ref_normalize(float* V, int64_t n, int id) {
    return guarded([&] { NormalizeByTemplate(vtx(V, n), id); });
}
REF_EXPORT int ref_denormalize(float* V, int64_t n, int id) {
    return guarded([&] { DenormalizeByTemplate(vtx(V, n), id); });
}

// DistanceFieldLoss_forward / _backward (distance_layer.cc:8-81).
REF_EXPORT int ref_df_forward(const float* V, int64_t n, int id, float* out) {
    return guarded([&] { copy_out(DistanceFieldLoss_forward(vtx(V, n), id), out); });
}
REF_EXPORT int ref_df_backward(const float* V, int64_t n, int id, float* out) {
    return guarded([&] { copy_out(DistanceFieldLoss_backward(vtx(V, n), id), out); });
}

// StoreRigidityInformation / RigidEdgeLoss_forward / _backward
// (rigid_layer.cc:11-133).
REF_EXPORT int ref_store_rigidity(const float* V, int64_t nv, const int* F, int64_t nf, int id) {
    return guarded([&] { StoreRigidityInformation(vtx(V, nv), idx(F, nf, 3), id); });
}
REF_EXPORT int ref_rigid_forward(const float* V, int64_t nv, const int* F, int64_t nf, int id, float* out) {
    return guarded([&] { copy_out(RigidEdgeLoss_forward(vtx(V, nv), idx(F, nf, 3), id), out); });
}
REF_EXPORT int ref_rigid_backward(const float* V, int64_t nv, const int* F, int64_t nf, int id, float* out) {
    return guarded([&] { copy_out(RigidEdgeLoss_backward(vtx(V, nv), idx(F, nf, 3), id), out); });
}

// StoreGraphInformation / GraphEdgeLoss_forward / _backward
// (graph_layer.cc:11-135).
REF_EXPORT int ref_store_graph(const float* V, int64_t nv, const int* E, int64_t ne, int id) {
    return guarded([&] { StoreGraphInformation(vtx(V, nv), idx(E, ne, 2), id); });
}
REF_EXPORT int ref_graph_forward(const float* V, int64_t nv, const int* E, int64_t ne, int id, float* out) {
    return guarded([&] { copy_out(GraphEdgeLoss_forward(vtx(V, nv), idx(E, ne, 2), id), out); });
}
REF_EXPORT int ref_graph_backward(const float* V, int64_t nv, const int* E, int64_t ne, int id, float* out) {
    return guarded([&] { copy_out(GraphEdgeLoss_backward(vtx(V, nv), idx(E, ne, 2), id), out); });
}

// StoreCadInformation / CadEdgeLoss_forward / _backward (cad_layer.cc:11-223).
REF_EXPORT int ref_store_cad(const float* V, int64_t nv, const int* F, int64_t nf, const int* E, int64_t ne,
                             int id) {
    return guarded([&] { StoreCadInformation(vtx(V, nv), idx(F, nf, 3), idx(E, ne, 2), id); });
}
REF_EXPORT int ref_cad_forward(const float* V, int64_t nv, const int* F, int64_t nf, const int* E, int64_t ne,
                               int id, float* out) {
    return guarded([&] { copy_out(CadEdgeLoss_forward(vtx(V, nv), idx(F, nf, 3), idx(E, ne, 2), id), out); });
}
REF_EXPORT int ref_cad_backward(const float* V, int64_t nv, const int* F, int64_t nf, const int* E, int64_t ne,
                                int id, float* out) {
    return guarded([&] { copy_out(CadEdgeLoss_backward(vtx(V, nv), idx(F, nf, 3), idx(E, ne, 2), id), out); });
}
