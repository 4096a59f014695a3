// Stand-in for libigl's igl::point_mesh_squared_distance (an un-vendored
// submodule of the reference): for every row p of P the exact squared
// distance to the nearest triangle of (V, F) and that triangle's index; the
// closest points C are not computed (NaN: Mesh::ConstructDistanceField, the
// one caller in the compiled sources, ignores them).  The distances come from the oracle's FP64 point-triangle
// distance over its AABB tree (orc_point_mesh_sqdist in
// oracle/meshode_oracle.c), so this part of oracle/_ref is the oracle's
// restatement of libigl, not libigl.
#ifndef MO_REFSHIM_IGL_PMSD_
#define MO_REFSHIM_IGL_PMSD_

#include <Eigen/Core>
#include <cstdint>
#include <stdexcept>

extern "C" int orc_point_mesh_sqdist(const double* P, int64_t np, const double* V, int64_t nv, const int* F,
                                     int64_t nf, double* sqrD, int* I, double* C, int nthreads);

namespace igl {
template <class DP, class DV, class DF, class DS, class DI, class DC>
void point_mesh_squared_distance(const DP& P, const DV& V, const DF& F, DS& sqrD, DI& I, DC& C) {
    const int np = P.rows();
    sqrD.resize(np, 1);
    I.resize(np, 1);
    C.resize(np, 3);
    const int rc = orc_point_mesh_sqdist(P.data(), np, V.data(), V.rows(), F.data(), F.rows(), sqrD.data(),
                                         I.data(), C.data(), 0);
    if (rc != 0) throw std::runtime_error("point_mesh_squared_distance stand-in failed");
}
}  // namespace igl

#endif
