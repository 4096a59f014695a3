// libigl's marching cubes is only reached by Mesh::FromDistanceField, which no
// pyDeform function calls; the stand-in refuses.
#ifndef MO_REFSHIM_IGL_MC_
#define MO_REFSHIM_IGL_MC_

#include <stdexcept>

namespace igl {
namespace copyleft {
template <class DS, class DGV, class DV, class DF>
void marching_cubes(const DS&, const DGV&, int, int, int, DV&, DF&) {
    throw std::runtime_error("marching_cubes is not part of oracle/_ref");
}
}  // namespace copyleft
}  // namespace igl

#endif
