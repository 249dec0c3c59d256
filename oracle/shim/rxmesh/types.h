// Stand-in for rxmesh/types.h with only the vector alias geometry_util.cuh
// uses (the real header also pulls in the logging and CUDA macros).
#pragma once
#include <glm/glm.hpp>

namespace rxmesh {
template <typename T, int N>
using vec = glm::vec<N, T, glm::defaultp>;
template <typename T>
using vec3 = vec<T, 3>;
}  // namespace rxmesh
