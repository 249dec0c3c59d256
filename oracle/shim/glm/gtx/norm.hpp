// Stand-in for glm/gtx/norm.hpp: length2 (squared length) only.
#pragma once
#include <glm/glm.hpp>

namespace glm {
template <typename T, qualifier Q>
inline T length2(const vec<3, T, Q>& a)
{
    return dot(a, a);
}
}  // namespace glm
