// Project-written stand-in for glm's length2 (squared Euclidean length over all
// components, summed x, y, z, w in that order). Test infrastructure only.
#ifndef NBODY_SHIM_GLM_GTX_NORM_HPP
#define NBODY_SHIM_GLM_GTX_NORM_HPP

#include "../glm.hpp"

namespace glm {
inline float length2(const vec4 &v) { return v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w; }
inline float length2(const vec3 &v) { return v.x * v.x + v.y * v.y + v.z * v.z; }
}  // namespace glm

#endif
