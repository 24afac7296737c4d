// glmshim/glm/gtx/component_wise.hpp -- TEST INFRASTRUCTURE ONLY (see ../glm.hpp).
#ifndef VKHR_GLMSHIM_COMPONENT_WISE_HPP
#define VKHR_GLMSHIM_COMPONENT_WISE_HPP
#include "../glm.hpp"
namespace glm {
inline float compMax(const vec3& v) { return max(max(v.x, v.y), v.z); }
}
#endif
