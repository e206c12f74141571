// glm::rotate(quat, vec3) for the reference's Camera.cpp: the rotation of v
// by a unit quaternion q = (w, u), v + 2 (w (u x v) + u x (u x v)).
#pragma once
#include "../gtc/quaternion.hpp"

namespace glm {

ATX_GLM_FN vec3 rotate(const quat& q, vec3 v)
{
    const vec3 u(q.x, q.y, q.z);
    const vec3 uv = cross(u, v);
    const vec3 uuv = cross(u, uv);
    return v + ((uv * q.w) + uuv) * 2.0f;
}

}  // namespace glm
