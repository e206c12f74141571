// Quaternion functions for the reference's Camera.cpp and SceneNode.cpp,
// written from the quaternion algebra:
//   mat4_cast:  the rotation matrix of a unit quaternion, 1 - 2(yy+zz),
//               2(xy+wz), 2(xz-wy) in column 0 and so on
//   angleAxis:  (cos(a/2), axis*sin(a/2)), the axis taken as given
//   cross:      the Hamilton product p q
//   normalize:  q / |q|, with |q| = sqrt((xx+yy) + (zz+ww)); identity if |q| = 0
#pragma once
#include "../glm.hpp"
#include "matrix_transform.hpp"

namespace glm {

ATX_GLM_FN mat4 mat4_cast(const quat& q)
{
    const float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    const float xz = q.x * q.z, xy = q.x * q.y, yz = q.y * q.z;
    const float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    mat4 r(1.0f);
    r[0][0] = 1.0f - 2.0f * (yy + zz);
    r[0][1] = 2.0f * (xy + wz);
    r[0][2] = 2.0f * (xz - wy);
    r[1][0] = 2.0f * (xy - wz);
    r[1][1] = 1.0f - 2.0f * (xx + zz);
    r[1][2] = 2.0f * (yz + wx);
    r[2][0] = 2.0f * (xz + wy);
    r[2][1] = 2.0f * (yz - wx);
    r[2][2] = 1.0f - 2.0f * (xx + yy);
    return r;
}

ATX_GLM_FN quat angleAxis(float angle, vec3 axis)
{
    const float s = sinf(angle * 0.5f);
    return quat(cosf(angle * 0.5f), axis.x * s, axis.y * s, axis.z * s);
}

ATX_GLM_FN quat cross(const quat& p, const quat& q)
{
    return quat(p.w * q.w - p.x * q.x - p.y * q.y - p.z * q.z, p.w * q.x + p.x * q.w + p.y * q.z - p.z * q.y,
                p.w * q.y + p.y * q.w + p.z * q.x - p.x * q.z, p.w * q.z + p.z * q.w + p.x * q.y - p.y * q.x);
}

ATX_GLM_FN quat normalize(const quat& q)
{
    const float len = sqrtf((q.x * q.x + q.y * q.y) + (q.z * q.z + q.w * q.w));
    if (len <= 0.0f) return quat(1.0f, 0.0f, 0.0f, 0.0f);
    const float inv = 1.0f / len;
    return quat(q.w * inv, q.x * inv, q.y * inv, q.z * inv);
}

}  // namespace glm
