// Projection and transform matrices for the reference's Camera.cpp and
// SceneNode.cpp, written from their definitions (right-handed, clip depth in
// [-1, 1], the OpenGL conventions):
//   perspective: P[0][0] = 1/(aspect*tan(fovy/2)), P[1][1] = 1/tan(fovy/2),
//                P[2][2] = -(f+n)/(f-n), P[2][3] = -1, P[3][2] = -2fn/(f-n)
//   lookAt:      f = normalize(center-eye), s = normalize(f x up), u = s x f;
//                rows s, u, -f; translation -s.eye, -u.eye, f.eye
//   translate:   column 3 = m0*v.x + m1*v.y + m2*v.z + m3
//   scale:       columns 0..2 multiplied by v.x, v.y, v.z
#pragma once
#include "../glm.hpp"

namespace glm {

ATX_GLM_FN mat4 perspective(float fovy, float aspect, float zNear, float zFar)
{
    const float th = tanf(fovy / 2.0f);
    mat4 r(0.0f);
    r[0][0] = 1.0f / (aspect * th);
    r[1][1] = 1.0f / th;
    r[2][2] = -(zFar + zNear) / (zFar - zNear);
    r[2][3] = -1.0f;
    r[3][2] = -(2.0f * zFar * zNear) / (zFar - zNear);
    return r;
}

ATX_GLM_FN mat4 lookAt(vec3 eye, vec3 center, vec3 up)
{
    const vec3 f = normalize(center - eye);
    const vec3 s = normalize(cross(f, up));
    const vec3 u = cross(s, f);
    mat4 r(1.0f);
    r[0][0] = s.x; r[1][0] = s.y; r[2][0] = s.z;
    r[0][1] = u.x; r[1][1] = u.y; r[2][1] = u.z;
    r[0][2] = -f.x; r[1][2] = -f.y; r[2][2] = -f.z;
    r[3][0] = -dot(s, eye);
    r[3][1] = -dot(u, eye);
    r[3][2] = dot(f, eye);
    return r;
}

ATX_GLM_FN mat4 translate(const mat4& m, vec3 v)
{
    mat4 r = m;
    r[3] = ((m[0] * v.x + m[1] * v.y) + m[2] * v.z) + m[3];
    return r;
}

ATX_GLM_FN mat4 scale(const mat4& m, vec3 v)
{
    return mat4(m[0] * v.x, m[1] * v.y, m[2] * v.z, m[3]);
}

}  // namespace glm
