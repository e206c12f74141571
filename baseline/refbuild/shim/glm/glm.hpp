// Minimal vector-math header standing in for glm, so that the reference's own
// render path (Engine/src/Renderer.cu, BRDF.cu, Camera.cpp, SceneNode.cpp) can
// be compiled unmodified without its un-vendored thirdparty/glm submodule.
//
// Written from the mathematics, for exactly the names those files use:
//   - vec2/vec3/vec4 of float, mat4 as four float columns, quat (x, y, z, w)
//   - component-wise arithmetic, dot, cross, length, normalize (v * 1/sqrt(v.v)),
//     mix (x*(1-a) + y*a, the GLSL definition), min/max/clamp (compare and
//     select), pi, radians
//   - mat4 * vec4 as a combination of columns summed pairwise,
//     (c0*v0 + c1*v1) + (c2*v2 + c3*v3); mat4 * mat4 column by column as
//     left-to-right sums (the conventions the project's own host code uses)
// Layouts are the plain float aggregates the reference's POD structs assume
// (vec3 = 12 B, vec4 = 16 B, 4-byte alignment), so Sphere is 20 B, Material
// 52 B, Light 28 B and DeviceCamera 40 B as in the reference.
//
// With GLM_FORCE_CUDA (Engine/include/Scene.h:5) every function is
// __host__ __device__; the reference's -use_fast_math then applies to them as
// it would to the real header's inline code.  Square roots and trigonometry
// call the float functions (sqrtf, tanf, sinf, cosf) on host and device alike:
// an unqualified sqrt of a float would resolve to the double function on the
// host and round twice.
#pragma once

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define ATX_GLM_FN __host__ __device__ inline
#define ATX_GLM_CFN __host__ __device__ constexpr
#else
#define ATX_GLM_FN inline
#define ATX_GLM_CFN constexpr
#endif

namespace glm {

struct vec2 {
    float x, y;
    vec2() = default;
    ATX_GLM_CFN explicit vec2(float s) : x(s), y(s) {}
    ATX_GLM_CFN vec2(float a, float b) : x(a), y(b) {}
    ATX_GLM_FN float& operator[](int i) { return i == 0 ? x : y; }
    ATX_GLM_FN float operator[](int i) const { return i == 0 ? x : y; }
};

struct vec4;

struct vec3 {
    float x, y, z;
    vec3() = default;
    ATX_GLM_CFN explicit vec3(float s) : x(s), y(s), z(s) {}
    ATX_GLM_CFN vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    ATX_GLM_CFN explicit vec3(const vec4& v);
    ATX_GLM_FN float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    ATX_GLM_FN float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct vec4 {
    float x, y, z, w;
    vec4() = default;
    ATX_GLM_CFN explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    ATX_GLM_CFN vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    ATX_GLM_CFN vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    ATX_GLM_FN float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    ATX_GLM_FN float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

ATX_GLM_CFN vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

// ---- vec2 ----
ATX_GLM_FN vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
ATX_GLM_FN vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
ATX_GLM_FN vec2 operator-(vec2 a, float s) { return vec2(a.x - s, a.y - s); }
ATX_GLM_FN vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
ATX_GLM_FN vec2 operator*(float s, vec2 a) { return vec2(s * a.x, s * a.y); }
ATX_GLM_FN float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }

// ---- vec3 ----
ATX_GLM_FN vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
ATX_GLM_FN vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
ATX_GLM_FN vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
ATX_GLM_FN vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
ATX_GLM_FN vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
ATX_GLM_FN vec3 operator+(vec3 a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
ATX_GLM_FN vec3 operator-(vec3 a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
ATX_GLM_FN vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
ATX_GLM_FN vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
ATX_GLM_FN vec3 operator+(float s, vec3 a) { return vec3(s + a.x, s + a.y, s + a.z); }
ATX_GLM_FN vec3 operator-(float s, vec3 a) { return vec3(s - a.x, s - a.y, s - a.z); }
ATX_GLM_FN vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
ATX_GLM_FN vec3 operator/(float s, vec3 a) { return vec3(s / a.x, s / a.y, s / a.z); }
ATX_GLM_FN vec3& operator+=(vec3& a, vec3 b) { a = a + b; return a; }
ATX_GLM_FN vec3& operator-=(vec3& a, vec3 b) { a = a - b; return a; }
ATX_GLM_FN vec3& operator*=(vec3& a, vec3 b) { a = a * b; return a; }
ATX_GLM_FN vec3& operator*=(vec3& a, float s) { a = a * s; return a; }
ATX_GLM_FN vec3& operator/=(vec3& a, float s) { a = a / s; return a; }
ATX_GLM_FN bool operator==(vec3 a, vec3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
ATX_GLM_FN bool operator!=(vec3 a, vec3 b) { return !(a == b); }

ATX_GLM_FN float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
ATX_GLM_FN vec3 cross(vec3 a, vec3 b)
{
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
ATX_GLM_FN float length(vec3 v) { return sqrtf(dot(v, v)); }
ATX_GLM_FN float inversesqrt(float x) { return 1.0f / sqrtf(x); }
ATX_GLM_FN vec3 normalize(vec3 v) { return v * inversesqrt(dot(v, v)); }

// ---- vec4 ----
ATX_GLM_FN vec4 operator+(vec4 a, vec4 b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
ATX_GLM_FN vec4 operator-(vec4 a, vec4 b) { return vec4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
ATX_GLM_FN vec4 operator*(vec4 a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
ATX_GLM_FN vec4 operator*(float s, vec4 a) { return vec4(s * a.x, s * a.y, s * a.z, s * a.w); }
ATX_GLM_FN vec4 operator/(vec4 a, float s) { return vec4(a.x / s, a.y / s, a.z / s, a.w / s); }
ATX_GLM_FN vec4& operator+=(vec4& a, vec4 b) { a = a + b; return a; }

// ---- scalar helpers (compare and select, as in GLSL) ----
ATX_GLM_FN float min(float a, float b) { return (b < a) ? b : a; }
ATX_GLM_FN float max(float a, float b) { return (a < b) ? b : a; }
ATX_GLM_FN float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
ATX_GLM_FN vec4 clamp(vec4 v, float lo, float hi)
{
    return vec4(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi), clamp(v.w, lo, hi));
}
ATX_GLM_FN vec3 mix(vec3 x, vec3 y, float a) { return x * (1.0f - a) + y * a; }

template <typename T> ATX_GLM_CFN T pi() { return T(3.14159265358979323846264338327950288); }
ATX_GLM_FN float radians(float deg) { return deg * 0.01745329251994329576923690768489f; }

// ---- mat4: four columns ----
struct mat4 {
    vec4 c[4];
    mat4() = default;
    ATX_GLM_CFN explicit mat4(float s)
        : c{vec4(s, 0.0f, 0.0f, 0.0f), vec4(0.0f, s, 0.0f, 0.0f), vec4(0.0f, 0.0f, s, 0.0f), vec4(0.0f, 0.0f, 0.0f, s)}
    {
    }
    ATX_GLM_CFN mat4(vec4 a, vec4 b, vec4 d, vec4 e) : c{a, b, d, e} {}
    ATX_GLM_FN vec4& operator[](int i) { return c[i]; }
    ATX_GLM_FN const vec4& operator[](int i) const { return c[i]; }
};

ATX_GLM_FN vec4 operator*(const mat4& m, vec4 v)
{
    return (m[0] * v.x + m[1] * v.y) + (m[2] * v.z + m[3] * v.w);
}

ATX_GLM_FN mat4 operator*(const mat4& a, const mat4& b)
{
    mat4 r;
    for (int j = 0; j < 4; ++j)
        r[j] = ((a[0] * b[j].x + a[1] * b[j].y) + a[2] * b[j].z) + a[3] * b[j].w;
    return r;
}

// Inverse by cofactors: 2x2 minors of the top two rows (s*) and of the bottom
// two rows (c*), determinant from their products, adjugate over determinant.
ATX_GLM_FN mat4 inverse(const mat4& m)
{
    auto A = [&](int r, int col) { return m[col][r]; };
    const float s0 = A(0, 0) * A(1, 1) - A(1, 0) * A(0, 1);
    const float s1 = A(0, 0) * A(1, 2) - A(1, 0) * A(0, 2);
    const float s2 = A(0, 0) * A(1, 3) - A(1, 0) * A(0, 3);
    const float s3 = A(0, 1) * A(1, 2) - A(1, 1) * A(0, 2);
    const float s4 = A(0, 1) * A(1, 3) - A(1, 1) * A(0, 3);
    const float s5 = A(0, 2) * A(1, 3) - A(1, 2) * A(0, 3);
    const float c5 = A(2, 2) * A(3, 3) - A(3, 2) * A(2, 3);
    const float c4 = A(2, 1) * A(3, 3) - A(3, 1) * A(2, 3);
    const float c3 = A(2, 1) * A(3, 2) - A(3, 1) * A(2, 2);
    const float c2 = A(2, 0) * A(3, 3) - A(3, 0) * A(2, 3);
    const float c1 = A(2, 0) * A(3, 2) - A(3, 0) * A(2, 2);
    const float c0 = A(2, 0) * A(3, 1) - A(3, 0) * A(2, 1);
    const float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    const float id = 1.0f / det;
    float b[4][4];
    b[0][0] = (A(1, 1) * c5 - A(1, 2) * c4 + A(1, 3) * c3) * id;
    b[0][1] = (-A(0, 1) * c5 + A(0, 2) * c4 - A(0, 3) * c3) * id;
    b[0][2] = (A(3, 1) * s5 - A(3, 2) * s4 + A(3, 3) * s3) * id;
    b[0][3] = (-A(2, 1) * s5 + A(2, 2) * s4 - A(2, 3) * s3) * id;
    b[1][0] = (-A(1, 0) * c5 + A(1, 2) * c2 - A(1, 3) * c1) * id;
    b[1][1] = (A(0, 0) * c5 - A(0, 2) * c2 + A(0, 3) * c1) * id;
    b[1][2] = (-A(3, 0) * s5 + A(3, 2) * s2 - A(3, 3) * s1) * id;
    b[1][3] = (A(2, 0) * s5 - A(2, 2) * s2 + A(2, 3) * s1) * id;
    b[2][0] = (A(1, 0) * c4 - A(1, 1) * c2 + A(1, 3) * c0) * id;
    b[2][1] = (-A(0, 0) * c4 + A(0, 1) * c2 - A(0, 3) * c0) * id;
    b[2][2] = (A(3, 0) * s4 - A(3, 1) * s2 + A(3, 3) * s0) * id;
    b[2][3] = (-A(2, 0) * s4 + A(2, 1) * s2 - A(2, 3) * s0) * id;
    b[3][0] = (-A(1, 0) * c3 + A(1, 1) * c1 - A(1, 2) * c0) * id;
    b[3][1] = (A(0, 0) * c3 - A(0, 1) * c1 + A(0, 2) * c0) * id;
    b[3][2] = (-A(3, 0) * s3 + A(3, 1) * s1 - A(3, 2) * s0) * id;
    b[3][3] = (A(2, 0) * s3 - A(2, 1) * s1 + A(2, 2) * s0) * id;
    mat4 r;
    for (int row = 0; row < 4; ++row)
        for (int col = 0; col < 4; ++col) r[col][row] = b[row][col];
    return r;
}

// ---- quat, stored x, y, z, w; constructed (w, x, y, z) ----
struct quat {
    float x, y, z, w;
    quat() = default;
    ATX_GLM_CFN quat(float w_, float x_, float y_, float z_) : x(x_), y(y_), z(z_), w(w_) {}
};

}  // namespace glm
