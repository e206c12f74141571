/*
 * Oracle driver: instantiates oracle_impl.h in three arithmetic modes and
 * exposes the C entry points declared in oracle.h.  Test infrastructure only
 * (see oracle.h).  Build: oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off).
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Random.h:59-64, the PCG output-permutation hash (state advance by the LCG
 * multiplier/increment, then a random xorshift and a multiply-xorshift). */
uint32_t orc_pcg_hash(uint32_t seed)
{
    uint32_t state = seed * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

float orc_pcg_float(uint32_t* seed)
{
    *seed = orc_pcg_hash(*seed);
    return (float)(*seed) / 4294967296.0f;
}

/* cos(2 pi u) and sin(2 pi u) for the samplers' angle 2*pi*u2.
 * Range reduction is exact: v = u - rint(u) in [-1/2, 1/2], q = rint(4v) the
 * quarter turn and w = v - q/4 in [-1/8, 1/8] (representable, so the fma is
 * exact).  sin and cos of 2*pi*w come from their Maclaurin series in w, with
 * coefficients (2 pi)^k / k! rounded to float, evaluated by Horner's rule in
 * fused multiply-adds; the truncation error for |2 pi w| <= pi/4 is below
 * 2e-9.  The quarter turn then rotates (cos, sin) by q * 90 degrees. */
void orc_sincos2pi(float u, float* c, float* s)
{
    float v = u - rintf(u);
    float q = rintf(v * 4.0f);
    float w = fmaf(q, -0.25f, v);
    float w2 = w * w;
    float ps = fmaf(w2, 0x1.507834p+5f, -0x1.32d2ccp+6f);
    ps = fmaf(w2, ps, 0x1.466bc6p+6f);
    ps = fmaf(w2, ps, -0x1.4abbcep+5f);
    ps = fmaf(w2, ps, 0x1.921fb6p+2f);
    float sn = w * ps;
    float pc = fmaf(w2, -0x1.a6d1f2p+4f, 0x1.e1f506p+5f);
    pc = fmaf(w2, pc, -0x1.55d3c8p+6f);
    pc = fmaf(w2, pc, 0x1.03c1f0p+6f);
    pc = fmaf(w2, pc, -0x1.3bd3ccp+4f);
    float cs = fmaf(w2, pc, 1.0f);
    switch (((int)q) & 3) {
    case 0: *c = cs; *s = sn; break;
    case 1: *c = -sn; *s = cs; break;
    case 2: *c = -cs; *s = -sn; break;
    default: *c = sn; *s = -cs; break;
    }
}

/* Branch-decision sink of one path (orc_decision_hash / orc_decision_events):
 * events go to ev[0..cap) and into an FNV-1a hash of the decision bits (the
 * shadow event's occluder field is recorded but not hashed). */
typedef struct { uint32_t* ev; int32_t cap; int32_t n; uint64_t hash; } orc_sink;

static inline void orc_emit(orc_sink* s, uint32_t kind, int32_t bounce, uint32_t value)
{
    if (!s) return;
    const uint32_t e = (kind << 28) | (((uint32_t)bounce & 0xFFu) << 20) | (value & 0xFFFFFu);
    const uint32_t decision = kind == ORC_EV_SHADOW ? (e & ~(0x3FFFFu << 2)) : e;
    s->hash = (s->hash ^ decision) * 0x100000001b3ull;
    if (s->ev && s->n < s->cap) s->ev[s->n] = e;
    s->n++;
}

/* --------------------------------------------------------- instantiation */

#define REAL float
#define FN(x) ex_##x
#define EXACT 1
#define F64 0
#include "oracle_impl.h"
#undef REAL
#undef FN
#undef EXACT
#undef F64

#define REAL float
#define FN(x) li_##x
#define EXACT 0
#define F64 0
#include "oracle_impl.h"
#undef REAL
#undef FN
#undef EXACT
#undef F64

#define REAL double
#define FN(x) d_##x
#define EXACT 0
#define F64 1
#include "oracle_impl.h"
#undef REAL
#undef FN
#undef EXACT
#undef F64

/* ------------------------------------------------------------ matrices */

/* Inverse by the Laplace expansion in complementary 2x2 minors of the top and
 * bottom row pairs (D. Eberly, "The Laplace Expansion Theorem: Computing the
 * Determinants and Inverses of Matrices").  Column-major in and out. */
void orc_mat4_inverse(const float m[16], float out[16])
{
#define A(r, c) m[(c) * 4 + (r)]
    float s0 = A(0, 0) * A(1, 1) - A(1, 0) * A(0, 1);
    float s1 = A(0, 0) * A(1, 2) - A(1, 0) * A(0, 2);
    float s2 = A(0, 0) * A(1, 3) - A(1, 0) * A(0, 3);
    float s3 = A(0, 1) * A(1, 2) - A(1, 1) * A(0, 2);
    float s4 = A(0, 1) * A(1, 3) - A(1, 1) * A(0, 3);
    float s5 = A(0, 2) * A(1, 3) - A(1, 2) * A(0, 3);
    float c5 = A(2, 2) * A(3, 3) - A(3, 2) * A(2, 3);
    float c4 = A(2, 1) * A(3, 3) - A(3, 1) * A(2, 3);
    float c3 = A(2, 1) * A(3, 2) - A(3, 1) * A(2, 2);
    float c2 = A(2, 0) * A(3, 3) - A(3, 0) * A(2, 3);
    float c1 = A(2, 0) * A(3, 2) - A(3, 0) * A(2, 2);
    float c0 = A(2, 0) * A(3, 1) - A(3, 0) * A(2, 1);
    float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    float id = 1.0f / det;
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
#undef A
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c * 4 + r] = b[r][c];
}

static void v3_normalize(const float a[3], float out[3])
{
    float d = (a[0] * a[0] + a[1] * a[1]) + a[2] * a[2];
    float inv = 1.0f / sqrtf(d);
    out[0] = a[0] * inv; out[1] = a[1] * inv; out[2] = a[2] * inv;
}

static void v3_cross(const float a[3], const float b[3], float out[3])
{
    out[0] = a[1] * b[2] - b[1] * a[2];
    out[1] = a[2] * b[0] - b[2] * a[0];
    out[2] = a[0] * b[1] - b[0] * a[1];
}

static float v3_dot(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

/* Camera.cpp:134-149 (perspective, right-handed, clip z in [-1, 1]) and
 * :151-159 (lookAt from position toward position + direction, up = +Y). */
void orc_camera_matrices(const float pos[3], const float dir[3], float fov_deg, float near_clip,
                         float far_clip, uint32_t width, uint32_t height,
                         float view[16], float inv_view[16], float proj[16], float inv_proj[16])
{
    float aspect = (float)width / (float)height;
    float fovy = fov_deg * 0.01745329251994329576923690768489f;
    float th = tanf(fovy / 2.0f);
    float P[16];
    memset(P, 0, sizeof(P));
    P[0 * 4 + 0] = 1.0f / (aspect * th);
    P[1 * 4 + 1] = 1.0f / th;
    P[2 * 4 + 2] = -(far_clip + near_clip) / (far_clip - near_clip);
    P[2 * 4 + 3] = -1.0f;
    P[3 * 4 + 2] = -(2.0f * far_clip * near_clip) / (far_clip - near_clip);

    float center[3] = { pos[0] + dir[0], pos[1] + dir[1], pos[2] + dir[2] };
    float fwd[3] = { center[0] - pos[0], center[1] - pos[1], center[2] - pos[2] };
    float f[3], s[3], u[3], sx[3];
    const float up[3] = { 0.0f, 1.0f, 0.0f };
    v3_normalize(fwd, f);
    v3_cross(f, up, sx);
    v3_normalize(sx, s);
    v3_cross(s, f, u);
    float V[16];
    memset(V, 0, sizeof(V));
    V[0 * 4 + 0] = s[0]; V[1 * 4 + 0] = s[1]; V[2 * 4 + 0] = s[2];
    V[0 * 4 + 1] = u[0]; V[1 * 4 + 1] = u[1]; V[2 * 4 + 1] = u[2];
    V[0 * 4 + 2] = -f[0]; V[1 * 4 + 2] = -f[1]; V[2 * 4 + 2] = -f[2];
    V[3 * 4 + 0] = -v3_dot(s, pos);
    V[3 * 4 + 1] = -v3_dot(u, pos);
    V[3 * 4 + 2] = v3_dot(f, pos);
    V[3 * 4 + 3] = 1.0f;

    if (proj) memcpy(proj, P, sizeof(P));
    if (view) memcpy(view, V, sizeof(V));
    if (inv_proj) orc_mat4_inverse(P, inv_proj);
    if (inv_view) orc_mat4_inverse(V, inv_view);
}

/* Camera::onUpdate (Camera.cpp:31-108) with the window's input passed in:
 * mouse delta (pos - last) * 0.002; nothing moves unless the right button is
 * held; W/S, A/D, Q/E move at speed 5 along direction, right = direction x up
 * (not normalised) and up, the first key of each pair winning; a mouse delta
 * turns the direction by normalize(angleAxis(-pitch, right) x
 * angleAxis(-yaw, up)) with yaw/pitch = delta * 0.3.  Quaternions are
 * (w, x, y, z); products, normalisation and rotation as glm states them
 * (Hamilton product; q * v = v + 2 (w (q x v) + q x (q x v))).  Returns 1 when
 * the camera moved. */
typedef struct { float w, x, y, z; } orc_quat;

static orc_quat q_angle_axis(float angle, const float axis[3])
{
    const float s = sinf(angle * 0.5f);
    orc_quat q = { cosf(angle * 0.5f), axis[0] * s, axis[1] * s, axis[2] * s };
    return q;
}

static orc_quat q_mul(orc_quat p, orc_quat q)
{
    orc_quat r;
    r.w = p.w * q.w - p.x * q.x - p.y * q.y - p.z * q.z;
    r.x = p.w * q.x + p.x * q.w + p.y * q.z - p.z * q.y;
    r.y = p.w * q.y + p.y * q.w + p.z * q.x - p.x * q.z;
    r.z = p.w * q.z + p.z * q.w + p.x * q.y - p.y * q.x;
    return r;
}

static orc_quat q_normalize(orc_quat q)
{
    const float len = sqrtf((q.x * q.x + q.y * q.y) + (q.z * q.z + q.w * q.w));
    if (len <= 0.0f) {
        orc_quat one = { 1.0f, 0.0f, 0.0f, 0.0f };
        return one;
    }
    const float inv = 1.0f / len;
    orc_quat r = { q.w * inv, q.x * inv, q.y * inv, q.z * inv };
    return r;
}

static void q_rotate(orc_quat q, const float v[3], float out[3])
{
    const float qv[3] = { q.x, q.y, q.z };
    float uv[3], uuv[3];
    v3_cross(qv, v, uv);
    v3_cross(qv, uv, uuv);
    for (int k = 0; k < 3; ++k) out[k] = v[k] + ((uv[k] * q.w) + uuv[k]) * 2.0f;
}

int orc_camera_on_update(float pos[3], float dir[3], float last_mouse[2], const float mouse[2], int right_button,
                         const int keys[6], float dt)
{
    const float mdx = (mouse[0] - last_mouse[0]) * 0.002f;
    const float mdy = (mouse[1] - last_mouse[1]) * 0.002f;
    last_mouse[0] = mouse[0];
    last_mouse[1] = mouse[1];
    if (!right_button) return 0;
    int moved = 0;
    const float up[3] = { 0.0f, 1.0f, 0.0f };
    float right[3];
    v3_cross(dir, up, right);
    const float speed = 5.0f;
    /* keys: W S A D Q E; each pair is if / else if, as Camera.cpp:51-88 */
    const float* axis[3] = { dir, right, up };
    const float sign_first[3] = { 1.0f, -1.0f, -1.0f };   /* W: +dir, A: -right, Q: -up */
    for (int a = 0; a < 3; ++a) {
        float sign = 0.0f;
        if (keys[2 * a]) sign = sign_first[a];
        else if (keys[2 * a + 1]) sign = -sign_first[a];
        if (sign == 0.0f) continue;
        for (int k = 0; k < 3; ++k) {
            const float step = (axis[a][k] * speed) * dt;
            pos[k] = (sign > 0.0f) ? pos[k] + step : pos[k] - step;
        }
        moved = 1;
    }
    if (mdx != 0.0f || mdy != 0.0f) {
        const float yaw = mdx * 0.3f, pitch = mdy * 0.3f;
        const orc_quat q = q_normalize(q_mul(q_angle_axis(-pitch, right), q_angle_axis(-yaw, up)));
        float nd[3];
        q_rotate(q, dir, nd);
        dir[0] = nd[0];
        dir[1] = nd[1];
        dir[2] = nd[2];
        moved = 1;
    }
    return moved;
}

void orc_ray_dirs(int mode, const orc_view* view, float* out)
{
    const uint32_t W = view->width, H = view->height;
#pragma omp parallel for schedule(static)
    for (int64_t y = 0; y < (int64_t)H; ++y) {
        for (uint32_t x = 0; x < W; ++x) {
            float* o = out + 3 * ((uint64_t)y * W + x);
            if (mode == ORC_EXACT) {
                ex_v3 d = ex_primary_dir(view, x, (uint32_t)y);
                o[0] = d.x; o[1] = d.y; o[2] = d.z;
            } else {
                li_v3 d = li_primary_dir(view, x, (uint32_t)y);
                o[0] = d.x; o[1] = d.y; o[2] = d.z;
            }
        }
    }
}

void orc_trace(int mode, const orc_sphere* spheres, int32_t n_spheres, const float* origins,
               const float* dirs, uint64_t n_rays, float* t_out, int32_t* id_out)
{
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n_rays; ++i) {
        float t;
        int32_t id;
        if (mode == ORC_EXACT) {
            id = ex_nearest(spheres, n_spheres, ex_mk(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]),
                            ex_mk(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]), &t, NULL);
        } else {
            id = li_nearest(spheres, n_spheres, li_mk(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]),
                            li_mk(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]), &t, NULL);
        }
        t_out[i] = id < 0 ? -1.0f : t;
        id_out[i] = id;
    }
}

void orc_cook_torrance(int mode, const float albedo[3], const float f0[3], float metallic, float roughness,
                       const float n[3], const float v[3], const float l[3], float out[3])
{
    if (mode == ORC_EXACT) {
        ex_v3 r = ex_cook_torrance(ex_ld(albedo), ex_ld(f0), metallic, roughness, ex_ld(n), ex_ld(v), ex_ld(l));
        out[0] = r.x; out[1] = r.y; out[2] = r.z;
    } else {
        li_v3 r = li_cook_torrance(li_ld(albedo), li_ld(f0), metallic, roughness, li_ld(n), li_ld(v), li_ld(l));
        out[0] = r.x; out[1] = r.y; out[2] = r.z;
    }
}

void orc_sample_cosine(int mode, const float n[3], uint32_t* seed, float out[3])
{
    if (mode == ORC_EXACT) {
        ex_v3 r = ex_sample_cosine(ex_ld(n), seed);
        out[0] = r.x; out[1] = r.y; out[2] = r.z;
    } else {
        li_v3 r = li_sample_cosine(li_ld(n), seed);
        out[0] = r.x; out[1] = r.y; out[2] = r.z;
    }
}

void orc_sample_ggx(int mode, const float n[3], float roughness, uint32_t* seed, float out[3])
{
    if (mode == ORC_EXACT) {
        ex_v3 r = ex_sample_ggx(ex_ld(n), roughness, seed);
        out[0] = r.x; out[1] = r.y; out[2] = r.z;
    } else {
        li_v3 r = li_sample_ggx(li_ld(n), roughness, seed);
        out[0] = r.x; out[1] = r.y; out[2] = r.z;
    }
}

/* ---------------------------------------------------------------- render */

static int check_args(const orc_scene* sc, const orc_view* v, const orc_job* j)
{
    if (!sc || !v || !j) return -1;
    if (v->width == 0 || v->height == 0) return -1;
    if (sc->n_spheres < 0 || sc->n_lights < 0 || sc->n_materials < 0) return -1;
    if (sc->n_spheres > 0 && sc->n_materials == 0) return -1;
    return 0;
}

static void stats_add(orc_stats* dst, const orc_stats* src)
{
    dst->ext_rays += src->ext_rays;
    dst->shadow_rays += src->shadow_rays;
    dst->shaded_hits += src->shaded_hits;
    dst->sphere_tests += src->sphere_tests;
}

int orc_render_f32(int mode, const orc_scene* sc, const orc_view* view, const orc_job* job,
                   float* accum, float* samples, orc_stats* stats)
{
    if (check_args(sc, view, job)) return -1;
    const uint64_t npx = job->pixels ? job->n_pixels : (uint64_t)view->width * view->height;
    orc_stats total;
    memset(&total, 0, sizeof(total));
#ifdef _OPENMP
    int nt = job->threads > 0 ? job->threads : omp_get_max_threads();
#endif
#pragma omp parallel num_threads(nt)
    {
        orc_stats st;
        memset(&st, 0, sizeof(st));
#pragma omp for schedule(dynamic, 16)
        for (int64_t k = 0; k < (int64_t)npx; ++k) {
            uint32_t p = job->pixels ? job->pixels[k] : (uint32_t)k;
            uint32_t x = p % view->width, y = p / view->width;
            float* acc = accum + 4 * k;
            for (uint32_t s = 0; s < job->spp; ++s) {
                uint32_t frame = job->frame0 + s;
                float c[3];
                if (mode == ORC_EXACT) {
                    ex_v3 r = ex_per_pixel(sc, view, x, y, frame, job->max_bounces, job->sky_light, &st, NULL);
                    c[0] = r.x; c[1] = r.y; c[2] = r.z;
                } else {
                    li_v3 r = li_per_pixel(sc, view, x, y, frame, job->max_bounces, job->sky_light, &st, NULL);
                    c[0] = r.x; c[1] = r.y; c[2] = r.z;
                }
                acc[0] += c[0]; acc[1] += c[1]; acc[2] += c[2]; acc[3] += 1.0f;
                if (samples) {
                    float* o = samples + 4 * ((uint64_t)k * job->spp + s);
                    o[0] = c[0]; o[1] = c[1]; o[2] = c[2]; o[3] = 1.0f;
                }
            }
        }
#pragma omp critical
        stats_add(&total, &st);
    }
    if (stats) *stats = total;
    return 0;
}

int orc_render_f64(const orc_scene* sc, const orc_view* view, const orc_job* job,
                   double* accum, double* samples, orc_stats* stats)
{
    if (check_args(sc, view, job)) return -1;
    const uint64_t npx = job->pixels ? job->n_pixels : (uint64_t)view->width * view->height;
    orc_stats total;
    memset(&total, 0, sizeof(total));
#ifdef _OPENMP
    int nt = job->threads > 0 ? job->threads : omp_get_max_threads();
#endif
#pragma omp parallel num_threads(nt)
    {
        orc_stats st;
        memset(&st, 0, sizeof(st));
#pragma omp for schedule(dynamic, 16)
        for (int64_t k = 0; k < (int64_t)npx; ++k) {
            uint32_t p = job->pixels ? job->pixels[k] : (uint32_t)k;
            uint32_t x = p % view->width, y = p / view->width;
            double* acc = accum + 4 * k;
            for (uint32_t s = 0; s < job->spp; ++s) {
                d_v3 r = d_per_pixel(sc, view, x, y, job->frame0 + s, job->max_bounces, job->sky_light, &st, NULL);
                acc[0] += r.x; acc[1] += r.y; acc[2] += r.z; acc[3] += 1.0;
                if (samples) {
                    double* o = samples + 4 * ((uint64_t)k * job->spp + s);
                    o[0] = r.x; o[1] = r.y; o[2] = r.z; o[3] = 1.0;
                }
            }
        }
#pragma omp critical
        stats_add(&total, &st);
    }
    if (stats) *stats = total;
    return 0;
}

/* ------------------------------------------------------ branch decisions */

static void decisions_of_path(int variant, const orc_scene* sc, const orc_view* view, uint32_t x, uint32_t y,
                              uint32_t frame, const orc_job* job, orc_stats* st, orc_sink* sk)
{
    if (variant == ORC_EXACT) (void)ex_per_pixel(sc, view, x, y, frame, job->max_bounces, job->sky_light, st, sk);
    else if (variant == ORC_LITERAL) (void)li_per_pixel(sc, view, x, y, frame, job->max_bounces, job->sky_light, st, sk);
    else (void)d_per_pixel(sc, view, x, y, frame, job->max_bounces, job->sky_light, st, sk);
}

int orc_decision_hash(int variant, const orc_scene* sc, const orc_view* view, const orc_job* job, uint64_t* hash)
{
    if (check_args(sc, view, job) || !hash || variant < ORC_EXACT || variant > ORC_F64) return -1;
    const uint64_t npx = job->pixels ? job->n_pixels : (uint64_t)view->width * view->height;
#ifdef _OPENMP
    int nt = job->threads > 0 ? job->threads : omp_get_max_threads();
#endif
#pragma omp parallel num_threads(nt)
    {
        orc_stats st;
        memset(&st, 0, sizeof(st));
#pragma omp for schedule(dynamic, 16)
        for (int64_t k = 0; k < (int64_t)npx; ++k) {
            uint32_t p = job->pixels ? job->pixels[k] : (uint32_t)k;
            orc_sink sk = { NULL, 0, 0, 0xcbf29ce484222325ull };
            for (uint32_t s = 0; s < job->spp; ++s)
                decisions_of_path(variant, sc, view, p % view->width, p / view->width, job->frame0 + s, job, &st, &sk);
            hash[k] = sk.hash;
        }
    }
    return 0;
}

int orc_decision_events(int variant, const orc_scene* sc, const orc_view* view, const orc_job* job, uint32_t* ev,
                        int32_t cap)
{
    if (check_args(sc, view, job) || !ev || cap <= 0 || variant < ORC_EXACT || variant > ORC_F64) return -1;
    const uint64_t npx = job->pixels ? job->n_pixels : (uint64_t)view->width * view->height;
#ifdef _OPENMP
    int nt = job->threads > 0 ? job->threads : omp_get_max_threads();
#endif
#pragma omp parallel num_threads(nt)
    {
        orc_stats st;
        memset(&st, 0, sizeof(st));
#pragma omp for schedule(dynamic, 16)
        for (int64_t k = 0; k < (int64_t)npx; ++k) {
            uint32_t p = job->pixels ? job->pixels[k] : (uint32_t)k;
            for (uint32_t s = 0; s < job->spp; ++s) {
                uint32_t* row = ev + ((uint64_t)k * job->spp + s) * (uint64_t)cap;
                memset(row, 0, sizeof(uint32_t) * (size_t)cap);
                orc_sink sk = { row, cap, 0, 0 };
                decisions_of_path(variant, sc, view, p % view->width, p / view->width, job->frame0 + s, job, &st, &sk);
            }
        }
    }
    return 0;
}

/* Renderer.cu:166-168: accum / frameIndex, clamped to [0, 1], then
 * colorUtils::vec4ToRGBA (Renderer.h:70-78): truncating x * 255 per channel
 * packed as A<<24 | B<<16 | G<<8 | R.  A NaN channel packs as 0. */
void orc_pack_rgba8(const float* accum, uint64_t n, uint32_t frame, uint32_t* out)
{
    const float f = (float)frame;
    for (uint64_t i = 0; i < n; ++i) {
        uint32_t ch[4];
        for (int c = 0; c < 4; ++c) {
            float v = accum[4 * i + c] / f;
            v = v < 0.0f ? 0.0f : v;
            v = v > 1.0f ? 1.0f : v;
            float s = v * 255.0f;
            ch[c] = (s == s) ? (uint32_t)s : 0u;
        }
        out[i] = (ch[3] << 24) | (ch[2] << 16) | (ch[1] << 8) | ch[0];
    }
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
