/*
 * Oracle for the Ataraxia per-pixel path tracer: a plain-C CPU restatement.
 *
 * TEST INFRASTRUCTURE ONLY.  The product (ataraxia_gb300/, include/atx.h)
 * never links, loads or calls anything in this directory; only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg (and its
 * `--impl reference` arm) do, and there only as the checker / the timed CPU
 * restatement of the reference.
 *
 * Parity pinned to the reference's own code: the reference ships no tests,
 * golden images or known-answer vectors, but its render path compiles from its
 * unmodified sources against the project's minimal glm and headless Image and
 * Input headers (baseline/refbuild).  The literal mode below agrees with the
 * reference's kernel built in IEEE arithmetic on at least 99.99% of pixels
 * (within 1e-3; the rest is libm vs CUDA last bits in sinf, cosf, powf); the
 * camera and scene-graph code equals the reference's host code bit for bit.
 * It is further checked against closed-form identities, an independent
 * pure-Python restatement on small images and committed fixtures
 * (tests/golden/).
 *
 * What is restated (reference paths are relative to the Ataraxia tree):
 *   Core/include/Random.h:59-70       PcgHash / PcgFloat
 *   Engine/src/Camera.cpp:134-159     perspective / lookAt / inverse matrices
 *   Engine/src/Camera.cpp:161-195     per-pixel primary ray directions
 *   Engine/src/Renderer.cu:251-285    traceRay (brute-force nearest hit)
 *   Engine/src/Renderer.cu:287-387    perPixel (the bounce loop / estimator)
 *   Engine/src/Renderer.cu:389-409    rayMiss / rayHit
 *   Engine/src/Renderer.cu:162-168    accumulate + clamp + RGBA8 pack
 *   Engine/include/Renderer.h:70-78   colorUtils::vec4ToRGBA
 *   Engine/src/BRDF.cu:9-117          Cook-Torrance, GGX, Smith, samplers
 *
 * Three arithmetic modes share one body (oracle_impl.h):
 *   ORC_EXACT    FP32 in the evaluation order the CUDA kernels use: vector dot
 *                products as fused multiply-add chains, the ray-sphere
 *                quadratic in its half-b form with fused terms, x^5 as three
 *                products, sin/cos(2*pi*u) from a Taylor polynomial after
 *                exact quarter-turn reduction, a vector over a scalar as a
 *                product with the scalar's reciprocal (tangent frame, the
 *                roulette's throughput), / pi as * (1 / pi) and the specular
 *                F * D * G / denom with one quotient for D * G / denom.
 *                Every other expression is the
 *                reference's, evaluated with IEEE single rounding and no
 *                contraction.  The kernels must equal this mode bit for bit.
 *   ORC_LITERAL  FP32 following the reference's expressions as written
 *                (b = 2*dot, disc = b*b - 4*a*c, libm sinf/cosf/powf), no
 *                contraction.  Differences to the kernels are rounding-level
 *                and are what "branch flips" are counted against.
 *   f64          the ORC_LITERAL expressions in double precision with the same
 *                integer random stream; used for converged-image checks.
 */
#ifndef ATX_ORACLE_H
#define ATX_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same memory layout as the reference's POD types (and include/atx.h). */
typedef struct { float center[3]; float radius; int32_t material; } orc_sphere;      /* SceneNode.h:11-21, 20 B */
typedef struct {
    float albedo[3]; float roughness; float metallic; float f0[3];
    float emission_color[3]; float emission_intensity; int32_t id;
} orc_material;                                                                       /* Scene.h:28-47, 52 B */
typedef struct { float position[3]; float color[3]; float intensity; } orc_light;     /* Scene.h:17-26, 28 B */

typedef struct {
    const orc_sphere* spheres; int32_t n_spheres;
    const orc_material* materials; int32_t n_materials;
    const orc_light* lights; int32_t n_lights;
} orc_scene;

/* Column-major 4x4 matrices, m[col*4 + row], as glm stores them. */
typedef struct {
    float inv_view[16]; float inv_proj[16]; float position[3];
    uint32_t width, height;
} orc_view;

typedef struct {
    int32_t max_bounces;      /* Settings::maxBounces */
    int32_t sky_light;        /* Settings::skyLight */
    uint32_t frame0;          /* frame index of the first sample (reference starts at 1) */
    uint32_t spp;             /* consecutive frames frame0 .. frame0+spp-1 */
    const uint32_t* pixels;   /* pixel indices x + y*W to render, or NULL for all, in order */
    uint64_t n_pixels;        /* ignored when pixels == NULL */
    int32_t threads;          /* OpenMP threads, <= 0 for the runtime default */
} orc_job;

typedef struct {
    uint64_t ext_rays;      /* extension rays traced (nearest hit) */
    uint64_t shadow_rays;   /* shadow rays traced */
    uint64_t shaded_hits;   /* bounces that reached the shading code */
    uint64_t sphere_tests;  /* ray-sphere tests, brute force */
} orc_stats;

enum { ORC_EXACT = 0, ORC_LITERAL = 1 };

/* Renders job->spp frames for the selected pixels.  accum (n_pixels x 4) is
 * read and each frame's (r, g, b, 1) is added to it in frame order, exactly as
 * Renderer.cu:165 does once per frame.  samples, when not NULL, receives each
 * frame's (r, g, b, 1) at [pixel][frame].  Returns 0, or -1 on bad arguments. */
int orc_render_f32(int mode, const orc_scene* scene, const orc_view* view, const orc_job* job,
                   float* accum, float* samples, orc_stats* stats);
int orc_render_f64(const orc_scene* scene, const orc_view* view, const orc_job* job,
                   double* accum, double* samples, orc_stats* stats);

/* Brute-force nearest hit (Renderer.cu:251-285) for n rays; t = -1, id = -1 on a miss. */
void orc_trace(int mode, const orc_sphere* spheres, int32_t n_spheres, const float* origins,
               const float* dirs, uint64_t n_rays, float* t_out, int32_t* id_out);

/* Camera.cpp:134-159 for a W x H viewport. */
void orc_camera_matrices(const float pos[3], const float dir[3], float fov_deg, float near_clip,
                         float far_clip, uint32_t width, uint32_t height,
                         float view[16], float inv_view[16], float proj[16], float inv_proj[16]);
void orc_mat4_inverse(const float m[16], float out[16]);

/* Camera::onUpdate (Camera.cpp:31-108); keys = W, S, A, D, Q, E held.  Updates
 * pos, dir and last_mouse; returns 1 when the camera moved. */
int orc_camera_on_update(float pos[3], float dir[3], float last_mouse[2], const float mouse[2], int right_button,
                         const int keys[6], float dt);

/* Camera.cpp:161-195: W*H*3 floats, pixel x + y*W. */
void orc_ray_dirs(int mode, const orc_view* view, float* out);

uint32_t orc_pcg_hash(uint32_t seed);
float orc_pcg_float(uint32_t* seed);
void orc_sincos2pi(float u, float* c, float* s);

void orc_cook_torrance(int mode, const float albedo[3], const float f0[3], float metallic, float roughness,
                       const float n[3], const float v[3], const float l[3], float out[3]);
void orc_sample_cosine(int mode, const float n[3], uint32_t* seed, float out[3]);
void orc_sample_ggx(int mode, const float n[3], float roughness, uint32_t* seed, float out[3]);

/* Branch decisions, for counting and classifying branch flips between
 * arithmetic modes.  variant: ORC_EXACT, ORC_LITERAL or ORC_F64 (the literal
 * expressions in double precision).  Each decision of a path is one event,
 * kind << 28 | bounce << 20 | value:
 *   ORC_EV_HIT       value = nearest sphere + 1, 0 on a miss (Renderer.cu:308-318)
 *   ORC_EV_SHADOW    value bits 0-1: 1 the light is visible, 2 occluded
 *                    (Renderer.cu:351-355); bits 2-19: the shadow ray's nearest
 *                    sphere + 1, recorded but not part of the decision
 *   ORC_EV_ROULETTE  value 1 when the path stops (Renderer.cu:375-377)
 *   ORC_EV_FRAME     value 1 when |N.x| > |N.y| picks the samplers' first
 *                    tangent (BRDF.cu:85, :109)
 * orc_decision_hash: per pixel (job->pixels or all), an FNV-1a hash of the
 * decisions of its frames frame0 .. frame0+spp-1.  orc_decision_events: per
 * pixel and frame, the first cap events (unused slots 0).  Both return 0, or
 * -1 on bad arguments. */
enum { ORC_F64 = 2 };
enum { ORC_EV_HIT = 1, ORC_EV_SHADOW = 2, ORC_EV_ROULETTE = 3, ORC_EV_FRAME = 4 };
int orc_decision_hash(int variant, const orc_scene* scene, const orc_view* view, const orc_job* job, uint64_t* hash);
int orc_decision_events(int variant, const orc_scene* scene, const orc_view* view, const orc_job* job,
                        uint32_t* events, int32_t cap);

/* Renderer.cu:166-168 + Renderer.h:70-78 */
void orc_pack_rgba8(const float* accum, uint64_t n, uint32_t frame, uint32_t* out);

int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
