/*
 * Body of the oracle, included once per arithmetic mode by oracle.c (test
 * infrastructure only; see oracle.h for what it restates and why parity is
 * unpinned).
 *
 * Expected macros:
 *   REAL     float or double
 *   FN(x)    mode-prefixed name
 *   EXACT    1: the kernels' evaluation order (fused dot chains, half-b
 *               quadratic, polynomial sincos, x^5 by products, reciprocal
 *               products for a vector over a scalar and for / pi, one
 *               quotient for the specular D * G / denom)
 *            0: the reference's expressions as written
 *   F64      1 in the double-precision build
 * The file is compiled with -ffp-contract=off, so every a*b+c below rounds
 * twice unless it is spelled fmaf().
 */

typedef struct { REAL x, y, z; } FN(v3);
#define V3 FN(v3)

static inline V3 FN(mk)(REAL x, REAL y, REAL z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline V3 FN(add)(V3 a, V3 b) { return FN(mk)(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 FN(sub)(V3 a, V3 b) { return FN(mk)(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 FN(mul)(V3 a, V3 b) { return FN(mk)(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline V3 FN(muls)(V3 a, REAL s) { return FN(mk)(a.x * s, a.y * s, a.z * s); }
static inline V3 FN(divs)(V3 a, REAL s) { return FN(mk)(a.x / s, a.y / s, a.z / s); }
/* a / s where the kernels multiply by the reciprocal (the tangent frame, the
 * roulette's throughput); the reference's a / s otherwise. */
static inline V3 FN(div_v)(V3 a, REAL s)
{
#if EXACT
    return FN(muls)(a, (REAL)1 / s);
#else
    return FN(divs)(a, s);
#endif
}
static inline V3 FN(neg)(V3 a) { return FN(mk)(-a.x, -a.y, -a.z); }
static inline V3 FN(ld)(const float* p) { return FN(mk)((REAL)p[0], (REAL)p[1], (REAL)p[2]); }

#if F64
#define SQRT sqrt
#define FABS fabs
#define PI_R 3.14159265358979323846
#define TWO_PI_R 6.28318530717958647692
#else
#define SQRT sqrtf
#define FABS fabsf
#define PI_R 0x1.921fb6p+1f      /* glm::pi<float>() */
#define TWO_PI_R 0x1.921fb6p+2f  /* 2.0f * glm::pi<float>(), folded exactly */
#endif

/* glm::dot for vec3 sums (x + y) + z. */
static inline REAL FN(dot)(V3 a, V3 b)
{
#if EXACT
    return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x));
#else
    return (a.x * b.x + a.y * b.y) + a.z * b.z;
#endif
}

/* glm::normalize(v) = v * inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x). */
static inline V3 FN(normalize)(V3 v) { REAL inv = (REAL)1 / SQRT(FN(dot)(v, v)); return FN(muls)(v, inv); }
static inline REAL FN(length)(V3 v) { return SQRT(FN(dot)(v, v)); }
static inline V3 FN(cross)(V3 a, V3 b)
{
    return FN(mk)(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
/* glm::max / glm::min on scalars: (a < b) ? b : a and (b < a) ? b : a. */
static inline REAL FN(maxr)(REAL a, REAL b) { return (a < b) ? b : a; }
static inline REAL FN(minr)(REAL a, REAL b) { return (b < a) ? b : a; }

/* Random.h:66-70.  float(UINT32_MAX) rounds to 2^32, so the division is an
 * exact scaling; the f64 build widens the same float. */
static inline REAL FN(pcg_float)(uint32_t* seed)
{
    *seed = orc_pcg_hash(*seed);
    return (REAL)((float)(*seed) / 4294967296.0f);
}

static inline void FN(sincos_2pi)(REAL u, REAL* c, REAL* s)
{
#if EXACT
    orc_sincos2pi(u, c, s);
#elif F64
    REAL th = TWO_PI_R * u;
    *c = cos(th); *s = sin(th);
#else
    REAL th = TWO_PI_R * u;   /* theta = 2.0f * pi * u (BRDF.cu:78, :104) */
    *c = cosf(th); *s = sinf(th);
#endif
}

static inline REAL FN(pow5)(REAL x)
{
#if EXACT
    REAL x2 = x * x;
    REAL x4 = x2 * x2;
    return x4 * x;
#elif F64
    return pow(x, 5.0);
#else
    return powf(x, 5.0f);
#endif
}

/* ------------------------------------------------------------------ camera */

/* Camera.cpp:161-195 for one pixel.  The reference computes the directions on
 * the host with IEEE single rounding and no contraction, so every mode
 * evaluates its expressions in that order: pairwise column sums for the
 * matrix-vector products and unfused dot products (x*x + y*y) + z*z in the two
 * normalisations (the kernels do the same). */
static inline V3 FN(normalize_host)(V3 v)
{
    REAL d = (v.x * v.x + v.y * v.y) + v.z * v.z;
    return FN(muls)(v, (REAL)1 / SQRT(d));
}

static V3 FN(primary_dir)(const orc_view* v, uint32_t x, uint32_t y)
{
    const float* P = v->inv_proj;
    const float* Vw = v->inv_view;
    REAL qx = (REAL)(float)x / (REAL)(float)v->width;
    REAL qy = (REAL)(float)y / (REAL)(float)v->height;
    REAL cx = qx * (REAL)2 - (REAL)1;
    REAL cy = qy * (REAL)2 - (REAL)1;
    REAL t[4];
    for (int r = 0; r < 4; ++r)
        t[r] = ((REAL)P[0 * 4 + r] * cx + (REAL)P[1 * 4 + r] * cy) +
               ((REAL)P[2 * 4 + r] * (REAL)1 + (REAL)P[3 * 4 + r] * (REAL)1);
    V3 tv = FN(normalize_host)(FN(mk)(t[0] / t[3], t[1] / t[3], t[2] / t[3]));
    REAL d[3];
    for (int r = 0; r < 3; ++r)
        d[r] = ((REAL)Vw[0 * 4 + r] * tv.x + (REAL)Vw[1 * 4 + r] * tv.y) +
               ((REAL)Vw[2 * 4 + r] * tv.z + (REAL)Vw[3 * 4 + r] * (REAL)0);
    return FN(normalize_host)(FN(mk)(d[0], d[1], d[2]));
}

/* ---------------------------------------------------------- intersection */

typedef struct { REAL t; V3 pos; V3 normal; int32_t id; } FN(hit);

/* Renderer.cu:251-285: nearest hit over all spheres, strict '<' so the lowest
 * index wins ties, only t > 0 accepted (an origin inside a sphere never hits
 * it).  Returns the sphere index or -1; *t_out is tmin. */
static int32_t FN(nearest)(const orc_sphere* sp, int32_t n, V3 o, V3 d, REAL* t_out, uint64_t* tests)
{
    int32_t best = -1;
#if F64
    REAL tmin = (REAL)FLT_MAX;
#else
    REAL tmin = FLT_MAX;
#endif
    const REAL a = FN(dot)(d, d);
    for (int32_t i = 0; i < n; ++i) {
        V3 c = FN(ld)(sp[i].center);
        REAL r = (REAL)sp[i].radius;
        V3 oc = FN(sub)(o, c);
#if EXACT
        /* half-b form: b' = dot(oc, d), disc' = b'^2 - a c, t = (-b' - sqrt(disc')) / a,
         * the reference's quadratic divided through by 2 */
        REAL b = fmaf(oc.z, d.z, fmaf(oc.y, d.y, oc.x * d.x));
        REAL cc = fmaf(oc.z, oc.z, fmaf(oc.y, oc.y, fmaf(oc.x, oc.x, -(r * r))));
        REAL disc = fmaf(b, b, -(a * cc));
        if (disc < 0.0f) continue;
        REAL t = -(b + sqrtf(disc)) / a;
#else
        REAL b = (REAL)2 * FN(dot)(oc, d);
        REAL cc = FN(dot)(oc, oc) - r * r;
        REAL disc = b * b - (REAL)4 * a * cc;
        if (disc < (REAL)0) continue;
        REAL t0 = (-b - SQRT(disc)) / ((REAL)2 * a);
        REAL t1 = (-b + SQRT(disc)) / ((REAL)2 * a);
        REAL t = t0 < t1 ? t0 : t1;
#endif
        if (t > (REAL)0 && t < tmin) { tmin = t; best = i; }
    }
    if (tests) *tests += (uint64_t)n;
    *t_out = tmin;
    return best;
}

/* Renderer.cu:396-409 */
static FN(hit) FN(ray_hit)(const orc_sphere* sp, V3 o, V3 d, REAL t, int32_t idx)
{
    FN(hit) h;
    V3 c = FN(ld)(sp[idx].center);
    V3 oc = FN(sub)(o, c);
    h.t = t;
    h.id = idx;
    h.pos = FN(add)(oc, FN(muls)(d, t));
    h.normal = FN(normalize)(h.pos);
    h.pos = FN(add)(h.pos, c);
    return h;
}

/* ------------------------------------------------------------------- BRDF */

/* BRDF.cu:36-40 */
static inline V3 FN(fresnel)(V3 f0, REAL cos_theta)
{
    cos_theta = FN(minr)(FN(maxr)(cos_theta, (REAL)0), (REAL)1);
    REAL p = FN(pow5)((REAL)1 - cos_theta);
    return FN(mk)(f0.x + ((REAL)1 - f0.x) * p, f0.y + ((REAL)1 - f0.y) * p, f0.z + ((REAL)1 - f0.z) * p);
}

/* BRDF.cu:42-53 */
static inline REAL FN(ggx_d)(REAL ndoth, REAL rough)
{
    const REAL a = rough * rough;
    const REAL a2 = a * a;
    REAL n2 = ndoth * ndoth;
    REAL den = n2 * (a2 - (REAL)1) + (REAL)1;
    den = PI_R * den * den;
    return a2 / den;
}

/* BRDF.cu:55-63 */
static inline REAL FN(schlick_g)(REAL ndotv, REAL rough)
{
    const REAL r = rough + (REAL)1;
    const REAL k = (r * r) / (REAL)8;
    return ndotv / (ndotv * ((REAL)1 - k) + k);
}

/* BRDF.cu:9-34 */
static V3 FN(cook_torrance)(V3 albedo, V3 f0, REAL metallic, REAL rough, V3 n, V3 v, V3 l)
{
    V3 h = FN(normalize)(FN(add)(v, l));
    REAL ndotl = FN(maxr)(FN(dot)(n, l), (REAL)1e-7f);
    REAL ndotv = FN(maxr)(FN(dot)(n, v), (REAL)1e-7f);
    REAL ndoth = FN(maxr)(FN(dot)(n, h), (REAL)0);
    REAL vdoth = FN(maxr)(FN(dot)(v, h), (REAL)0);

    V3 F = FN(fresnel)(f0, vdoth);
    V3 kd = FN(muls)(FN(sub)(FN(mk)(1, 1, 1), F), (REAL)1 - metallic);
    REAL denom = (REAL)4 * ndotl * ndotv + (REAL)0.001f;
#if EXACT
    /* The kernels' grouping: F * (D * G) / denom as F * X, X = (a2 * ndotv *
     * ndotl) / (den * g_v * g_l * denom), one division; / pi as * (1 / pi). */
    const REAL a = rough * rough;
    const REAL a2 = a * a;
    REAL den = (ndoth * ndoth) * (a2 - (REAL)1) + (REAL)1;
    den = PI_R * den * den;
    const REAL r = rough + (REAL)1;
    const REAL k = (r * r) * (REAL)0.125f;
    const REAL gv = ndotv * ((REAL)1 - k) + k;
    const REAL gl = ndotl * ((REAL)1 - k) + k;
    const REAL X = ((a2 * ndotv) * ndotl) / (((den * gv) * gl) * denom);
    V3 spec = FN(muls)(F, X);
    V3 diffuse = FN(muls)(FN(mul)(FN(sub)(FN(mk)(1, 1, 1), F), albedo), (REAL)1 / PI_R);
#else
    REAL D = FN(ggx_d)(ndoth, rough);
    REAL G = FN(schlick_g)(ndotv, rough) * FN(schlick_g)(ndotl, rough);
    V3 num = FN(muls)(F, D * G);
    V3 spec = FN(divs)(num, denom);
    V3 diffuse = FN(divs)(FN(mul)(FN(sub)(FN(mk)(1, 1, 1), F), albedo), PI_R);
#endif
    return FN(muls)(FN(add)(FN(mul)(kd, diffuse), spec), ndotl);
}

/* Tangent frame used by both samplers (BRDF.cu:84-90, :108-114). */
static inline void FN(frame)(V3 n, V3* t, V3* b)
{
    if (FABS(n.x) > FABS(n.y))
        *t = FN(div_v)(FN(mk)(-n.z, 0, n.x), SQRT(n.x * n.x + n.z * n.z));
    else
        *t = FN(div_v)(FN(mk)(0, -n.z, n.y), SQRT(n.y * n.y + n.z * n.z));
    *b = FN(cross)(n, *t);
}

/* x*T + y*B + z*N summed left to right (BRDF.cu:92, :116). */
static inline V3 FN(to_world)(REAL x, REAL y, REAL z, V3 t, V3 b, V3 n)
{
    return FN(add)(FN(add)(FN(muls)(t, x), FN(muls)(b, y)), FN(muls)(n, z));
}

/* BRDF.cu:72-93 */
static V3 FN(sample_cosine)(V3 n, uint32_t* seed)
{
    const REAL u1 = FN(pcg_float)(seed);
    const REAL u2 = FN(pcg_float)(seed);
    const REAL r = SQRT(u1);
    REAL c, s;
    FN(sincos_2pi)(u2, &c, &s);
    const REAL x = r * c;
    const REAL y = r * s;
    const REAL z = SQRT((REAL)1 - u1);
    V3 t, b;
    FN(frame)(n, &t, &b);
    return FN(to_world)(x, y, z, t, b, n);
}

/* BRDF.cu:95-117: returns the sampled half vector itself as the new direction. */
static V3 FN(sample_ggx)(V3 n, REAL rough, uint32_t* seed)
{
    const REAL u1 = FN(pcg_float)(seed);
    const REAL u2 = FN(pcg_float)(seed);
    const REAL a = rough * rough;
    const REAL cos_t = SQRT(((REAL)1 - u1) / ((REAL)1 + (a * a - (REAL)1) * u1));
    const REAL sin_t = SQRT((REAL)1 - cos_t * cos_t);
    REAL c, s;
    FN(sincos_2pi)(u2, &c, &s);
    V3 t, b;
    FN(frame)(n, &t, &b);
    return FN(to_world)(sin_t * c, sin_t * s, cos_t, t, b, n);
}

/* ---------------------------------------------------------------- perPixel */

/* Renderer.cu:287-387.  Returns the path colour; alpha is always 1. */
static V3 FN(per_pixel)(const orc_scene* sc, const orc_view* view, uint32_t x, uint32_t y, uint32_t frame,
                        int32_t max_bounces, int32_t sky, orc_stats* st, orc_sink* sk)
{
    V3 o = FN(ld)(view->position);
    V3 d = FN(primary_dir)(view, x, y);
    V3 color = FN(mk)(0, 0, 0);
    V3 thr = FN(mk)(1, 1, 1);
    uint32_t seed = x + y * view->width;
    seed *= frame;

    for (int32_t i = 0; i < max_bounces; ++i) {
        seed += (uint32_t)i;
        REAL tmin;
        st->ext_rays++;
        int32_t idx = FN(nearest)(sc->spheres, sc->n_spheres, o, d, &tmin, &st->sphere_tests);
        orc_emit(sk, ORC_EV_HIT, i, (uint32_t)(idx + 1));
        if (idx < 0) {
            if (sky) color = FN(add)(color, FN(mul)(FN(mk)((REAL)0.6f, (REAL)0.7f, (REAL)0.9f), thr));
            break;
        }
        FN(hit) h = FN(ray_hit)(sc->spheres, o, d, tmin, idx);
        st->shaded_hits++;
        int32_t mid = sc->spheres[idx].material;
        if ((uint32_t)mid >= (uint32_t)sc->n_materials) mid = 0; /* host clamp, Renderer.cu:30-37 */
        const orc_material* m = &sc->materials[mid];
        V3 albedo = FN(ld)(m->albedo);

        if (m->emission_intensity > 0.0f) {
            V3 e = FN(muls)(FN(ld)(m->emission_color), (REAL)m->emission_intensity);
            color = FN(add)(color, FN(mul)(e, thr));
        }

        const REAL metallic = (REAL)m->metallic;
        /* glm::mix(F0, albedo, metallic) = F0 * (1 - m) + albedo * m */
        V3 base = FN(add)(FN(muls)(FN(ld)(m->f0), (REAL)1 - metallic), FN(muls)(albedo, metallic));

        if (sc->n_lights > 0) {
            uint32_t li = orc_pcg_hash(seed) % (uint32_t)sc->n_lights;
            const orc_light* lt = &sc->lights[li];
            V3 L = FN(sub)(FN(ld)(lt->position), h.pos);
            REAL dist2 = FN(dot)(L, L);
            L = FN(normalize)(L);
            V3 so = FN(add)(h.pos, FN(muls)(h.normal, (REAL)0.0001f));
            REAL ts;
            st->shadow_rays++;
            int32_t sidx = FN(nearest)(sc->spheres, sc->n_spheres, so, L, &ts, &st->sphere_tests);
            REAL tsh = sidx < 0 ? (REAL)-1 : ts;
            const int occluded = tsh > (REAL)0 && tsh * tsh < dist2;
            orc_emit(sk, ORC_EV_SHADOW, i, (occluded ? 2u : 1u) | ((uint32_t)(sidx + 1) << 2));
            if (occluded) {
                /* occluded */
            } else {
                V3 f = FN(cook_torrance)(albedo, base, metallic, (REAL)m->roughness, h.normal, FN(neg)(d), L);
                V3 le = FN(muls)(FN(ld)(lt->color), (REAL)lt->intensity);
                V3 contrib = FN(divs)(FN(mul)(FN(mul)(le, f), thr), (REAL)1);
                color = FN(add)(color, contrib);
            }
        }

        thr = FN(mul)(thr, albedo);
        o = FN(add)(h.pos, FN(muls)(h.normal, (REAL)0.0001f));

        REAL p = FN(maxr)((REAL)0.1f, FN(minr)((REAL)1, FN(length)(thr)));
        const int stop = FN(pcg_float)(&seed) > p;
        orc_emit(sk, ORC_EV_ROULETTE, i, (uint32_t)stop);
        if (stop) break;
        thr = FN(div_v)(thr, p);
        orc_emit(sk, ORC_EV_FRAME, i, (uint32_t)(FABS(h.normal.x) > FABS(h.normal.y)));

        if (m->metallic > 0.0f)
            d = FN(sample_ggx)(h.normal, (REAL)m->roughness, &seed);
        else
            d = FN(sample_cosine)(h.normal, &seed);
    }
    return color;
}

#undef V3
#undef SQRT
#undef FABS
#undef PI_R
#undef TWO_PI_R
