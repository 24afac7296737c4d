/*
 * raymarch_body.h -- CPU oracle (test infrastructure only): the raymarch of
 * share/shaders/volumes/volume.frag:31-103 and its includes, written once and
 * instantiated by raymarch.c for REAL = double (parity oracle) and
 * REAL = float (CPU baseline).  The loop variables `t` are FP32 in both, as
 * in the GLSL, so both instantiations run the same iteration counts.
 *
 * Expects: REAL, SFX(name) (suffixing macro), SQRT_FN, POW_FN, FLOOR_FN.
 */

typedef struct SFX(vec3) { REAL x, y, z; } SFX(vec3);

static inline SFX(vec3) SFX(v3)(REAL x, REAL y, REAL z) { SFX(vec3) r = {x, y, z}; return r; }
static inline SFX(vec3) SFX(add)(SFX(vec3) a, SFX(vec3) b) { return SFX(v3)(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline SFX(vec3) SFX(sub)(SFX(vec3) a, SFX(vec3) b) { return SFX(v3)(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline SFX(vec3) SFX(scale)(SFX(vec3) a, REAL s) { return SFX(v3)(a.x * s, a.y * s, a.z * s); }
static inline SFX(vec3) SFX(mul)(SFX(vec3) a, SFX(vec3) b) { return SFX(v3)(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline REAL SFX(dot)(SFX(vec3) a, SFX(vec3) b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline SFX(vec3) SFX(from)(const float* f) { return SFX(v3)((REAL)f[0], (REAL)f[1], (REAL)f[2]); }

/* GLSL normalize(v) = v / length(v); a zero vector gives NaN components, as
 * 0/0 does on the GPU, and the output clamp below turns them into 0. */
static inline SFX(vec3) SFX(normalize)(SFX(vec3) a, REAL* len_out)
{
    REAL l = SQRT_FN(SFX(dot)(a, a));
    if (len_out) *len_out = l;
    return SFX(v3)(a.x / l, a.y / l, a.z / l);
}

/* GLSL mix(x, y, a) = x * (1 - a) + y * a. */
static inline SFX(vec3) SFX(mix)(SFX(vec3) a, SFX(vec3) b, REAL t)
{
    return SFX(add)(SFX(scale)(a, (REAL)1 - t), SFX(scale)(b, t));
}

typedef struct SFX(vol) {
    const void* data;
    int fmt;       /* vkhr_density_format or vkhr_tangent_format */
    int n[3];
    SFX(vec3) origin, size;
} SFX(vol);

static inline REAL SFX(texel_density)(const SFX(vol)* v, long i, long j, long k)
{
    if (i < 0 || j < 0 || k < 0 || i >= v->n[0] || j >= v->n[1] || k >= v->n[2]) return 0; /* border */
    size_t at = (size_t)i + (size_t)v->n[0] * ((size_t)j + (size_t)v->n[1] * (size_t)k);
    switch (v->fmt) {
    case VKHR_DENSITY_U8_UNORM: return (REAL)((const uint8_t*)v->data)[at] / (REAL)255; /* UNORM: c/255 */
    case VKHR_DENSITY_U32_COUNT: return (REAL)((const uint32_t*)v->data)[at];
    case ORACLE_F64: return (REAL)((const double*)v->data)[at];
    default: return (REAL)((const float*)v->data)[at];
    }
}

static inline SFX(vec3) SFX(texel_tangent)(const SFX(vol)* v, long i, long j, long k)
{
    if (i < 0 || j < 0 || k < 0 || i >= v->n[0] || j >= v->n[1] || k >= v->n[2]) return SFX(v3)(0, 0, 0);
    size_t at = (size_t)i + (size_t)v->n[0] * ((size_t)j + (size_t)v->n[1] * (size_t)k);
    if (v->fmt == VKHR_TANGENT_I8_SNORM) {
        const int8_t* q = (const int8_t*)v->data + 4 * at;
        REAL c[3];
        for (int a = 0; a < 3; ++a) { /* SNORM: max(c/127, -1) */
            c[a] = (REAL)q[a] / (REAL)127;
            if (c[a] < (REAL)-1) c[a] = (REAL)-1;
        }
        return SFX(v3)(c[0], c[1], c[2]);
    }
    if (v->fmt == ORACLE_F64) {
        const double* g = (const double*)v->data + 4 * at;
        return SFX(v3)((REAL)g[0], (REAL)g[1], (REAL)g[2]);
    }
    const float* f = (const float*)v->data + 4 * at;
    return SFX(v3)((REAL)f[0], (REAL)f[1], (REAL)f[2]);
}

/* Texel-space coordinate set-up of a LINEAR, CLAMP_TO_BORDER lookup (Vulkan
 * spec "Texel Coordinate Systems": u = s*size - 0.5, i0 = floor(u), alpha =
 * frac(u)).  Returns 0 when all eight taps are border texels. */
static inline int SFX(tex_setup)(const SFX(vol)* v, SFX(vec3) P, long i0[3], REAL a[3])
{
    /* sample_volume.glsl:8 -- (fragment_position - volume_origin) / volume_size */
    SFX(vec3) uvw = SFX(v3)((P.x - v->origin.x) / v->size.x, (P.y - v->origin.y) / v->size.y,
                            (P.z - v->origin.z) / v->size.z);
    REAL s[3] = {uvw.x, uvw.y, uvw.z};
    for (int c = 0; c < 3; ++c) {
        REAL u = s[c] * (REAL)v->n[c] - (REAL)0.5;
        if (!(u > (REAL)-2 && u < (REAL)(v->n[c] + 1))) return 0;
        REAL f = FLOOR_FN(u);
        i0[c] = (long)f;
        a[c] = u - f;
    }
    return 1;
}

/* Distance, in texels, from sample P to the boundary where the shader's
 * `density != 0.0` test flips.  A texel j carries nonzero trilinear weight
 * iff max_k |j_k - u_k| < 1 (u = texel-space position).  For a nonzero
 * sample the margin is the largest, over its nonzero taps, of min_k(1 - |j_k - u_k|);
 * for a zero sample it is the smallest, over nonzero texels of the 4^3
 * neighbourhood, of max_k |j_k - u_k| - 1 (capped at 1).  Test-side only. */
static double SFX(support_margin)(const SFX(vol)* v, SFX(vec3) P)
{
    long i0[3];
    REAL a[3];
    if (!SFX(tex_setup)(v, P, i0, a)) return 1.0;
    double best_nz = -1.0;
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                if (SFX(texel_density)(v, i0[0] + dx, i0[1] + dy, i0[2] + dz) == (REAL)0) continue;
                double wx = dx ? (double)a[0] : 1.0 - (double)a[0];
                double wy = dy ? (double)a[1] : 1.0 - (double)a[1];
                double wz = dz ? (double)a[2] : 1.0 - (double)a[2];
                double m = wx < wy ? wx : wy;
                m = m < wz ? m : wz;
                if (m > best_nz) best_nz = m;
            }
    if (best_nz >= 0.0) return best_nz; /* weight 0 on every nonzero tap still counts as zero */
    double best = 1.0;
    for (int ez = -1; ez <= 2; ++ez)
        for (int ey = -1; ey <= 2; ++ey)
            for (int ex = -1; ex <= 2; ++ex) {
                const int e[3] = {ex, ey, ez};
                double dmax = 0.0;
                for (int k = 0; k < 3; ++k) {
                    double d = e[k] == -1 ? 1.0 + (double)a[k]
                             : e[k] == 0 ? (double)a[k]
                             : e[k] == 1 ? 1.0 - (double)a[k] : 2.0 - (double)a[k];
                    if (d > dmax) dmax = d;
                }
                if (dmax - 1.0 >= best) continue;
                if (SFX(texel_density)(v, i0[0] + ex, i0[1] + ey, i0[2] + ez) != (REAL)0) best = dmax - 1.0;
            }
    return best;
}

static REAL SFX(sample_density)(const SFX(vol)* v, SFX(vec3) P)
{
    long i0[3];
    REAL a[3];
    if (!SFX(tex_setup)(v, P, i0, a)) return 0;
    REAL acc = 0;
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                REAL w = (dx ? a[0] : (REAL)1 - a[0]) * (dy ? a[1] : (REAL)1 - a[1]) * (dz ? a[2] : (REAL)1 - a[2]);
                acc += w * SFX(texel_density)(v, i0[0] + dx, i0[1] + dy, i0[2] + dz);
            }
    return acc;
}

/* |grad rho|_1 of the trilinear density at P in texel units: how much the
 * sample can change per texel of movement.  Test-side only. */
static double SFX(density_slope)(const SFX(vol)* v, SFX(vec3) P)
{
    long i0[3];
    REAL a[3];
    if (!SFX(tex_setup)(v, P, i0, a)) return 0.0;
    double g[3] = {0, 0, 0};
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                const double t = (double)SFX(texel_density)(v, i0[0] + dx, i0[1] + dy, i0[2] + dz);
                const double wx = dx ? (double)a[0] : 1.0 - (double)a[0];
                const double wy = dy ? (double)a[1] : 1.0 - (double)a[1];
                const double wz = dz ? (double)a[2] : 1.0 - (double)a[2];
                g[0] += (dx ? 1.0 : -1.0) * wy * wz * t;
                g[1] += wx * (dy ? 1.0 : -1.0) * wz * t;
                g[2] += wx * wy * (dz ? 1.0 : -1.0) * t;
            }
    return fabs(g[0]) + fabs(g[1]) + fabs(g[2]);
}

static SFX(vec3) SFX(sample_tangent)(const SFX(vol)* v, SFX(vec3) P)
{
    long i0[3];
    REAL a[3];
    SFX(vec3) acc = SFX(v3)(0, 0, 0);
    if (!SFX(tex_setup)(v, P, i0, a)) return acc;
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                REAL w = (dx ? a[0] : (REAL)1 - a[0]) * (dy ? a[1] : (REAL)1 - a[1]) * (dz ? a[2] : (REAL)1 - a[2]);
                acc = SFX(add)(acc, SFX(scale)(SFX(texel_tangent)(v, i0[0] + dx, i0[1] + dy, i0[2] + dz), w));
            }
    return acc;
}

/* (projection * view * vec4(P, 1)).z / .w with pv = projection * view. */
static inline REAL SFX(clip_depth)(const REAL pv[16], SFX(vec3) P)
{
    REAL z = pv[2] * P.x + pv[6] * P.y + pv[10] * P.z + pv[14];
    REAL w = pv[3] * P.x + pv[7] * P.y + pv[11] * P.z + pv[15];
    return z / w;
}

/* volume_rendering.glsl:19-52 (volume_surface). */
static void SFX(volume_surface)(const SFX(vol)* dv, const REAL pv[16], SFX(vec3) start, SFX(vec3) end,
                                float steps, REAL iso, float depth_buffer, SFX(vec3)* surf_out,
                                REAL* a_out, double* margin, int* taken, double* support_margin,
                                double* iso_shift)
{
    double sm = 1.0 / 0.0, shift = 1.0 / 0.0, slope = 0.0;
    REAL acc = 0;
    float step_size = 1.0f / steps;
    SFX(vec3) surface_point = SFX(v3)(0, 0, 0);
    int surface_point_found = 0, entry_point_found = 0;
    SFX(vec3) entry_point = SFX(v3)(0, 0, 0);
    double m = 1.0 / 0.0;
    int k = 0;
    for (float t = 0.0f; t < 1.0f; t += step_size) {
        SFX(vec3) P = SFX(mix)(start, end, (REAL)t);
        REAL depth = SFX(clip_depth)(pv, P);
        if ((REAL)depth_buffer < depth) break;
        ++k;
        REAL density = SFX(sample_density)(dv, P);
        /* before the surface point freezes, a sample's zero/nonzero status
         * decides the entry and surface points */
        if (support_margin && !(acc > iso)) {
            double sup = SFX(support_margin)(dv, P);
            if (sup < sm) sm = sup;
        }
        if (iso_shift && !(acc > iso)) slope += SFX(density_slope)(dv, P);
        acc += density;
        if (density != (REAL)0) {
            double dm = fabs((double)acc - (double)iso) / (double)iso;
            if (dm < m) m = dm;
            if (iso_shift && slope > 0.0) {
                double sh = fabs((double)acc - (double)iso) / slope;
                if (sh < shift) shift = sh;
            }
            if (acc <= iso) surface_point = P;
            if (acc >= iso) surface_point_found = 1;
            if (!entry_point_found) {
                entry_point = P;
                entry_point_found = 1;
            }
        }
    }
    if (!surface_point_found && entry_point_found) surface_point = entry_point;
    *surf_out = surface_point;
    *a_out = acc / iso;
    if (margin) *margin = m;
    if (taken) *taken = k;
    if (support_margin) *support_margin = sm;
    if (iso_shift) *iso_shift = shift;
}

/* One Kajiya-Kay specular lobe (kajiya-kay.glsl:15-21) of unit tangent t. */
static REAL SFX(kk_lobe)(SFX(vec3) tangent, SFX(vec3) light, SFX(vec3) eye, REAL p)
{
    REAL cosTL = SFX(dot)(tangent, light);
    REAL cosTE = SFX(dot)(tangent, eye);
    REAL a = (REAL)1 - cosTL * cosTL, b = (REAL)1 - cosTE * cosTE;
    REAL sinTL = SQRT_FN(a > 0 ? a : 0); /* sqrt of a negative rounding residue: 0 */
    REAL sinTE = SQRT_FN(b > 0 ? b : 0);
    REAL c = cosTL * cosTE + sinTL * sinTE;
    return POW_FN(c > 0 ? c : 0, p);
}

/* Extension: the tangent of a shifted lobe, normalize(t + shift * N) with N
 * the unit direction towards the camera perpendicular to t (eye points from
 * the camera to the surface); t itself where N is undefined (t || eye). */
static SFX(vec3) SFX(shift_tangent)(SFX(vec3) t, SFX(vec3) eye, REAL shift)
{
    SFX(vec3) v = SFX(scale)(eye, (REAL)-1);
    SFX(vec3) n = SFX(sub)(v, SFX(scale)(t, SFX(dot)(t, v)));
    REAL len = SQRT_FN(SFX(dot)(n, n));
    if (!(len > 0)) return t;
    return SFX(normalize)(SFX(add)(t, SFX(scale)(n, shift / len)), NULL);
}

/* kajiya-kay.glsl:7-24; `kd` scales the diffuse term (1 = reference).
 * Extension (all zero: the reference): a second, hair-coloured lobe of
 * exponent p2 > 0 and per-lobe tangent shifts. */
static SFX(vec3) SFX(kajiya_kay)(SFX(vec3) diffuse, SFX(vec3) specular, REAL p, SFX(vec3) tangent,
                                  SFX(vec3) light, SFX(vec3) eye, REAL kd, REAL p2, REAL shift1, REAL shift2)
{
    REAL cosTL = SFX(dot)(tangent, light);
    REAL cosTE = SFX(dot)(tangent, eye);
    REAL a = (REAL)1 - cosTL * cosTL, b = (REAL)1 - cosTE * cosTE;
    REAL sinTL = SQRT_FN(a > 0 ? a : 0); /* sqrt of a negative rounding residue: 0 */
    REAL sinTE = SQRT_FN(b > 0 ? b : 0);
    REAL spec;
    if (shift1 == 0) {
        REAL c = cosTL * cosTE + sinTL * sinTE;
        spec = POW_FN(c > 0 ? c : 0, p);
    } else {
        spec = SFX(kk_lobe)(SFX(shift_tangent)(tangent, eye, shift1), light, eye, p);
    }
    SFX(vec3) out = SFX(add)(SFX(scale)(diffuse, kd * sinTL), SFX(scale)(specular, spec));
    if (p2 > 0) {
        SFX(vec3) t2 = shift2 == 0 ? tangent : SFX(shift_tangent)(tangent, eye, shift2);
        out = SFX(add)(out, SFX(scale)(SFX(mul)(specular, diffuse), SFX(kk_lobe)(t2, light, eye, p2)));
    }
    return out;
}

/* approximate_deep_shadows.glsl:24-36. */
static REAL SFX(deep_shadows)(const SFX(vol)* dv, SFX(vec3) s, SFX(vec3) light, float steps, REAL alpha,
                               REAL thickness)
{
    REAL strands = 0;
    float step_size = 1.0f / steps;
    for (float t = 0.0f; t < 1.0f; t += step_size) {
        SFX(vec3) point = SFX(mix)(s, light, (REAL)t);
        strands += SFX(sample_density)(dv, point) * thickness;
    }
    return POW_FN((REAL)1 - alpha, strands);
}

/* Extension: AO direction i of n, the Fibonacci-sphere point with y as the
 * polar axis (the directional AO of vkhr_raymarch_params). */
static inline void SFX(ao_direction)(int i, int n, double d[3])
{
    const double pi = 3.14159265358979323846;
    double y = 1.0 - (2.0 * i + 1.0) / (double)n;
    double r = sqrt(1.0 - y * y);
    double phi = (double)i * pi * (3.0 - sqrt(5.0));
    d[0] = r * cos(phi);
    d[1] = y;
    d[2] = r * sin(phi);
}

/* local_ambient_occlusion.glsl:9-30; directions > 0: the directional
 * extension, taps at s + d_i * radius * sqrt(3) * voxel size. */
static REAL SFX(lao)(const SFX(vol)* dv, SFX(vec3) s, float kernel_size, REAL radius, REAL intensity,
                     REAL min_intensity, int directions)
{
    REAL density = 0;
    SFX(vec3) voxel_space = SFX(v3)(dv->size.x / (REAL)dv->n[0], dv->size.y / (REAL)dv->n[1],
                                    dv->size.z / (REAL)dv->n[2]);
    if (directions > 0) {
        for (int i = 0; i < directions; ++i) {
            double d[3];
            SFX(ao_direction)(i, directions, d);
            const double reach = (double)radius * sqrt(3.0);
            SFX(vec3) q = SFX(add)(s, SFX(mul)(SFX(v3)((REAL)(d[0] * reach), (REAL)(d[1] * reach),
                                                       (REAL)(d[2] * reach)), voxel_space));
            REAL r = SFX(sample_density)(dv, q);
            density += r < min_intensity ? r : min_intensity;
        }
        return POW_FN((REAL)1 - density / (REAL)directions, intensity);
    }
    float kernel_radius = (kernel_size - 1.0f) / 2.0f;
    REAL voxel_scaling = radius / (REAL)kernel_radius;
    SFX(vec3) sc = SFX(scale)(voxel_space, voxel_scaling);
    for (float z = -kernel_radius; z <= +kernel_radius; z += 1.0f)
        for (float y = -kernel_radius; y <= +kernel_radius; y += 1.0f)
            for (float x = -kernel_radius; x <= +kernel_radius; x += 1.0f) {
                SFX(vec3) q = SFX(add)(s, SFX(mul)(SFX(v3)((REAL)x, (REAL)y, (REAL)z), sc));
                REAL r = SFX(sample_density)(dv, q);
                density += r < min_intensity ? r : min_intensity;
            }
    REAL k3 = (REAL)kernel_size * (REAL)kernel_size * (REAL)kernel_size;
    return POW_FN((REAL)1 - density / k3, intensity);
}

/* scheme.glsl:7-11 */
static REAL SFX(lod)(int renderer, REAL mag, REAL min_d, REAL cur)
{
    if (renderer == 0) return 0;
    if (renderer == 2) return 1;
    REAL t = (cur - mag) / (min_d - mag);
    t = t < 0 ? 0 : (t > 1 ? 1 : t);
    return t * t * ((REAL)3 - (REAL)2 * t);
}

/* packUnorm4x8's clamp(c, 0, 1) (ppll.glsl:32) with IEEE 754-2008 min/max,
 * which return the non-NaN operand: NaN maps to 0. */
static inline float SFX(clamp01)(REAL x) { return (float)(x > 0 ? (x < 1 ? x : 1) : 0); }

/* volume.frag:31-103 for one pixel whose entry point is `start`. */
static void SFX(shade_pixel)(const vkhr_raymarch_params* p, const SFX(vol)* dv, const SFX(vol)* tv,
                             const REAL pv[16], SFX(vec3) start, float depth_buffer, float* rgba,
                             float* depth_out, oracle_pixel_diag* diag)
{
    SFX(vec3) cam = SFX(from)(p->camera_position);
    REAL radius = (REAL)p->volume_bounds.radius;
    SFX(vec3) dir = SFX(normalize)(SFX(sub)(start, cam), NULL);
    SFX(vec3) end = SFX(add)(start, SFX(scale)(dir, radius));

    SFX(vec3) surf;
    REAL a;
    double margin, support;
    int taken;
    double shift;
    SFX(volume_surface)(dv, pv, start, end, p->raycast_steps, (REAL)p->isosurface, depth_buffer, &surf, &a,
                        &margin, &taken, diag ? &support : NULL, diag ? &shift : NULL);
    if (diag) {
        diag->iso_margin = margin;
        diag->steps_taken = taken;
        diag->tangent_len = 0;
        diag->support_margin = support;
        diag->iso_shift = shift;
        double tsc = 0, sc = 0;
        for (int c = 0; c < 3; ++c) {
            const double t = (double)p->volume_resolution[c] / (double)p->volume_bounds.size[c];
            if (t > tsc) tsc = t;
        }
        sc = sqrt((double)(start.x * start.x + start.y * start.y + start.z * start.z));
        diag->fp32_res = ldexp(sc + (double)p->volume_bounds.radius, -24) * tsc;
    }
    rgba[0] = rgba[1] = rgba[2] = rgba[3] = 0.0f;
    if (depth_out) *depth_out = 1.0f;
    if (a == (REAL)0) return; /* discard */

    REAL coverage = SFX(lod)(p->renderer, (REAL)p->magnified_distance, (REAL)p->minified_distance,
                             (REAL)p->look_at_distance) * a * (REAL)p->hair_alpha;
    SFX(vec3) shading = SFX(v3)(1, 1, 1);
    SFX(vec3) lo = SFX(from)(p->light_origin);
    SFX(vec3) L = SFX(normalize)(SFX(sub)(lo, surf), NULL);
    SFX(vec3) E = SFX(normalize)(SFX(sub)(surf, cam), NULL);
    REAL tlen;
    SFX(vec3) T = SFX(normalize)(SFX(sample_tangent)(tv, surf), &tlen);
    if (diag) diag->tangent_len = (double)tlen;
    if (p->shading_model == VKHR_SHADING_KAJIYA_KAY)
        shading = SFX(kajiya_kay)(SFX(from)(p->hair_color), SFX(from)(p->light_intensity), (REAL)p->hair_exponent,
                                  T, L, E, (REAL)p->kd, (REAL)p->spec_exponent2, (REAL)p->spec_shift[0],
                                  (REAL)p->spec_shift[1]);
    REAL occlusion = 1;
    if (p->deep_shadows_on == 1 && p->shading_model != VKHR_SHADING_LAO) {
        float ss = p->shadow_steps > 0.0f ? p->shadow_steps : p->raycast_steps;
        occlusion *= SFX(deep_shadows)(dv, surf, lo, ss, (REAL)p->hair_alpha, (REAL)p->shadow_thickness);
    }
    if (p->shading_model != VKHR_SHADING_ADSM)
        occlusion *= SFX(lao)(dv, surf, p->ao_kernel_size, (REAL)p->occlusion_radius, (REAL)p->ao_exponent,
                              (REAL)p->ao_max, p->ao_directions);
    rgba[0] = SFX(clamp01)(shading.x * occlusion);
    rgba[1] = SFX(clamp01)(shading.y * occlusion);
    rgba[2] = SFX(clamp01)(shading.z * occlusion);
    rgba[3] = SFX(clamp01)(coverage);
    if (depth_out) *depth_out = (float)SFX(clip_depth)(pv, surf);
}

static void SFX(raymarch_rows)(const vkhr_raymarch_params* p, const void* density, const void* tangent,
                               const float* depth_in, float* rgba, float* depth_out, oracle_pixel_diag* diag,
                               int row_begin, int row_end, int threads)
{
    SFX(vol) dv, tv;
    dv.data = density; dv.fmt = p->density_format;
    tv.data = tangent; tv.fmt = p->tangent_format;
    for (int c = 0; c < 3; ++c) { dv.n[c] = tv.n[c] = p->volume_resolution[c]; }
    dv.origin = tv.origin = SFX(from)(p->volume_bounds.origin);
    dv.size = tv.size = SFX(from)(p->volume_bounds.size);
    REAL pv[16];
    for (int c = 0; c < 4; ++c)       /* column c of projection * view */
        for (int r = 0; r < 4; ++r) {
            REAL s = 0;
            for (int k = 0; k < 4; ++k) s += (REAL)p->projection[k * 4 + r] * (REAL)p->view[c * 4 + k];
            pv[c * 4 + r] = s;
        }
    const int W = p->width;
    double inv[16];
    int invertible = oracle_vp_inverse(p, inv);
    if (threads <= 0) threads = oracle_max_threads();
    /* pixels, not rows, are the unit of work: a call over a few rows (or the
     * footprint of a small volume) still uses every thread */
#pragma omp parallel for collapse(2) schedule(dynamic, 64) num_threads(threads)
    for (int y = row_begin; y < row_end; ++y) {
        for (int x = 0; x < W; ++x) {
            size_t at = (size_t)y * (size_t)W + (size_t)x;
            double st[3];
            oracle_pixel_diag* dg = diag ? diag + at : NULL;
            if (dg) {
                dg->iso_margin = 1.0 / 0.0;
                dg->support_margin = 1.0 / 0.0;
                dg->iso_shift = 1.0 / 0.0;
                dg->fp32_res = 0;
                dg->tangent_len = 0;
                dg->steps_taken = 0;
                dg->covered = 0;
            }
            if (!invertible || !oracle_pixel_entry_inv(p, inv, x, y, st)) {
                rgba[4 * at + 0] = rgba[4 * at + 1] = rgba[4 * at + 2] = rgba[4 * at + 3] = 0.0f;
                if (depth_out) depth_out[at] = 1.0f;
                continue;
            }
            if (dg) dg->covered = 1;
            float db = depth_in ? depth_in[at] : 1.0f;
            SFX(shade_pixel)(p, &dv, &tv, pv, SFX(v3)((REAL)st[0], (REAL)st[1], (REAL)st[2]), db, rgba + 4 * at,
                             depth_out ? depth_out + at : NULL, dg);
            if (dg) dg->covered = 1;
        }
    }
}
