/*
 * adjoint.c -- CPU oracle (test infrastructure only): the differentiable
 * raymarch in FP64 and its analytic gradient, and the trilinear splat.
 *
 * The forward is volume.frag:31-103 as in raymarch_body.h (instantiated here
 * for double, volumes in ORACLE_F64), with the output kept in double so that
 * central finite differences of the loss are not polluted by rounding.  The
 * gradient treats the discrete decisions (surface point, zero tests) as
 * constants and differentiates the rest:
 *   coverage = lod * acc / iso * alpha (acc = sum of all primary samples),
 *   rgb = clamp(KK(T(surf)) * (1 - alpha)^(thickness * sum shadow samples)
 *              * (1 - sum min(rho, ao_max) / taps)^ao_exp),
 *   T = normalize(trilinear tangent), samples trilinear in their 8 texels;
 * the clamps pass gradient strictly inside (0, 1).  KK is the dual-lobe,
 * shifted form of the vkhr_raymarch_params extension (one unshifted lobe
 * with its knobs at zero); its gradient goes through the scalar form of the
 * shift (lobe_grad below), while the forward evaluates the vector definition
 * (raymarch_body.h), so the finite-difference tests check one against the other.
 */
#include "vkhr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define REAL double
#define SFX(name) name##_ad
#define SQRT_FN sqrt
#define POW_FN pow
#define FLOOR_FN floor
#include "raymarch_body.h"

typedef struct grads {
    double* density; /* per voxel */
    double* tangent; /* 4 per voxel */
    double params[3];
} grads;

/* One specular lobe as a function of a = T.L and b = T.E, with c = L.E
 * fixed.  Shifting T by s towards the camera (normalize(T + s N), N the unit
 * component of -E perpendicular to T) gives
 *   a_s = k (a + s (a b - c) / sb),  b_s = k (b - s sb),
 *   sb = sqrt(1 - b^2) = sin(T, E),  k = 1 / sqrt(1 + s^2),
 * and the lobe is max(a_s b_s + sqrt(1 - a_s^2) sqrt(1 - b_s^2), 0)^p.
 * Returns the lobe; *da, *db and *dp receive its partials. */
static double lobe_grad(double a, double b, double c, double s, double p, double* da, double* db, double* dp)
{
    double as = a, bs = b, j00 = 1, j01 = 0, j11 = 1; /* d(a_s, b_s) / d(a, b); d b_s / d a = 0 */
    const double sb = sqrt(1 - b * b > 0 ? 1 - b * b : 0);
    if (s != 0 && sb > 0) {
        const double k = 1 / sqrt(1 + s * s);
        as = k * (a + s * (a * b - c) / sb);
        bs = k * (b - s * sb);
        j00 = k * (1 + s * b / sb);
        j01 = k * s * (a / sb + (a * b - c) * b / (sb * sb * sb));
        j11 = k * (1 + s * b / sb);
    }
    const double sa2 = sqrt(1 - as * as > 0 ? 1 - as * as : 0), sb2 = sqrt(1 - bs * bs > 0 ? 1 - bs * bs : 0);
    double base = as * bs + sa2 * sb2;
    base = base > 0 ? base : 0;
    const double spec = pow(base, p);
    *da = *db = *dp = 0;
    if (base > 0) {
        const double ds = p * pow(base, p - 1);
        double gas = bs, gbs = as; /* d base / d a_s, d base / d b_s */
        if (sa2 > 0) gas -= sb2 * as / sa2;
        if (sb2 > 0) gbs -= sa2 * bs / sb2;
        *da = ds * gas * j00;
        *db = ds * (gas * j01 + gbs * j11);
        *dp = spec * log(base);
    }
    return spec;
}

static void scatter_density(const vol_ad* v, vec3_ad P, double g, double* grad)
{
    long i0[3];
    double a[3];
    if (!grad || g == 0.0 || !tex_setup_ad(v, P, i0, a)) return;
    for (int k = 0; k < 8; ++k) {
        const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
        const long x = i0[0] + dx, y = i0[1] + dy, z = i0[2] + dz;
        if (x < 0 || y < 0 || z < 0 || x >= v->n[0] || y >= v->n[1] || z >= v->n[2]) continue;
        const double w = (dx ? a[0] : 1 - a[0]) * (dy ? a[1] : 1 - a[1]) * (dz ? a[2] : 1 - a[2]);
        grad[(size_t)x + (size_t)v->n[0] * ((size_t)y + (size_t)v->n[1] * (size_t)z)] += g * w;
    }
}

static void scatter_tangent(const vol_ad* v, vec3_ad P, vec3_ad g, double* grad)
{
    long i0[3];
    double a[3];
    if (!grad || !tex_setup_ad(v, P, i0, a)) return;
    for (int k = 0; k < 8; ++k) {
        const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
        const long x = i0[0] + dx, y = i0[1] + dy, z = i0[2] + dz;
        if (x < 0 || y < 0 || z < 0 || x >= v->n[0] || y >= v->n[1] || z >= v->n[2]) continue;
        const double w = (dx ? a[0] : 1 - a[0]) * (dy ? a[1] : 1 - a[1]) * (dz ? a[2] : 1 - a[2]);
        double* t = grad + 4 * ((size_t)x + (size_t)v->n[0] * ((size_t)y + (size_t)v->n[1] * (size_t)z));
        t[0] += g.x * w;
        t[1] += g.y * w;
        t[2] += g.z * w;
    }
}

static double clamp01_d(double x) { return x > 0 ? (x < 1 ? x : 1) : 0; }
static double clamp_grad(double x, double g) { return (x > 0 && x < 1) ? g : 0; }

/* Position of directional AO tap i (the extension of local_ambient_occlusion.glsl). */
static vec3_ad ao_tap(const vkhr_raymarch_params* p, vec3_ad s, vec3_ad voxel_space, int i)
{
    double d[3];
    ao_direction_ad(i, p->ao_directions, d);
    const double reach = (double)p->occlusion_radius * sqrt(3.0);
    return add_ad(s, mul_ad(v3_ad(d[0] * reach, d[1] * reach, d[2] * reach), voxel_space));
}

/* One pixel: returns its loss sum_c (rgba_c - target_c)^2 and, with gr,
 * adds its gradient. */
static double diff_pixel(const vkhr_raymarch_params* p, const vol_ad* dv, const vol_ad* tv, vec3_ad start,
                         const float* target, grads* gr)
{
    const vec3_ad cam = from_ad(p->camera_position);
    const vec3_ad dir = normalize_ad(sub_ad(start, cam), NULL);
    const vec3_ad end = add_ad(start, scale_ad(dir, (double)p->volume_bounds.radius));
    const double iso = p->isosurface;
    /* volume_surface (volume_rendering.glsl:19-52) without a depth buffer */
    const float step = 1.0f / p->raycast_steps;
    double acc = 0;
    vec3_ad surf = v3_ad(0, 0, 0), entry = v3_ad(0, 0, 0);
    int found = 0, entered = 0;
    for (float t = 0.0f; t < 1.0f; t += step) {
        const vec3_ad P = mix_ad(start, end, (double)t);
        const double rho = sample_density_ad(dv, P);
        acc += rho;
        if (rho != 0) {
            if (acc <= iso) surf = P;
            if (acc >= iso) found = 1;
            if (!entered) { entry = P; entered = 1; }
        }
    }
    if (!found && entered) surf = entry;
    double rgba[4] = {0, 0, 0, 0};
    const double a = acc / iso;
    if (a == 0) { /* discarded: nothing depends smoothly on the volume */
        double l = 0;
        for (int c = 0; c < 4; ++c) l += (double)target[c] * (double)target[c];
        return l;
    }
    const double lodv = lod_ad(p->renderer, p->magnified_distance, p->minified_distance, p->look_at_distance);
    const double alpha = p->hair_alpha;
    const double coverage = lodv * a * alpha;
    const vec3_ad light = from_ad(p->light_origin);
    const int kk = p->shading_model == VKHR_SHADING_KAJIYA_KAY;
    vec3_ad shading = v3_ad(1, 1, 1), L = v3_ad(0, 0, 0), E = v3_ad(0, 0, 0), T = v3_ad(0, 0, 0);
    vec3_ad Tr = v3_ad(0, 0, 0);
    double cosTL = 0, cosTE = 0, sinTL = 0, tlen = 0;
    const vec3_ad color = from_ad(p->hair_color), inten = from_ad(p->light_intensity);
    const double p2 = p->spec_exponent2 > 0 ? (double)p->spec_exponent2 : 0;
    if (kk) {
        L = normalize_ad(sub_ad(light, surf), NULL);
        E = normalize_ad(sub_ad(surf, cam), NULL);
        Tr = sample_tangent_ad(tv, surf);
        T = normalize_ad(Tr, &tlen);
        cosTL = dot_ad(T, L);
        cosTE = dot_ad(T, E);
        sinTL = sqrt(1 - cosTL * cosTL > 0 ? 1 - cosTL * cosTL : 0);
        shading = kajiya_kay_ad(color, inten, (double)p->hair_exponent, T, L, E, (double)p->kd, p2,
                                (double)p->spec_shift[0], (double)p->spec_shift[1]);
    }
    const int shadows = p->deep_shadows_on == 1 && p->shading_model != VKHR_SHADING_LAO;
    const int lao = p->shading_model != VKHR_SHADING_ADSM;
    double occl_s = 1, strands = 0;
    const float ss = p->shadow_steps > 0.0f ? p->shadow_steps : p->raycast_steps;
    const float sstep = 1.0f / ss;
    if (shadows) {
        for (float t = 0.0f; t < 1.0f; t += sstep)
            strands += sample_density_ad(dv, mix_ad(surf, light, (double)t)) * (double)p->shadow_thickness;
        occl_s = pow(1 - alpha, strands);
    }
    const float kr = (p->ao_kernel_size - 1.0f) / 2.0f;
    const int ndir = p->ao_directions;
    const double k3 = ndir > 0 ? (double)ndir
                               : (double)p->ao_kernel_size * (double)p->ao_kernel_size * (double)p->ao_kernel_size;
    const vec3_ad vs = v3_ad((double)p->volume_bounds.size[0] / p->volume_resolution[0],
                             (double)p->volume_bounds.size[1] / p->volume_resolution[1],
                             (double)p->volume_bounds.size[2] / p->volume_resolution[2]);
    const vec3_ad sc = scale_ad(vs, (double)p->occlusion_radius / (double)kr);
    double dsum = 0, occl_a = 1;
    if (lao && ndir > 0) { /* the directional taps */
        for (int i = 0; i < ndir; ++i) {
            const double r = sample_density_ad(dv, ao_tap(p, surf, vs, i));
            dsum += r < p->ao_max ? r : (double)p->ao_max;
        }
        occl_a = pow(1 - dsum / k3, (double)p->ao_exponent);
    } else if (lao) {
        for (float z = -kr; z <= kr; z += 1.0f)
            for (float y = -kr; y <= kr; y += 1.0f)
                for (float x = -kr; x <= kr; x += 1.0f) {
                    const double r = sample_density_ad(dv, add_ad(surf, mul_ad(v3_ad(x, y, z), sc)));
                    dsum += r < p->ao_max ? r : (double)p->ao_max;
                }
        occl_a = pow(1 - dsum / k3, (double)p->ao_exponent);
    }
    const double occl = occl_s * occl_a;
    const double x[3] = {shading.x * occl, shading.y * occl, shading.z * occl};
    for (int c = 0; c < 3; ++c) rgba[c] = clamp01_d(x[c]);
    rgba[3] = clamp01_d(coverage);
    double loss = 0, g[4];
    for (int c = 0; c < 4; ++c) {
        const double d = rgba[c] - (double)target[c];
        loss += d * d;
        g[c] = 2 * d;
    }
    if (!gr) return loss;
    /* ---- backward ---- */
    const double ga = clamp_grad(coverage, g[3]) * lodv * alpha / iso;
    const double gx[3] = {clamp_grad(x[0], g[0]), clamp_grad(x[1], g[1]), clamp_grad(x[2], g[2])};
    const vec3_ad gsh = v3_ad(gx[0] * occl, gx[1] * occl, gx[2] * occl);
    const double gocc = gx[0] * shading.x + gx[1] * shading.y + gx[2] * shading.z;
    if (kk) {
        const double gi = dot_ad(gsh, inten), gc = dot_ad(gsh, color);
        const double gic = gsh.x * inten.x * color.x + gsh.y * inten.y * color.y + gsh.z * inten.z * color.z;
        const double cosLE = dot_ad(L, E);
        gr->params[0] += gc * sinTL;
        double da, db, dp;
        lobe_grad(cosTL, cosTE, cosLE, (double)p->spec_shift[0], (double)p->hair_exponent, &da, &db, &dp);
        double gcosTL = gi * da, gcosTE = gi * db;
        gr->params[1] += gi * dp;
        if (p2 > 0) {
            lobe_grad(cosTL, cosTE, cosLE, (double)p->spec_shift[1], p2, &da, &db, &dp);
            gcosTL += gic * da;
            gcosTE += gic * db;
            gr->params[2] += gic * dp;
        }
        if (sinTL > 0) gcosTL -= gc * (double)p->kd * cosTL / sinTL; /* the diffuse kd sin(T, L) */
        const vec3_ad gT = add_ad(scale_ad(L, gcosTL), scale_ad(E, gcosTE));
        if (tlen > 0) {
            const vec3_ad gTr = scale_ad(sub_ad(gT, scale_ad(T, dot_ad(gT, T))), 1 / tlen);
            scatter_tangent(tv, surf, gTr, gr->tangent);
        }
    }
    if (shadows && gocc != 0) {
        const double gs = gocc * occl_a * occl_s * log(1 - alpha) * (double)p->shadow_thickness;
        for (float t = 0.0f; t < 1.0f; t += sstep) scatter_density(dv, mix_ad(surf, light, (double)t), gs, gr->density);
    }
    if (lao && gocc != 0) {
        const double gd = -gocc * occl_s * (double)p->ao_exponent *
                          pow(1 - dsum / k3, (double)p->ao_exponent - 1) / k3;
        for (int i = 0; i < ndir; ++i) {
            const vec3_ad q = ao_tap(p, surf, vs, i);
            if (sample_density_ad(dv, q) < p->ao_max) scatter_density(dv, q, gd, gr->density);
        }
        for (float z = -kr; ndir <= 0 && z <= kr; z += 1.0f) /* the cube's taps */
            for (float y = -kr; y <= kr; y += 1.0f)
                for (float x = -kr; x <= kr; x += 1.0f) {
                    const vec3_ad q = add_ad(surf, mul_ad(v3_ad(x, y, z), sc));
                    if (sample_density_ad(dv, q) < p->ao_max) scatter_density(dv, q, gd, gr->density);
                }
    }
    if (ga != 0)
        for (float t = 0.0f; t < 1.0f; t += step) scatter_density(dv, mix_ad(start, end, (double)t), ga, gr->density);
    return loss;
}

double oracle_diff_loss(const vkhr_raymarch_params* p, const double* density, const double* tangent,
                        const float* target, const uint8_t* mask, double* g_density, double* g_tangent,
                        double* g_params, int threads)
{
    vol_ad dv, tv;
    dv.data = density;
    tv.data = tangent;
    dv.fmt = tv.fmt = ORACLE_F64;
    for (int c = 0; c < 3; ++c) dv.n[c] = tv.n[c] = p->volume_resolution[c];
    dv.origin = tv.origin = from_ad(p->volume_bounds.origin);
    dv.size = tv.size = from_ad(p->volume_bounds.size);
    double inv[16];
    if (!oracle_vp_inverse(p, inv)) return NAN;
    const int want = g_density || g_tangent || g_params;
    grads gr = {g_density, g_tangent, {0, 0, 0}};
    if (threads <= 0) threads = oracle_max_threads();
    if (want) threads = 1; /* the gradient scatter is serial */
    double loss = 0;
    const int W = p->width, H = p->height;
#pragma omp parallel for schedule(dynamic) num_threads(threads) reduction(+ : loss)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t at = (size_t)y * W + x;
            if (mask && !mask[at]) continue; /* excluded from the loss */
            double st[3];
            if (!oracle_pixel_entry_inv(p, inv, x, y, st)) {
                for (int c = 0; c < 4; ++c) loss += (double)target[4 * at + c] * (double)target[4 * at + c];
                continue;
            }
            loss += diff_pixel(p, &dv, &tv, v3_ad(st[0], st[1], st[2]), target + 4 * at, want ? &gr : NULL);
        }
    if (g_params) {
        g_params[0] += gr.params[0];
        g_params[1] += gr.params[1];
        g_params[2] += gr.params[2];
    }
    return loss;
}

/* Texel coordinate of the splat: u = (v - origin) / size * N - 0.5. */
static int splat_setup(const float* v, const vkhr_aabb* b, const int n[3], long i0[3], double a[3], double s[3])
{
    for (int k = 0; k < 3; ++k) {
        s[k] = (double)n[k] / (double)b->size[k];
        const double u = ((double)v[k] - (double)b->origin[k]) * s[k] - 0.5;
        if (!(u > -1 && u < n[k])) return 0;
        const double f = floor(u);
        i0[k] = (long)f;
        a[k] = u - f;
    }
    return 1;
}

void oracle_splat(const float* vertices, uint32_t nv, const vkhr_aabb* b, int w, int h, int d, double* density)
{
    const int n[3] = {w, h, d};
    for (uint32_t i = 0; i < nv; ++i) {
        long i0[3];
        double a[3], s[3];
        if (!splat_setup(vertices + 3 * (size_t)i, b, n, i0, a, s)) continue;
        for (int k = 0; k < 8; ++k) {
            const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
            const long x = i0[0] + dx, y = i0[1] + dy, z = i0[2] + dz;
            if (x < 0 || y < 0 || z < 0 || x >= w || y >= h || z >= d) continue;
            density[(size_t)x + (size_t)w * ((size_t)y + (size_t)h * (size_t)z)] +=
                (dx ? a[0] : 1 - a[0]) * (dy ? a[1] : 1 - a[1]) * (dz ? a[2] : 1 - a[2]);
        }
    }
}

void oracle_splat_adjoint(const float* vertices, uint32_t nv, const vkhr_aabb* b, int w, int h, int d,
                          const double* g_density, double* g_vertices)
{
    const int n[3] = {w, h, d};
    for (uint32_t i = 0; i < nv; ++i) {
        long i0[3];
        double a[3], s[3], gu[3] = {0, 0, 0};
        if (splat_setup(vertices + 3 * (size_t)i, b, n, i0, a, s)) {
            for (int k = 0; k < 8; ++k) {
                const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
                const long x = i0[0] + dx, y = i0[1] + dy, z = i0[2] + dz;
                if (x < 0 || y < 0 || z < 0 || x >= w || y >= h || z >= d) continue;
                const double gt = g_density[(size_t)x + (size_t)w * ((size_t)y + (size_t)h * (size_t)z)];
                const double wx = dx ? a[0] : 1 - a[0], wy = dy ? a[1] : 1 - a[1], wz = dz ? a[2] : 1 - a[2];
                gu[0] += gt * (dx ? 1 : -1) * wy * wz;
                gu[1] += gt * wx * (dy ? 1 : -1) * wz;
                gu[2] += gt * wx * wy * (dz ? 1 : -1);
            }
        }
        for (int k = 0; k < 3; ++k) g_vertices[3 * (size_t)i + k] = gu[k] * s[k];
    }
}
