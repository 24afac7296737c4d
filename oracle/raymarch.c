/*
 * raymarch.c -- CPU oracle (test infrastructure only): instantiates
 * raymarch_body.h in FP64 and FP32 and provides the rasterizer stand-in for
 * the volume proxy cube.
 *
 * Proxy cube (src/vkhr/rasterizer/volume.cc:60-102, volume.vert:17-25): the
 * reference rasterizes the AABB's 12 triangles with back-face culling, so a
 * pixel spawns exactly one fragment when the ray through its centre enters
 * the box from outside, and the fragment's interpolated world position is the
 * entry point.  Here that is a slab test on the ray from camera.position
 * through the pixel centre (Vulkan: pixel centre (x+0.5, y+0.5), NDC in
 * [-1,1], projection already y-flipped by the camera, camera.cc:229).
 */
#include "vkhr_oracle.h"

#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* inverse(projection * view) in FP64 by Gauss-Jordan; column-major. */
int oracle_vp_inverse(const vkhr_raymarch_params* p, double inv[16])
{
    double m[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            double s = 0;
            for (int k = 0; k < 4; ++k) s += (double)p->projection[k * 4 + r] * (double)p->view[c * 4 + k];
            m[r][c] = s;
            m[r][c + 4] = (r == c) ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if (fabs(m[r][c]) > fabs(m[piv][c])) piv = r;
        if (m[piv][c] == 0.0) return 0;
        if (piv != c)
            for (int k = 0; k < 8; ++k) { double t = m[c][k]; m[c][k] = m[piv][k]; m[piv][k] = t; }
        double d = m[c][c];
        for (int k = 0; k < 8; ++k) m[c][k] /= d;
        for (int r = 0; r < 4; ++r)
            if (r != c) {
                double f = m[r][c];
                for (int k = 0; k < 8; ++k) m[r][k] -= f * m[c][k];
            }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) inv[c * 4 + r] = m[r][c + 4];
    return 1;
}

int oracle_pixel_entry_inv(const vkhr_raymarch_params* p, const double inv[16], int px, int py, double start[3])
{
    double nx = 2.0 * ((double)px + 0.5) / (double)p->width - 1.0;
    double ny = 2.0 * ((double)py + 0.5) / (double)p->height - 1.0;
    double f[4];
    for (int r = 0; r < 4; ++r) f[r] = inv[r] * nx + inv[4 + r] * ny + inv[8 + r] * 1.0 + inv[12 + r];
    double o[3], d[3];
    for (int c = 0; c < 3; ++c) {
        o[c] = (double)p->camera_position[c];
        d[c] = f[c] / f[3] - o[c];
    }
    double tmin = -INFINITY, tmax = INFINITY;
    for (int c = 0; c < 3; ++c) {
        double lo = (double)p->volume_bounds.origin[c];
        double hi = lo + (double)p->volume_bounds.size[c];
        if (d[c] == 0.0) {
            if (o[c] < lo || o[c] > hi) return 0;
            continue;
        }
        double t0 = (lo - o[c]) / d[c], t1 = (hi - o[c]) / d[c];
        if (t0 > t1) { double t = t0; t0 = t1; t1 = t; }
        if (t0 > tmin) tmin = t0;
        if (t1 < tmax) tmax = t1;
    }
    if (!(tmin > 0.0) || !(tmin <= tmax)) return 0; /* miss, or camera inside (only back faces) */
    for (int c = 0; c < 3; ++c) start[c] = o[c] + tmin * d[c];
    return 1;
}

int oracle_pixel_entry(const vkhr_raymarch_params* p, int px, int py, double start[3])
{
    double inv[16];
    if (!oracle_vp_inverse(p, inv)) return 0;
    return oracle_pixel_entry_inv(p, inv, px, py, start);
}

#define REAL double
#define SFX(name) name##_f64
#define SQRT_FN sqrt
#define POW_FN pow
#define FLOOR_FN floor
#include "raymarch_body.h"
#undef REAL
#undef SFX
#undef SQRT_FN
#undef POW_FN
#undef FLOOR_FN

#define REAL float
#define SFX(name) name##_f32
#define SQRT_FN sqrtf
#define POW_FN powf
#define FLOOR_FN floorf
#include "raymarch_body.h"

void oracle_raymarch_f64(const vkhr_raymarch_params* p, const void* density, const void* tangent,
                         const float* depth_in, float* rgba, float* depth_out, oracle_pixel_diag* diag,
                         int row_begin, int row_end, int threads)
{
    raymarch_rows_f64(p, density, tangent, depth_in, rgba, depth_out, diag, row_begin, row_end, threads);
}

void oracle_raymarch_f32(const vkhr_raymarch_params* p, const void* density, const void* tangent,
                         const float* depth_in, float* rgba, float* depth_out, int row_begin, int row_end,
                         int threads)
{
    raymarch_rows_f32(p, density, tangent, depth_in, rgba, depth_out, NULL, row_begin, row_end, threads);
}
