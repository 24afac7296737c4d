// adjoint.cu -- the differentiable form of the volume path: a training
// forward that runs the raymarch of volume.frag:31-103 (march.cuh, the same
// device code as vkhr_raymarch) and records a per-ray tape with checkpoints,
// the hand-written adjoint of that raymarch with respect to an FP32 density
// volume, an FP32 tangent field and the Kajiya-Kay parameters (kd and the
// specular exponents of both lobes), and a continuous trilinear-splat
// voxelizer of strand vertices with its adjoint.
//
// The model's discrete decisions (the isosurface point, the early exit, the
// zero tests) are constants of the derivative; everything else is
// differentiated exactly:
//   coverage = lod * acc / iso * alpha, acc = sum of the primary samples;
//   rgb = clamp(shading * occl_s * occl_a), with shading the (dual-lobe,
//   shifted) Kajiya-Kay of the normalised trilinear tangent at the surface
//   point, occl_s = (1 - alpha)^(thickness * sum of the shadow samples) and
//   occl_a = (1 - sum(min(rho, ao_max)) / taps)^ao_exp;
//   every sample is trilinear in its 8 texels.
// The primary march is replayed from checkpoints of t stored every K
// iterations: one thread per (ray, K-iteration segment).
#include "march.cuh"

namespace {

// ---- training forward ------------------------------------------------------------------

template <int DF, int TF>
__global__ void __launch_bounds__(32 * kWarpsX * kWarpsY)
train_kernel(const __grid_constant__ RayConsts c, const typename DensityTexel<DF>::T* __restrict__ dens,
             const void* __restrict__ tang, const uint32_t* __restrict__ occ, float4* __restrict__ rgba,
             float* __restrict__ depth_out, PixelTape* __restrict__ tape, float* __restrict__ ckpt, uint32_t K,
             uint32_t nckpt)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int px = (blockIdx.x * kWarpsX + (warp % kWarpsX)) * kTileW + (lane % kTileW);
    const int py = (blockIdx.y * kWarpsY + (warp / kWarpsX)) * kTileH + (lane / kTileW);
    if (px >= c.W || py >= c.H) return;
    const size_t at = (size_t)py * c.W + px;
    float4 out;
    float out_depth;
    march_pixel<DF, TF, true>(c, dens, tang, occ, nullptr, px, py, out, out_depth, tape + at, ckpt + at * nckpt, K,
                              nckpt);
    rgba[at] = out;
    if (depth_out) depth_out[at] = out_depth;
}

// ---- adjoint -----------------------------------------------------------------------------

// Adds g * (trilinear weight) to the gradient of each of the 8 texels of a
// sample at P that lie inside the grid (border texels are not parameters).
__device__ __forceinline__ void scatter_density(const RayConsts& c, float* __restrict__ grad, Vec3 P, float g)
{
    int i0[3];
    float a[3];
    if (!tex_setup(c, P, i0, a)) return;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
        const int x = i0[0] + dx, y = i0[1] + dy, z = i0[2] + dz;
        if (x < 0 || y < 0 || z < 0 || x >= c.res[0] || y >= c.res[1] || z >= c.res[2]) continue;
        const float w = (dx ? a[0] : 1.0f - a[0]) * (dy ? a[1] : 1.0f - a[1]) * (dz ? a[2] : 1.0f - a[2]);
        atomicAdd(grad + (size_t)x + (size_t)c.res[0] * ((size_t)y + (size_t)c.res[1] * z), g * w);
    }
}

__device__ __forceinline__ void scatter_tangent(const RayConsts& c, float4* __restrict__ grad, Vec3 P, Vec3 g)
{
    int i0[3];
    float a[3];
    if (!tex_setup(c, P, i0, a)) return;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
        const int x = i0[0] + dx, y = i0[1] + dy, z = i0[2] + dz;
        if (x < 0 || y < 0 || z < 0 || x >= c.res[0] || y >= c.res[1] || z >= c.res[2]) continue;
        const float w = (dx ? a[0] : 1.0f - a[0]) * (dy ? a[1] : 1.0f - a[1]) * (dz ? a[2] : 1.0f - a[2]);
        float* t = reinterpret_cast<float*>(grad + (size_t)x + (size_t)c.res[0] * ((size_t)y + (size_t)c.res[1] * z));
        atomicAdd(t + 0, g.x * w);
        atomicAdd(t + 1, g.y * w);
        atomicAdd(t + 2, g.z * w);
    }
}

__device__ __forceinline__ float clamp_grad(float x, float g) { return (x > 0.0f && x < 1.0f) ? g : 0.0f; }

// kk_lobe and its partials with respect to a = T.L (da), b = T.E (db) and
// the exponent (dp), through the shifted cosines of shift_cosines (c = L.E
// is a constant of the derivative: L and E depend on the surface point only).
__device__ __forceinline__ float kk_lobe_grad(float a, float b, float sa, float sb, float cab, float s, float p,
                                              float& da, float& db, float& dp)
{
    float as = a, bs = b, sas = sa, sbs = sb, j00 = 1.0f, j01 = 0.0f, j11 = 1.0f;
    if (s != 0.0f && sb > 0.0f) {
        shift_cosines(a, b, sb, cab, s, as, bs);
        const float k = 1.0f / sqrtf(fmaf(s, s, 1.0f));
        j00 = j11 = k * (1.0f + s * b / sb);
        j01 = k * s * (a / sb + (a * b - cab) * b / (sb * sb * sb));
        sas = sqrtf(fmaxf(1.0f - as * as, 0.0f));
        sbs = sqrtf(fmaxf(1.0f - bs * bs, 0.0f));
    }
    const float base = fmaxf(as * bs + sas * sbs, 0.0f);
    const float spec = powf(base, p);
    da = db = dp = 0.0f;
    if (base > 0.0f) {
        const float ds = p * powf(base, p - 1.0f);
        float gas = bs, gbs = as; // d base / d a_s, d base / d b_s
        if (sas > 0.0f) gas -= sbs * as / sas;
        if (sbs > 0.0f) gbs -= sas * bs / sbs;
        da = ds * gas * j00;
        db = ds * (gas * j01 + gbs * j11);
        dp = spec * logf(base);
    }
    return spec;
}

// Per pixel: the gradient of the pixel's accumulated density (g_acc, for
// the segment replay below), and the shading, shadow and LAO parts of the
// adjoint, which depend on the surface point only.  kd and the specular
// exponents are reduced per warp into double accumulators.
template <int DF, int TF>
__global__ void __launch_bounds__(128) adjoint_pixel_kernel(const __grid_constant__ RayConsts c,
                                                            const float* __restrict__ dens,
                                                            const float4* __restrict__ tang,
                                                            const PixelTape* __restrict__ tape,
                                                            const float4* __restrict__ g_rgba,
                                                            float* __restrict__ g_acc, float* __restrict__ g_dens,
                                                            float4* __restrict__ g_tang, double* __restrict__ g_par)
{
    const uint32_t pixels = (uint32_t)c.W * (uint32_t)c.H;
    const uint32_t at = blockIdx.x * blockDim.x + threadIdx.x;
    float gkd = 0.0f, gexp = 0.0f, gexp2 = 0.0f;
    if (at < pixels) {
        const PixelTape tp = tape[at];
        float ga = 0.0f;
        if (tp.flags & kTapeEmitted) {
            const float4 g = g_rgba[at];
            const float a = tp.acc / c.iso;
            const float coverage = c.lod * a * c.alpha;
            ga = clamp_grad(coverage, g.w) * c.lod * c.alpha / c.iso;
            const Vec3 surf = v3(tp.surf[0], tp.surf[1], tp.surf[2]);
            const Vec3 cam = v3(c.cam[0], c.cam[1], c.cam[2]);
            const Vec3 light = v3(c.light[0], c.light[1], c.light[2]);
            // forward quantities at the surface point
            Vec3 shading = v3(1.0f, 1.0f, 1.0f);
            Vec3 L, E, T, Tr;
            float cosTL = 0.0f, cosTE = 0.0f, sinTL = 0.0f, sinTE = 0.0f, cosLE = 0.0f;
            float da1 = 0.0f, db1 = 0.0f, dp1 = 0.0f, da2 = 0.0f, db2 = 0.0f, dp2 = 0.0f;
            const bool kk = c.shading_model == VKHR_SHADING_KAJIYA_KAY;
            if (kk) {
                L = normalize(light - surf);
                E = normalize(surf - cam);
                Tr = sample_tangent<TF>(c, tang, surf);
                T = normalize(Tr);
                cosTL = dot(T, L);
                cosTE = dot(T, E);
                sinTL = sqrtf(fmaxf(1.0f - cosTL * cosTL, 0.0f));
                sinTE = sqrtf(fmaxf(1.0f - cosTE * cosTE, 0.0f));
                cosLE = dot(L, E);
                const float spec = kk_lobe_grad(cosTL, cosTE, sinTL, sinTE, cosLE, c.shift[0], c.exponent, da1, db1, dp1);
                const float dk = c.kd * sinTL;
                shading = v3(c.color[0] * dk + c.intensity[0] * spec, c.color[1] * dk + c.intensity[1] * spec,
                             c.color[2] * dk + c.intensity[2] * spec);
                if (c.exponent2 > 0.0f) {
                    const float spec2 =
                        kk_lobe_grad(cosTL, cosTE, sinTL, sinTE, cosLE, c.shift[1], c.exponent2, da2, db2, dp2);
                    shading = shading + v3(c.intensity[0] * c.color[0] * spec2, c.intensity[1] * c.color[1] * spec2,
                                           c.intensity[2] * c.color[2] * spec2);
                }
            }
            const bool shadows = c.deep_shadows_on == 1 && c.shading_model != VKHR_SHADING_LAO;
            const bool lao = c.shading_model != VKHR_SHADING_ADSM;
            const float k3 = c.ao_n > 0 ? (float)c.ao_n : c.ao_kernel * c.ao_kernel * c.ao_kernel; // taps
            const float ao_base = 1.0f - tp.dsum / k3;
            const float occl_a = lao ? powf(ao_base, c.ao_exp) : 1.0f;
            const float occl = (shadows ? tp.occl_s : 1.0f) * occl_a;
            // rgb = clamp(shading * occl)
            const Vec3 gx = v3(clamp_grad(shading.x * occl, g.x), clamp_grad(shading.y * occl, g.y),
                               clamp_grad(shading.z * occl, g.z));
            const Vec3 gsh = gx * occl;
            const float gocc = dot(gx, shading);
            if (kk) {
                const float gi = gsh.x * c.intensity[0] + gsh.y * c.intensity[1] + gsh.z * c.intensity[2];
                const float gc = gsh.x * c.color[0] + gsh.y * c.color[1] + gsh.z * c.color[2];
                const float gic = gsh.x * c.intensity[0] * c.color[0] + gsh.y * c.intensity[1] * c.color[1] +
                                  gsh.z * c.intensity[2] * c.color[2];
                gkd = gc * sinTL;
                gexp = gi * dp1;
                float gcosTL = gi * da1, gcosTE = gi * db1;
                if (c.exponent2 > 0.0f) {
                    gexp2 = gic * dp2;
                    gcosTL += gic * da2;
                    gcosTE += gic * db2;
                }
                if (sinTL > 0.0f) gcosTL -= gc * c.kd * cosTL / sinTL; // the diffuse kd sin(T, L)
                const Vec3 gT = L * gcosTL + E * gcosTE;
                const float len = sqrtf(dot(Tr, Tr));
                if (len > 0.0f) { // through T = Tr / |Tr|
                    const Vec3 gTr = (gT - T * dot(gT, T)) * (1.0f / len);
                    scatter_tangent(c, g_tang, surf, gTr);
                }
            }
            if (shadows && gocc != 0.0f) { // d occl / d strands = occl * ln(1 - alpha)
                const float gs = gocc * occl_a * tp.occl_s * logf(1.0f - c.alpha) * c.thickness;
                const float sstep = 1.0f / c.shadow_steps;
                for (float t = 0.0f; t < 1.0f; t += sstep) scatter_density(c, g_dens, mix(surf, light, t), gs);
            }
            if (lao && gocc != 0.0f && ao_base > 0.0f) {
                const float gd = -gocc * (shadows ? tp.occl_s : 1.0f) * c.ao_exp * powf(ao_base, c.ao_exp - 1.0f) / k3;
                for (int i = 0; i < c.ao_n; ++i) { // the directional taps
                    const Vec3 q = v3(surf.x + c.ao_off[i][0], surf.y + c.ao_off[i][1], surf.z + c.ao_off[i][2]);
                    if (sample_density<DF>(c, dens, q) < c.ao_max) scatter_density(c, g_dens, q, gd);
                }
                if (c.ao_n == 0) { // the cube's taps
                    const float kr = (c.ao_kernel - 1.0f) / 2.0f;
                    const float scale = c.ao_radius / kr;
                    const Vec3 sc = v3(c.voxel_space[0] * scale, c.voxel_space[1] * scale, c.voxel_space[2] * scale);
                    for (float z = -kr; z <= kr; z += 1.0f)
                        for (float y = -kr; y <= kr; y += 1.0f)
                            for (float x = -kr; x <= kr; x += 1.0f) {
                                const Vec3 q = v3(surf.x + x * sc.x, surf.y + y * sc.y, surf.z + z * sc.z);
                                if (sample_density<DF>(c, dens, q) < c.ao_max) scatter_density(c, g_dens, q, gd);
                            }
                }
            }
        }
        g_acc[at] = ga;
    }
    // kd and the exponents: warp sums, one double atomic per warp and parameter
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        gkd += __shfl_down_sync(0xffffffffu, gkd, o);
        gexp += __shfl_down_sync(0xffffffffu, gexp, o);
        gexp2 += __shfl_down_sync(0xffffffffu, gexp2, o);
    }
    if ((threadIdx.x & 31) == 0 && (gkd != 0.0f || gexp != 0.0f || gexp2 != 0.0f)) {
        atomicAdd(g_par + 0, (double)gkd);
        atomicAdd(g_par + 1, (double)gexp);
        atomicAdd(g_par + 2, (double)gexp2);
    }
}

// The primary march replayed from its checkpoints: thread (pixel, m) walks
// iterations [m K, min((m + 1) K, n)) from t = ckpt[m] and adds g_acc times
// each sample's trilinear weights to the density gradient.
__global__ void __launch_bounds__(128) adjoint_march_kernel(const __grid_constant__ RayConsts c,
                                                            const PixelTape* __restrict__ tape,
                                                            const float* __restrict__ ckpt, uint32_t K,
                                                            uint32_t nckpt, const float* __restrict__ g_acc,
                                                            float* __restrict__ g_dens)
{
    const uint64_t items = (uint64_t)c.W * c.H * nckpt;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < items; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t at = (uint32_t)(i / nckpt), m = (uint32_t)(i - (uint64_t)at * nckpt);
        const float g = g_acc[at];
        if (g == 0.0f) continue;
        const uint32_t n = tape[at].n;
        if ((uint64_t)m * K >= n) continue;
        Vec3 start, end;
        if (!ray_entry(c, (int)(at % (uint32_t)c.W), (int)(at / (uint32_t)c.W), start, end)) continue;
        const float step = 1.0f / c.steps;
        float t = ckpt[(size_t)at * nckpt + m];
        const uint32_t k1 = min(n, (m + 1) * K);
        for (uint32_t k = m * K; k < k1; ++k) {
            scatter_density(c, g_dens, mix(start, end, t), g);
            t += step;
        }
    }
}

// ---- trilinear-splat voxelizer ---------------------------------------------------------
// A continuous stand-in for the count voxelizer: each vertex adds its
// trilinear weights to the 8 texels around it, in the texel convention the
// raymarch samples with (u = (v - origin) / size * N - 0.5, texel centres
// at integers), so that splat and lookup are adjoint to each other.

struct SplatGrid {
    float tsc[3], tbias[3];
    int res[3];
};

__device__ __forceinline__ bool splat_setup(const SplatGrid& g, const float* __restrict__ v, uint32_t i, int i0[3],
                                            float a[3])
{
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float u = fmaf(__ldg(v + 3 * (size_t)i + k), g.tsc[k], g.tbias[k]);
        if (!(u > -1.0f && u < (float)g.res[k])) return false; // no tap inside the grid (or NaN)
        const float f = floorf(u);
        i0[k] = (int)f;
        a[k] = u - f;
    }
    return true;
}

__global__ void splat_kernel(SplatGrid g, const float* __restrict__ v, uint32_t n, float* __restrict__ dens)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int i0[3];
        float a[3];
        if (!splat_setup(g, v, i, i0, a)) continue;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
            const int x = i0[0] + dx, y = i0[1] + dy, z = i0[2] + dz;
            if (x < 0 || y < 0 || z < 0 || x >= g.res[0] || y >= g.res[1] || z >= g.res[2]) continue;
            const float w = (dx ? a[0] : 1.0f - a[0]) * (dy ? a[1] : 1.0f - a[1]) * (dz ? a[2] : 1.0f - a[2]);
            atomicAdd(dens + (size_t)x + (size_t)g.res[0] * ((size_t)y + (size_t)g.res[1] * z), w);
        }
    }
}

// d L / d vertex = sum over its 8 texels of g_texel * d w / d u * d u / d v.
__global__ void splat_adjoint_kernel(SplatGrid g, const float* __restrict__ v, uint32_t n,
                                     const float* __restrict__ g_dens, float* __restrict__ g_v)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int i0[3];
        float a[3];
        float gu[3] = {0.0f, 0.0f, 0.0f};
        if (splat_setup(g, v, i, i0, a)) {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
                const int x = i0[0] + dx, y = i0[1] + dy, z = i0[2] + dz;
                if (x < 0 || y < 0 || z < 0 || x >= g.res[0] || y >= g.res[1] || z >= g.res[2]) continue;
                const float gt = __ldg(g_dens + (size_t)x + (size_t)g.res[0] * ((size_t)y + (size_t)g.res[1] * z));
                const float wx = dx ? a[0] : 1.0f - a[0], wy = dy ? a[1] : 1.0f - a[1], wz = dz ? a[2] : 1.0f - a[2];
                gu[0] += gt * (dx ? 1.0f : -1.0f) * wy * wz;
                gu[1] += gt * wx * (dy ? 1.0f : -1.0f) * wz;
                gu[2] += gt * wx * wy * (dz ? 1.0f : -1.0f);
            }
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) g_v[3 * (size_t)i + k] = gu[k] * g.tsc[k];
    }
}

// Iterations of `for (float t = 0; t < 1; t += 1 / steps)` in FP32, as the
// device runs them (the checkpoint count depends on it).
uint32_t march_iterations(float steps)
{
    const float step = 1.0f / steps;
    uint32_t n = 0;
    for (volatile float t = 0.0f; t < 1.0f; t = t + step) ++n;
    return n;
}

uint32_t tape_checkpoints(const vkhr_raymarch_params* p, int32_t K)
{
    return (march_iterations(p->raycast_steps) + (uint32_t)K - 1) / (uint32_t)K + 1;
}

vkhr_status check_diff_params(vkhr_ctx* ctx, const vkhr_raymarch_params* p, int32_t K, RayConsts& c)
{
    if (!p) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "params is NULL");
    if (p->density_format != VKHR_DENSITY_F32 || p->tangent_format != VKHR_TANGENT_F32X4)
        return vkhr_fail(ctx, VKHR_ERR_NOT_SUPPORTED, "the differentiable raymarch takes F32 density and F32X4 tangents");
    if (K < 1 || K > 4096) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "checkpoint interval must be in [1, 4096]");
    return make_consts(ctx, p, c);
}

vkhr_status make_splat_grid(vkhr_ctx* ctx, const vkhr_aabb* b, int32_t w, int32_t h, int32_t d, SplatGrid& g)
{
    if (!b) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "bounds is NULL");
    if (w <= 0 || h <= 0 || d <= 0 || (uint64_t)w * h * d >= (1ull << 32))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "grid dimensions must be positive, < 2^32 voxels");
    const int r[3] = {w, h, d};
    for (int k = 0; k < 3; ++k) {
        if (!(b->size[k] > 0.0f) || !std::isfinite(b->size[k]))
            return vkhr_fail(ctx, VKHR_ERR_DEGENERATE_AABB, "every AABB extent must be finite and > 0");
        const double s = (double)r[k] / (double)b->size[k]; // as the raymarch's texel set-up
        g.tsc[k] = (float)s;
        g.tbias[k] = (float)(-(double)b->origin[k] * s - 0.5);
        g.res[k] = r[k];
    }
    return VKHR_OK;
}

} // namespace

extern "C" {

size_t vkhr_raymarch_tape_bytes(const vkhr_raymarch_params* params, int32_t checkpoint_interval)
{
    if (!params || params->width <= 0 || params->height <= 0 || checkpoint_interval < 1 ||
        !(params->raycast_steps > 0.0f) || !(params->raycast_steps <= 1048576.0f))
        return 0;
    const size_t px = (size_t)params->width * (size_t)params->height;
    return px * sizeof(PixelTape) + px * tape_checkpoints(params, checkpoint_interval) * sizeof(float);
}

vkhr_status vkhr_raymarch_train(vkhr_ctx* ctx, const vkhr_raymarch_params* params, const float* d_density,
                                const float* d_tangent, float* d_rgba, float* d_depth_out, void* d_tape,
                                size_t tape_bytes, int32_t checkpoint_interval, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    RayConsts c;
    vkhr_status s = check_diff_params(ctx, params, checkpoint_interval, c);
    if (s != VKHR_OK) return s;
    if (!d_density || !d_tangent || !d_rgba || !d_tape)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_density, d_tangent, d_rgba and d_tape are required");
    if ((reinterpret_cast<uintptr_t>(d_tangent) | reinterpret_cast<uintptr_t>(d_rgba) |
         reinterpret_cast<uintptr_t>(d_tape)) & 15u)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_tangent, d_rgba and d_tape must be 16-byte aligned");
    if (tape_bytes < vkhr_raymarch_tape_bytes(params, checkpoint_interval))
        return vkhr_fail(ctx, VKHR_ERR_CAPACITY, "tape smaller than vkhr_raymarch_tape_bytes()");
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t bricks = (size_t)c.nb[0] * c.nb[1] * c.nb[2], words = (bricks + 31) / 32;
    s = vkhr_reserve(ctx, (void**)&ctx->occ, &ctx->occ_cap, words, sizeof(uint32_t));
    if (s != VKHR_OK) return s;
    VKHR_CUDA_TRY(ctx, cudaMemsetAsync(ctx->occ, 0, words * sizeof(uint32_t), st));
    {
        const int L = occupancy_lanes(c.res[0], c.res[1], c.res[2], ctx->sm_count);
        const unsigned ob = occupancy_blocks(c.res[0], c.res[1], c.res[2], ctx->sm_count, L);
        if (L == 8)
            VKHR_LAUNCH(ctx, (occupancy_kernel<VKHR_DENSITY_F32, 8>), ob, 128, 0, st, d_density, c.res[0], c.res[1],
                        c.res[2], c.nb[0], c.nb[1], c.nb[2], ctx->occ);
        else
            VKHR_LAUNCH(ctx, (occupancy_kernel<VKHR_DENSITY_F32, 1>), ob, 128, 0, st, d_density, c.res[0], c.res[1],
                        c.res[2], c.nb[0], c.nb[1], c.nb[2], ctx->occ);
    }
    const size_t px = (size_t)c.W * c.H;
    const uint32_t nckpt = tape_checkpoints(params, checkpoint_interval);
    PixelTape* tape = reinterpret_cast<PixelTape*>(d_tape);
    float* ckpt = reinterpret_cast<float*>(tape + px);
    const dim3 block(32 * kWarpsX * kWarpsY);
    const dim3 grid((c.W + kTileW * kWarpsX - 1) / (kTileW * kWarpsX), (c.H + kTileH * kWarpsY - 1) / (kTileH * kWarpsY));
    VKHR_LAUNCH(ctx, (train_kernel<VKHR_DENSITY_F32, VKHR_TANGENT_F32X4>), grid, block, 0, st, c, d_density, d_tangent,
                ctx->occ, reinterpret_cast<float4*>(d_rgba), d_depth_out, tape, ckpt, (uint32_t)checkpoint_interval,
                nckpt);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    return VKHR_OK;
}

vkhr_status vkhr_raymarch_adjoint(vkhr_ctx* ctx, const vkhr_raymarch_params* params, const float* d_density,
                                  const float* d_tangent, const void* d_tape, int32_t checkpoint_interval,
                                  const float* d_grad_rgba, float* d_grad_density, float* d_grad_tangent,
                                  double* d_grad_params, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    RayConsts c;
    vkhr_status s = check_diff_params(ctx, params, checkpoint_interval, c);
    if (s != VKHR_OK) return s;
    if (!d_density || !d_tangent || !d_tape || !d_grad_rgba || !d_grad_density || !d_grad_tangent || !d_grad_params)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "every buffer of the adjoint is required");
    if ((reinterpret_cast<uintptr_t>(d_tangent) | reinterpret_cast<uintptr_t>(d_tape) |
         reinterpret_cast<uintptr_t>(d_grad_rgba) | reinterpret_cast<uintptr_t>(d_grad_tangent)) & 15u)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "tangent, tape and gradient buffers must be 16-byte aligned");
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t px = (size_t)c.W * c.H;
    const uint32_t nckpt = tape_checkpoints(params, checkpoint_interval);
    s = vkhr_reserve(ctx, (void**)&ctx->g_acc, &ctx->g_acc_cap, px, sizeof(float));
    if (s != VKHR_OK) return s;
    const PixelTape* tape = reinterpret_cast<const PixelTape*>(d_tape);
    const float* ckpt = reinterpret_cast<const float*>(tape + px);
    VKHR_LAUNCH(ctx, (adjoint_pixel_kernel<VKHR_DENSITY_F32, VKHR_TANGENT_F32X4>), vkhr_blocks(px, 128), 128, 0, st, c,
                d_density, reinterpret_cast<const float4*>(d_tangent), tape,
                reinterpret_cast<const float4*>(d_grad_rgba), ctx->g_acc, d_grad_density,
                reinterpret_cast<float4*>(d_grad_tangent), d_grad_params);
    const uint64_t items = (uint64_t)px * nckpt;
    VKHR_LAUNCH(ctx, adjoint_march_kernel, (unsigned)std::min<uint64_t>((items + 127) / 128, (uint64_t)ctx->sm_count * 64),
                128, 0, st, c, tape, ckpt, (uint32_t)checkpoint_interval, nckpt, ctx->g_acc, d_grad_density);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    return VKHR_OK;
}

vkhr_status vkhr_splat_vertices(vkhr_ctx* ctx, const float* d_vertices, uint32_t vertex_count, const vkhr_aabb* bounds,
                                int32_t width, int32_t height, int32_t depth, float* d_density, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    SplatGrid g;
    vkhr_status s = make_splat_grid(ctx, bounds, width, height, depth, g);
    if (s != VKHR_OK) return s;
    if (!d_density || (vertex_count && !d_vertices))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_vertices and d_density are required");
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    if (vertex_count)
        VKHR_LAUNCH(ctx, splat_kernel, std::min(vkhr_blocks(vertex_count, 256), (unsigned)ctx->sm_count * 16), 256, 0,
                    (cudaStream_t)stream, g, d_vertices, vertex_count, d_density);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    return VKHR_OK;
}

vkhr_status vkhr_splat_vertices_adjoint(vkhr_ctx* ctx, const float* d_vertices, uint32_t vertex_count,
                                        const vkhr_aabb* bounds, int32_t width, int32_t height, int32_t depth,
                                        const float* d_grad_density, float* d_grad_vertices, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    SplatGrid g;
    vkhr_status s = make_splat_grid(ctx, bounds, width, height, depth, g);
    if (s != VKHR_OK) return s;
    if (vertex_count && (!d_vertices || !d_grad_density || !d_grad_vertices))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_vertices, d_grad_density and d_grad_vertices are required");
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    if (vertex_count)
        VKHR_LAUNCH(ctx, splat_adjoint_kernel, std::min(vkhr_blocks(vertex_count, 256), (unsigned)ctx->sm_count * 16),
                    256, 0, (cudaStream_t)stream, g, d_vertices, vertex_count, d_grad_density, d_grad_vertices);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    return VKHR_OK;
}

} // extern "C"
