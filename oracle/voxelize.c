/*
 * voxelize.c -- CPU oracle (test infrastructure only) restating vkhr's strand
 * data preparation and voxelization, src/vkhr/scene_graph/hair_style.cc.
 *
 * Every FP32 operation follows the reference's operation order and glm's
 * component-wise semantics (glm::min(x, y) = y < x ? y : x, glm::max(x, y) =
 * x < y ? y : x, glm::normalize(v) = v * (1 / sqrt(dot(v, v))),
 * dot = (x*x + y*y) + z*z).  Build without fast-math and without FP
 * contraction so that the results are bit-identical to the reference.
 */
#include "vkhr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static inline float glm_min(float x, float y) { return (y < x) ? y : x; }
static inline float glm_max(float x, float y) { return (x < y) ? y : x; }

/* hair_style.cc:215-234 (generate_bounding_box) and :236-255 (get_bounding_box). */
void oracle_bounding_box(const float* v, uint32_t n, vkhr_aabb* out)
{
    float mn[3] = {0.0f, 0.0f, 0.0f}, mx[3] = {0.0f, 0.0f, 0.0f};
    for (uint32_t i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) {
            mn[c] = glm_min(v[3 * (size_t)i + c], mn[c]);
            mx[c] = glm_max(v[3 * (size_t)i + c], mx[c]);
        }
    }
    float size[3];
    for (int c = 0; c < 3; ++c) {
        out->origin[c] = mn[c];
        size[c] = mx[c] - mn[c];
        out->size[c] = size[c];
    }
    /* glm::length = sqrt(dot(size, size)) */
    float dot = (size[0] * size[0] + size[1] * size[1]) + size[2] * size[2];
    out->radius = sqrtf(dot);
    out->volume = (size[0] * size[1]) * size[2];
}

/* hair_style.cc:171-194. */
void oracle_generate_tangents(const float* v, const uint16_t* segments, uint32_t strand_count, float* t)
{
    size_t vertex = 0;
    size_t written = 0;
    for (uint32_t s = 0; s < strand_count; ++s) {
        for (unsigned seg = 0; seg < segments[s]; ++seg) {
            float d[3];
            for (int c = 0; c < 3; ++c) d[c] = v[3 * (vertex + 1) + c] - v[3 * vertex + c];
            float dot = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
            float inv = 1.0f / sqrtf(dot);
            for (int c = 0; c < 3; ++c) t[3 * written + c] = d[c] * inv;
            ++written;
            ++vertex;
        }
        /* tangents.push_back(tangents.back()): repeat the previous tangent. */
        for (int c = 0; c < 3; ++c) t[3 * written + c] = written ? t[3 * (written - 1) + c] : 0.0f;
        ++written;
        ++vertex;
    }
}

/* hair_style.cc:196-213. */
void oracle_generate_indices(const uint16_t* segments, uint32_t strand_count, uint32_t* idx)
{
    uint32_t vertex = 0;
    size_t k = 0;
    for (uint32_t s = 0; s < strand_count; ++s) {
        for (unsigned seg = 0; seg < segments[s]; ++seg) {
            idx[k++] = vertex++;
            idx[k++] = vertex;
        }
        ++vertex;
    }
}

typedef struct grid_t {
    int w, h, d;
    float res[3];
    float voxel_size[3];
    uint64_t n;
} grid_t;

static void grid_init(grid_t* g, const vkhr_aabb* b, int w, int h, int d)
{
    g->w = w; g->h = h; g->d = d;
    g->res[0] = (float)w; g->res[1] = (float)h; g->res[2] = (float)d;
    /* glm::vec3 voxel_size { volume.bounds.size / volume.resolution } */
    for (int c = 0; c < 3; ++c) g->voxel_size[c] = b->size[c] / g->res[c];
    g->n = (uint64_t)w * (uint64_t)h * (uint64_t)d;
}

/* Linear index of a clamped voxel coordinate; returns 0 and sets *out on
 * success, -1 when the visit falls outside the grid (dropped). */
static int voxel_index(const grid_t* g, const float vox[3], int mode, uint64_t* out)
{
    if (mode == VKHR_INDEX_REF_FP32) {
        /* voxel.x + voxel.y*width + voxel.z*width*height, all FP32
         * (hair_style.cc:276 and :321). */
        float fw = (float)g->w, fh = (float)g->h;
        float a = vox[1] * fw;
        float b = (vox[2] * fw) * fh;
        float fi = (vox[0] + a) + b;
        if (!(fi >= 0.0f) || !(fi < (float)g->n) || (uint64_t)fi >= g->n) return -1;
        *out = (uint64_t)fi;
        return 0;
    }
    for (int c = 0; c < 3; ++c)
        if (!(vox[c] >= 0.0f)) return -1;
    uint64_t x = (uint64_t)vox[0], y = (uint64_t)vox[1], z = (uint64_t)vox[2];
    *out = x + (uint64_t)g->w * (y + (uint64_t)g->h * z);
    return 0;
}

/* Tangent quantisation loop, hair_style.cc:285-291 / :333-339:
 * i8vec3(precise / float(density) * 127.0f), truncation toward zero.  An
 * empty voxel (0 / 0 in the reference) and a NaN sum give 0. */
static void quantize(const float* tsum, const uint8_t* dens, uint64_t n, int8_t* q)
{
    for (uint64_t i = 0; i < n; ++i) {
        float dd = (float)dens[i];
        for (int c = 0; c < 3; ++c) {
            int8_t r = 0;
            if (dens[i] != 0) {
                float x = (tsum[3 * i + c] / dd) * 127.0f;
                if (x == x) r = (int8_t)(int)x;
            }
            q[4 * i + c] = r;
        }
        q[4 * i + 3] = 0;
    }
}

static void visit(uint64_t pos, const float* tan, uint32_t* counts, uint8_t* dens, float* tsum)
{
    if (counts) counts[pos] += 1u;
    if (dens[pos] != 255) {
        tsum[3 * pos + 0] += tan[0];
        tsum[3 * pos + 1] += tan[1];
        tsum[3 * pos + 2] += tan[2];
        dens[pos] += 1;
    }
}

/* hair_style.cc:257-294. */
uint64_t oracle_voxelize_vertices(const float* v, const float* tangents, uint32_t n, const vkhr_aabb* b,
                                  int w, int h, int d, int mode, uint32_t* counts, uint8_t* densities,
                                  int8_t* tangents_q)
{
    grid_t g;
    grid_init(&g, b, w, h, d);
    uint8_t* dens = densities ? densities : (uint8_t*)malloc(g.n);
    float* tsum = (float*)calloc(3 * g.n, sizeof(float));
    memset(dens, 0, g.n);
    if (counts) memset(counts, 0, g.n * sizeof(uint32_t));
    uint64_t dropped = 0;
    static const float zero3[3] = {0.0f, 0.0f, 0.0f};
    for (uint32_t i = 0; i < n; ++i) {
        float vox[3];
        for (int c = 0; c < 3; ++c) vox[c] = (v[3 * (size_t)i + c] - b->origin[c]) / g.voxel_size[c];
        for (int c = 0; c < 3; ++c) vox[c] = glm_min(floorf(vox[c]), g.res[c] - 1.0f);
        uint64_t pos;
        if (voxel_index(&g, vox, mode, &pos)) { ++dropped; continue; }
        visit(pos, tangents ? tangents + 3 * (size_t)i : zero3, counts, dens, tsum);
    }
    if (tangents_q) quantize(tsum, dens, g.n, tangents_q);
    free(tsum);
    if (!densities) free(dens);
    return dropped;
}

/* The per-pair set-up of voxelize_segments, hair_style.cc:312-317. */
static float segment_setup(const grid_t* g, const float* v, const uint32_t* idx, uint64_t pair,
                           const vkhr_aabb* b, float root[3], float dir[3])
{
    float tip[3];
    for (int c = 0; c < 3; ++c) {
        root[c] = (v[3 * (size_t)idx[2 * pair] + c] - b->origin[c]) / g->voxel_size[c];
        tip[c] = (v[3 * (size_t)idx[2 * pair + 1] + c] - b->origin[c]) / g->voxel_size[c];
    }
    for (int c = 0; c < 3; ++c) dir[c] = tip[c] - root[c];
    /* glm::compMax(glm::abs(direction)) */
    float steps = glm_max(glm_max(fabsf(dir[0]), fabsf(dir[1])), fabsf(dir[2]));
    for (int c = 0; c < 3; ++c) dir[c] = dir[c] / steps;
    return steps;
}

uint32_t oracle_segment_visits(const float* v, const uint32_t* idx, uint64_t pair, const vkhr_aabb* b,
                               int w, int h, int d)
{
    grid_t g;
    grid_init(&g, b, w, h, d);
    float root[3], dir[3];
    float steps = segment_setup(&g, v, idx, pair, b, root, dir);
    uint32_t k = 0;
    while (steps-- > 0.0f) ++k;
    return k;
}

/* hair_style.cc:296-342. */
uint64_t oracle_voxelize_segments(const float* v, const float* tangents, const uint32_t* idx, uint64_t nidx,
                                  const vkhr_aabb* b, int w, int h, int d, int mode, uint32_t* counts,
                                  uint8_t* densities, int8_t* tangents_q)
{
    grid_t g;
    grid_init(&g, b, w, h, d);
    uint8_t* dens = densities ? densities : (uint8_t*)malloc(g.n);
    float* tsum = (float*)calloc(3 * g.n, sizeof(float));
    memset(dens, 0, g.n);
    if (counts) memset(counts, 0, g.n * sizeof(uint32_t));
    uint64_t dropped = 0;
    static const float zero3[3] = {0.0f, 0.0f, 0.0f};
    /* for (i = 0; i < indices.size() - 1; i += 2): floor(n / 2) pairs, none if empty. */
    uint64_t pairs = nidx / 2;
    for (uint64_t p = 0; p < pairs; ++p) {
        float root[3], dir[3];
        float steps = segment_setup(&g, v, idx, p, b, root, dir);
        const float* tan = tangents ? tangents + 3 * (size_t)idx[2 * p] : zero3;
        while (steps-- > 0.0f) {
            float vox[3];
            for (int c = 0; c < 3; ++c) vox[c] = glm_min(floorf(root[c]), g.res[c] - 1.0f);
            uint64_t pos;
            if (voxel_index(&g, vox, mode, &pos)) ++dropped;
            else visit(pos, tan, counts, dens, tsum);
            for (int c = 0; c < 3; ++c) root[c] = root[c] + dir[c];
        }
    }
    if (tangents_q) quantize(tsum, dens, g.n, tangents_q);
    free(tsum);
    if (!densities) free(dens);
    return dropped;
}

/* hair_style.cc:344-357. */
void oracle_normalize(uint8_t* dens, uint64_t n)
{
    uint8_t dmin = 255, dmax = 0;
    for (uint64_t i = 0; i < n; ++i) {
        if (dens[i] > dmax) dmax = dens[i];
        if (dens[i] < dmin) dmin = dens[i];
    }
    if (dmax == dmin) { /* 255 / 0: the reference's result is undefined; define 0 */
        memset(dens, 0, n);
        return;
    }
    float scaling = 255.0f / (float)(dmax - dmin);
    for (uint64_t i = 0; i < n; ++i) {
        uint8_t x = (uint8_t)(dens[i] - dmin);
        dens[i] = (uint8_t)(x * scaling);
    }
}

/* HairStyle::Volume::downsample (hair_style.hh:228-257) with the ABI's
 * filters: max, min, floor(sum / 8), min(sum, 255); even dimensions. */
void oracle_downsample(const uint8_t* in, int w, int h, int d, int filter, uint8_t* out)
{
    const int ow = w / 2, oh = h / 2, od = d / 2;
    for (int k = 0; k < od; ++k)
        for (int j = 0; j < oh; ++j)
            for (int i = 0; i < ow; ++i) {
                unsigned mx = 0, mn = 255, sum = 0;
                for (int z = 0; z < 2; ++z)
                    for (int y = 0; y < 2; ++y)
                        for (int x = 0; x < 2; ++x) {
                            const unsigned v = in[(size_t)(2 * i + x) + (size_t)(2 * j + y) * w +
                                                  (size_t)(2 * k + z) * w * h];
                            if (v > mx) mx = v;
                            if (v < mn) mn = v;
                            sum += v;
                        }
                unsigned r = filter == 0 ? mx : filter == 1 ? mn : filter == 2 ? sum / 8u : (sum < 255u ? sum : 255u);
                out[(size_t)i + (size_t)j * ow + (size_t)k * ow * oh] = (uint8_t)r;
            }
}
