/* resolve.c -- TEST INFRASTRUCTURE ONLY: the CPU oracle of the hybrid-LoD
 * compositing.  Only tests/, __graft_entry__.smoke() and the CPU baseline of
 * bench.py call it; the library never does.
 *
 * oracle_resolve_ppll restates the per-pixel linked-list resolve of the
 * reference, share/shaders/transparency/resolve.comp:15-101, over the node
 * layout of share/shaders/transparency/ppll.glsl:4-11 (12-byte nodes, NULL
 * 0xffffffff, empty k-buffer slots at depth 3e38).  oracle_composite is the
 * library's PPLL-free form of the same step: it builds, per pixel, the list a
 * PPLL holds when the strand fragments were linked in buffer order (strand.frag
 * :81-84) and the volume fragment after them (volume.frag:97-100 runs in the
 * subpass after the strands, rasterizer.cc:245-257), then resolves it the same
 * way.  Both are pinned against the reference's own resolve.comp, compiled as
 * C++ (oracle/ref_resolve.cc), by tests/test_oracle_composite.py.
 *
 * Arithmetic as GLSL defines it, in FP32 without contraction:
 *   unpackUnorm4x8 / imageLoad of rgba8: c / 255;
 *   mix(x, y, a) = x * (1 - a) + y * a;
 *   packUnorm4x8 / imageStore to rgba8: clamp to [0, 1], times 255, rounded
 *   to the nearest code (the specs leave ties to the implementation; this
 *   build takes ties to even). */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "vkhr_oracle.h"

enum { K_BUFFER = 16, MAX_TAIL = 1024, MAX_LIST = K_BUFFER + MAX_TAIL };
#define NULL_NODE 0xffffffffu

typedef struct {
    uint32_t color;
    float depth;
} frag;

static float unorm8(uint32_t c, int ch) { return (float)((c >> (8 * ch)) & 0xffu) / 255.0f; }

uint32_t oracle_pack_unorm8x4(const float v[4])
{
    uint32_t r = 0;
    for (int ch = 0; ch < 4; ++ch) {
        float x = v[ch];
        x = x > 0.0f ? (x < 1.0f ? x : 1.0f) : 0.0f;
        r |= (uint32_t)nearbyintf(x * 255.0f) << (8 * ch);
    }
    return r;
}

/* resolved = mix(resolved, c, c.a), resolve.comp:69-73 and :94-98. */
static void blend(float r[4], uint32_t c)
{
    const float a = unorm8(c, 3);
    const float t = 1.0f - a;
    for (int ch = 0; ch < 4; ++ch) r[ch] = r[ch] * t + unorm8(c, ch) * a;
}

/* First slot of the largest depth above 0 (slot 0 if none), resolve.comp:51-57. */
static int furthest(const frag* kb, float* depth)
{
    float fd = 0.0f;
    int fi = 0;
    for (int k = 0; k < K_BUFFER; ++k)
        if (kb[k].depth > fd) {
            fd = kb[k].depth;
            fi = k;
        }
    *depth = fd;
    return fi;
}

/* One invocation of resolve.comp over a list of n nodes in list order. */
static uint32_t resolve_list(const frag* list, uint32_t n, uint32_t background)
{
    frag kb[K_BUFFER];
    for (int k = 0; k < K_BUFFER; ++k) {
        kb[k].depth = (float)3.e+38; /* PPLL_MAXIMUM_DEPTH */
        kb[k].color = 0;
    }
    uint32_t next = 0;
    for (int k = 0; k < K_BUFFER; ++k)
        if (next < n) kb[k] = list[next++];
    float r[4];
    for (int ch = 0; ch < 4; ++ch) r[ch] = unorm8(background, ch);
    for (int f = 0; f < MAX_TAIL && next < n; ++f) {
        float fd;
        const int fi = furthest(kb, &fd);
        frag fr = list[next++];
        if (fr.depth < fd) {
            const frag t = kb[fi];
            kb[fi] = fr;
            fr = t;
        }
        blend(r, fr.color);
    }
    for (int k = 0; k < K_BUFFER; ++k) {
        float fd;
        const int fi = furthest(kb, &fd);
        kb[fi].depth = 0.0f;
        blend(r, kb[fi].color);
    }
    return oracle_pack_unorm8x4(r);
}

static frag node_at(const uint32_t* words, uint32_t i)
{
    frag f;
    f.color = words[3 * (size_t)i];
    memcpy(&f.depth, &words[3 * (size_t)i + 1], 4);
    return f;
}

int oracle_resolve_ppll(const uint32_t* heads, const uint32_t* nodes, uint32_t node_count, int width, int height,
                        uint32_t* color, int threads)
{
    int bad = 0;
    if (threads <= 0) threads = oracle_max_threads();
#pragma omp parallel for schedule(dynamic) num_threads(threads) reduction(| : bad)
    for (int y = 0; y < height; ++y) {
        frag list[MAX_LIST];
        for (int x = 0; x < width; ++x) {
            const size_t p = (size_t)y * (size_t)width + (size_t)x;
            uint32_t node = heads[p];
            if (node == NULL_NODE) continue;
            uint32_t n = 0;
            while (node != NULL_NODE && n < MAX_LIST) {
                if (node >= node_count) {
                    bad = 1;
                    break;
                }
                list[n++] = node_at(nodes, node);
                node = nodes[3 * (size_t)node + 2];
            }
            color[p] = resolve_list(list, n, color[p]);
        }
    }
    return bad ? -1 : 0;
}

int oracle_composite(const uint32_t* fragments, uint32_t fragment_count, const float* volume_rgba,
                     const float* volume_depth, int width, int height, uint32_t* color, int threads)
{
    const size_t npix = (size_t)width * (size_t)height;
    for (uint32_t i = 0; i < fragment_count; ++i)
        if (fragments[3 * (size_t)i + 2] >= npix) return -1;
    /* stable counting sort of the fragments by pixel: start[p] .. start[p+1] */
    uint32_t* start = (uint32_t*)calloc(npix + 1, sizeof(uint32_t));
    uint32_t* order = (uint32_t*)malloc(((size_t)fragment_count + 1) * sizeof(uint32_t));
    if (!start || !order) {
        free(start);
        free(order);
        return -2;
    }
    for (uint32_t i = 0; i < fragment_count; ++i) ++start[fragments[3 * (size_t)i + 2] + 1];
    for (size_t p = 0; p < npix; ++p) start[p + 1] += start[p];
    {
        uint32_t* cursor = (uint32_t*)malloc((npix + 1) * sizeof(uint32_t));
        if (!cursor) {
            free(start);
            free(order);
            return -2;
        }
        memcpy(cursor, start, (npix + 1) * sizeof(uint32_t));
        for (uint32_t i = 0; i < fragment_count; ++i) order[cursor[fragments[3 * (size_t)i + 2]]++] = i;
        free(cursor);
    }
    if (threads <= 0) threads = oracle_max_threads();
    const int has_volume = volume_rgba && volume_depth;
#pragma omp parallel for schedule(dynamic) num_threads(threads)
    for (int y = 0; y < height; ++y) {
        frag list[MAX_LIST];
        for (int x = 0; x < width; ++x) {
            const size_t p = (size_t)y * (size_t)width + (size_t)x;
            uint32_t n = 0;
            if (has_volume && volume_depth[p] < 1.0f) {
                list[0].color = oracle_pack_unorm8x4(volume_rgba + 4 * p);
                list[0].depth = volume_depth[p];
                n = 1;
            }
            /* the PPLL's head is the last fragment linked */
            for (uint32_t j = start[p + 1]; j > start[p] && n < MAX_LIST;) {
                --j;
                list[n++] = node_at(fragments, order[j]);
            }
            if (n) color[p] = resolve_list(list, n, color[p]);
        }
    }
    free(start);
    free(order);
    return 0;
}
