/*
 * oracle.c — CPU restatement of the uni_slam feature front-end.
 *
 * TEST INFRASTRUCTURE ONLY: this is the parity checker.  Only tests/, the
 * smoke check and the benchmark's CPU-baseline leg may load it.  Parity
 * status and sources are listed in oracle.h.
 *
 * Arithmetic: IEEE binary32, round-to-nearest-even, no contraction (built
 * with -ffp-contract=off), evaluation order exactly as written.  WGSL
 * `round` is half-to-even, so rintf() is used; `i32(f)` truncates.
 * Texture loads follow Tint's robustness clamp, min(u32(coord), dim - 1)
 * (vendor/dawn/src/tint/lang/core/ir/transform/robustness.cc:344-354), so a
 * negative coordinate reads the FAR edge.  Sampler reads use the Vulkan
 * clamp-to-edge bilinear formula with full f32 weights (canonical_bilinear).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../include/uslam_canon.h"

/* ---------------------------------------------------------------- dims -- */

void orc_level_dims(int W0, int H0, int levels, uint32_t* w_out, uint32_t* h_out) {
    /* wslam/src/common.cpp:41-45: factor = lod == 0 ? 1 : pow(1.2, lod) */
    for (int l = 0; l < levels; ++l) {
        const double factor = l == 0 ? 1.0 : pow(1.2, (double)l);
        w_out[l] = (uint32_t)((double)W0 / factor);
        h_out[l] = (uint32_t)((double)H0 / factor);
    }
}

/* ------------------------------------------------------------ sampling -- */

/* Tint robustness clamp for textureLoad: min(u32(c), n - 1). */
static inline uint32_t tint_clamp(int32_t c, uint32_t n) {
    const uint32_t u = (uint32_t)c;
    return u < n ? u : n - 1u;
}

/* Clamp-to-edge index for an integer-valued float (may be huge or negative). */
static inline uint32_t edge_index(float f, uint32_t n) {
    if (f <= 0.0f) return 0u;
    if (f >= (float)(n - 1u)) return n - 1u;
    return (uint32_t)f;
}

/* texel fetch callback: LOD0 from u8, other levels from f32 */
typedef struct {
    const uint8_t* u8;
    const float* f32;
    int pitch;
    uint32_t w, h;
} tex_t;

static inline float texel(const tex_t* t, uint32_t x, uint32_t y) {
    if (t->u8) return (float)t->u8[(size_t)y * (size_t)t->pitch + x] / 255.0f;
    return t->f32[(size_t)y * t->w + x];
}

/* Canonical bilinear sample S(tex, uv) with clamp-to-edge:
 *   u = uv.x*w - 0.5, i0 = floor(u), alpha = u - i0 (same for v)
 *   r = ((1-a)(1-b))T00 + (a(1-b))T10 + ((1-a)b)T01 + (ab)T11, left to right. */
static float canonical_bilinear(const tex_t* t, float uvx, float uvy) {
    const float u = uvx * (float)t->w - 0.5f;
    const float v = uvy * (float)t->h - 0.5f;
    const float fi = floorf(u);
    const float fj = floorf(v);
    const float a = u - fi;
    const float b = v - fj;
    const uint32_t i0 = edge_index(fi, t->w), i1 = edge_index(fi + 1.0f, t->w);
    const uint32_t j0 = edge_index(fj, t->h), j1 = edge_index(fj + 1.0f, t->h);
    const float t00 = texel(t, i0, j0), t10 = texel(t, i1, j0);
    const float t01 = texel(t, i0, j1), t11 = texel(t, i1, j1);
    const float na = 1.0f - a, nb = 1.0f - b;
    float r = (na * nb) * t00;
    r = r + (a * nb) * t10;
    r = r + (na * b) * t01;
    r = r + (a * b) * t11;
    return r;
}

/* ------------------------------------------------------------- pyramid -- */

void orc_pyramid_level(const uint8_t* img, int W0, int H0, int pitch, uint32_t w, uint32_t h,
                       int is_lod0, float* out) {
    const tex_t src = {img, NULL, pitch, (uint32_t)W0, (uint32_t)H0};
    for (uint32_t y = 0; y < h; ++y) {
        for (uint32_t x = 0; x < w; ++x) {
            float v;
            if (is_lod0) {
                /* data/src/provider_base.cpp:121-124: f32(u8) / 255 */
                v = (float)img[(size_t)y * (size_t)pitch + x] / 255.0f;
            } else {
                /* create_pyramid.wgsl:11-12: uv = (id + 0.5) / dst_size */
                const float uvx = ((float)x + 0.5f) / (float)w;
                const float uvy = ((float)y + 0.5f) / (float)h;
                v = canonical_bilinear(&src, uvx, uvy);
            }
            out[(size_t)y * w + x] = v;
        }
    }
}

/* -------------------------------------------------------------- detect -- */

static const int kCircleX[16] = {0, 1, 2, 3, 3, 3, 2, 1, 0, -1, -2, -3, -3, -3, -2, -1};
static const int kCircleY[16] = {-3, -3, -2, -1, 0, 1, 2, 3, 3, 3, 2, 1, 0, -1, -2, -3};

void orc_detect(const float* lvl, uint32_t w, uint32_t h, uint32_t* resp) {
    /* detect_corners.wgsl:58-81 */
    for (uint32_t y = 0; y < h; ++y) {
        for (uint32_t x = 0; x < w; ++x) {
            uint32_t curr = 1, streak = 1;
            const float center = lvl[(size_t)y * w + x];
            for (int i = 0; i < 16; ++i) {
                const uint32_t cx = tint_clamp((int32_t)x + kCircleX[i], w);
                const uint32_t cy = tint_clamp((int32_t)y + kCircleY[i], h);
                const float counter = lvl[(size_t)cy * w + cx];
                const int is_different = fabsf(center - counter) > 0.15f;
                curr = is_different ? curr + 1u : 1u;
                streak = curr > streak ? curr : streak;
            }
            resp[(size_t)y * w + x] = streak > 9u ? streak : 0u;
        }
    }
}

/* ---------------------------------------------------------------- cull -- */

static uint32_t ceil_div(uint32_t n, uint32_t d) { return (n + d - 1u) / d; }

void orc_cull(const uint32_t* S, uint32_t w, uint32_t h, int W0, int H0, uint32_t* out) {
    const uint32_t region = 3u;          /* REGION_SIZE (cull_corners.wgsl:19) */
    const uint32_t wg = 64u;             /* kWgSize (cull_corners.cpp:20) */
    const uint32_t blk = (uint32_t)W0 * (uint32_t)H0; /* CORNER_BLOCK_SZ (cull_corners.cpp:29-31) */
    /* dispatch sizes (cull_corners.cpp:332-353) times the workgroup size */
    const uint32_t gx_h = ceil_div(ceil_div((uint32_t)W0, region), wg) * wg;
    const uint32_t gy_h = (uint32_t)H0;
    const uint32_t gx_v = ceil_div((uint32_t)W0, wg) * wg;
    const uint32_t gy_v = ceil_div((uint32_t)H0, region);
    const uint32_t n = w * h;
    const size_t cap = (size_t)blk + 4u * (size_t)w + 16u;
    uint32_t* H = (uint32_t*)calloc(cap, sizeof(uint32_t));
    uint32_t* V = (uint32_t*)calloc(cap, sizeof(uint32_t));

    /* main_horizontal (cull_corners.wgsl:22-57) */
    for (uint32_t y = 0; y < gy_h; ++y) {
        for (uint32_t gx = 0; gx < gx_h; ++gx) {
            const uint32_t xr = gx * region;
            const uint32_t start = xr * region + y * w;
            const uint32_t end = start + region < w ? start + region : w;
            if (start >= n) continue;
            uint32_t max_idx = start;
            int found = S[start] > 0u;
            for (uint32_t q = start; q < end; ++q) {
                if (S[q] > S[max_idx]) {
                    max_idx = q;
                    found = 1;
                }
                H[q] = 0u;
            }
            if (found) H[max_idx] = S[max_idx];
        }
    }
    /* main_vertical (cull_corners.wgsl:60-109) */
    for (uint32_t gy = 0; gy < gy_v; ++gy) {
        for (uint32_t gx = 0; gx < gx_v; ++gx) {
            const uint32_t start = gx * region + gy * region * w;
            if (start >= n) continue;
            const uint32_t left = blk - start;
            uint32_t steps = left / w;
            if (steps > region) steps = region;
            const uint32_t end = start + w * steps;
            uint32_t max_idx = start;
            int found = H[start] > 0u;
            for (uint32_t i = start; i < end; i += w) {
                if (H[i] > H[max_idx]) {
                    max_idx = i;
                    found = 1;
                }
                V[i] = H[i];
            }
            if (found) V[max_idx] = H[max_idx];
        }
    }
    memcpy(out, V, (size_t)n * sizeof(uint32_t));
    free(H);
    free(V);
}

/* ------------------------------------------------------------ describe -- */

float orc_gauss_tap9(const float* lvl, uint32_t w, uint32_t h, uint32_t px, uint32_t py) {
    /* generate_features.wgsl:149-172 */
    const tex_t t = {NULL, lvl, 0, w, h};
    const float tx = 1.0f / (float)w;
    const float ty = 1.0f / (float)h;
    const float uvx = ((float)px + 0.5f) * tx;
    const float uvy = ((float)py + 0.5f) * ty;
    static const float off[3] = {-1.2f, 0.0f, 1.2f};
    static const float wt[3] = {0.3125f, 0.375f, 0.3125f};
    float sum = 0.0f;
    for (int j = 0; j < 3; ++j) {
        for (int i = 0; i < 3; ++i) {
            const float ox = off[i] * tx;
            const float oy = off[j] * ty;
            const float s = canonical_bilinear(&t, uvx + ox, uvy + oy);
            sum = sum + (s * wt[i]) * wt[j];
        }
    }
    return sum;
}

void orc_blur_level(const float* lvl, uint32_t w, uint32_t h, float* out) {
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) out[(size_t)y * w + x] = orc_gauss_tap9(lvl, w, h, x, y);
}

void orc_describe(const float* lvl, uint32_t w, uint32_t h, int x, int y, const int32_t* pattern,
                  float* theta_out, uint32_t desc_out[8]) {
    /* getOrientation, generate_features.wgsl:80-99 (r = 3, dy outer, dx inner) */
    float m10 = 0.0f, m01 = 0.0f;
    for (int dy = -3; dy <= 3; ++dy) {
        for (int dx = -3; dx <= 3; ++dx) {
            if (dx * dx + dy * dy > 9) continue;
            const uint32_t cx = tint_clamp(x + dx, w);
            const uint32_t cy = tint_clamp(y + dy, h);
            const float p = lvl[(size_t)cy * w + cx];
            m10 = m10 + (float)dx * p;
            m01 = m01 + (float)dy * p;
        }
    }
    const float theta = uslam_atan2f(m01, m10);
    /* computeDescriptor, generate_features.wgsl:101-137 */
    float s, c;
    uslam_sincosf(theta, &s, &c);
    uint32_t desc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 256; ++i) {
        const float ax = (float)pattern[4 * i + 0], ay = (float)pattern[4 * i + 1];
        const float bx = (float)pattern[4 * i + 2], by = (float)pattern[4 * i + 3];
        const int32_t rax = (int32_t)rintf(ax * c - ay * s);
        const int32_t ray = (int32_t)rintf(ax * s + ay * c);
        const int32_t rbx = (int32_t)rintf(bx * c - by * s);
        const int32_t rby = (int32_t)rintf(bx * s + by * c);
        const float ga = orc_gauss_tap9(lvl, w, h, (uint32_t)(x + rax), (uint32_t)(y + ray));
        const float gb = orc_gauss_tap9(lvl, w, h, (uint32_t)(x + rbx), (uint32_t)(y + rby));
        if (ga > gb) desc[i / 32] |= 1u << (i % 32);
    }
    *theta_out = theta;
    memcpy(desc_out, desc, sizeof(desc));
}

/* --------------------------------------------------------------- frame -- */

/* ---------------------------------------------------- cfg detector -- */
/* The benchmark's `cfg` detection profile (no counterpart in the reference,
 * pinned by this definition): FAST 9-of-16 with wrap-around on the level's
 * f32 pixels, threshold T = 20/255 (brighter iff p - c > T, darker iff
 * c - p > T), circle of resources/detect_corners.wgsl:31-32; pixels within 3
 * of a level edge are never corners; score = sum over the qualifying
 * polarity's points, in circle order, of (|p - c| - T); 3x3 non-maximum
 * suppression on the score, a tie going to the first pixel in raster order;
 * strength = the longest circular arc (9..16). */
static const int circ_x[16] = {0, 1, 2, 3, 3, 3, 2, 1, 0, -1, -2, -3, -3, -3, -2, -1};
static const int circ_y[16] = {-3, -3, -2, -1, 0, 1, 2, 3, 3, 3, 2, 1, 0, -1, -2, -3};

static uint32_t circ_run(uint32_t m) {
    if (m == 0xffffu) return 16u;
    uint32_t x = m | (m << 16), run = 0;
    while (x) {
        x &= x << 1;
        ++run;
    }
    return run;
}

void orc_detect_cfg(const float* lvl, uint32_t w, uint32_t h, uint32_t* out) {
    const float T = 20.0f / 255.0f;
    const size_t n = (size_t)w * h;
    float* score = (float*)calloc(n, sizeof(float));
    uint32_t* arc = (uint32_t*)calloc(n, sizeof(uint32_t));
    for (uint32_t y = 3; y + 3 < h; ++y)
        for (uint32_t x = 3; x + 3 < w; ++x) {
            const float c = lvl[(size_t)y * w + x];
            uint32_t mb = 0, md = 0;
            for (int i = 0; i < 16; ++i) {
                const float p = lvl[(size_t)(y + circ_y[i]) * w + (x + circ_x[i])];
                if (p - c > T) mb |= 1u << i;
                if (c - p > T) md |= 1u << i;
            }
            const uint32_t rb = circ_run(mb), rd = circ_run(md);
            if (rb < 9u && rd < 9u) continue;
            const int bright = rb >= 9u;
            const uint32_t m = bright ? mb : md;
            float sc = 0.0f;
            for (int i = 0; i < 16; ++i) {
                if (!((m >> i) & 1u)) continue;
                const float p = lvl[(size_t)(y + circ_y[i]) * w + (x + circ_x[i])];
                sc = sc + ((bright ? p - c : c - p) - T);
            }
            score[(size_t)y * w + x] = sc;
            arc[(size_t)y * w + x] = bright ? rb : rd;
        }
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) {
            const size_t p = (size_t)y * w + x;
            uint32_t keep = arc[p];
            for (int dy = -1; dy <= 1 && keep; ++dy)
                for (int dx = -1; dx <= 1 && keep; ++dx) {
                    if (dy == 0 && dx == 0) continue;
                    const long qy = (long)y + dy, qx = (long)x + dx;
                    if (qy < 0 || qx < 0 || qy >= (long)h || qx >= (long)w) continue;
                    const float q = score[(size_t)qy * w + (size_t)qx];
                    const int earlier = dy < 0 || (dy == 0 && dx < 0);
                    if (earlier ? !(score[p] > q) : !(score[p] >= q)) keep = 0;
                }
            out[p] = keep;
        }
    free(score);
    free(arc);
}

/* Keep one keypoint: header plus descriptor; returns 0 if feats is full. */
static int emit(const float* lvl, uint32_t w, uint32_t h, int x, int y, uint32_t strength, const int32_t* pattern,
                orc_feature* feats, int max_feats, int* total) {
    if (*total >= max_feats) return 0;
    orc_feature* f = &feats[*total];
    f->x = (float)x;
    f->y = (float)y;
    f->strength = strength;
    orc_describe(lvl, w, h, x, y, pattern, &f->orientation, f->descriptor);
    ++*total;
    return 1;
}

int orc_frame_fc(const uint8_t* img, int W0, int H0, int pitch, int levels, int cap, int cell_cap, int detector,
                 int frame_cap, const int32_t* pattern, orc_feature* feats, int max_feats, int* kept, int* raw) {
    uint32_t ws[32], hs[32];
    orc_level_dims(W0, H0, levels, ws, hs);
    int total = 0, ok = 1;
    const int level_cap = cap;
    for (int l = 0; l < levels && ok; ++l) {
        const uint32_t w = ws[l], h = hs[l];
        /* per-frame cap: the levels are filled in order, each level keeping at
         * most what the earlier levels left of frame_cap */
        cap = level_cap;
        if (frame_cap > 0 && frame_cap - total < cap) cap = frame_cap - total > 0 ? frame_cap - total : 0;
        const size_t n = (size_t)w * h;
        float* lvl = (float*)malloc(n * sizeof(float));
        uint32_t* resp = (uint32_t*)malloc(n * sizeof(uint32_t));
        uint32_t* culled = (uint32_t*)malloc(n * sizeof(uint32_t));
        orc_pyramid_level(img, W0, H0, pitch, w, h, l == 0, lvl);
        if (detector == 1) {
            orc_detect_cfg(lvl, w, h, culled);
        } else {
            orc_detect(lvl, w, h, resp);
            orc_cull(resp, w, h, W0, H0, culled);
        }
        int nraw = 0, nkept = 0;
        for (size_t p = 0; p < n; ++p) nraw += culled[p] != 0u;
        if (cell_cap <= 0) {
            /* canonical order (y, x); keep the first `cap` (the reference's
             * atomic append order is nondeterministic, generate_features.wgsl:67-70) */
            for (size_t p = 0; p < n && ok && nkept < cap; ++p) {
                if (culled[p] == 0u) continue;
                ok = emit(lvl, w, h, (int)(p % w), (int)(p / w), culled[p], pattern, feats, max_feats, &total);
                nkept += ok;
            }
        } else {
            /* per-cell caps: 32x32 cells in row-major order, (y, x) within a
             * cell, the first cell_cap of each cell, then the level cap */
            for (uint32_t cy = 0; cy * 32u < h && ok; ++cy)
                for (uint32_t cx = 0; cx * 32u < w && ok; ++cx) {
                    int in_cell = 0;
                    for (uint32_t y = cy * 32u; y < cy * 32u + 32u && y < h && ok; ++y)
                        for (uint32_t x = cx * 32u; x < cx * 32u + 32u && x < w && ok; ++x) {
                            const uint32_t s = culled[(size_t)y * w + x];
                            if (s == 0u) continue;
                            if (in_cell < cell_cap && nkept < cap) {
                                ok = emit(lvl, w, h, (int)x, (int)y, s, pattern, feats, max_feats, &total);
                                nkept += ok;
                            }
                            ++in_cell;
                        }
                }
        }
        kept[l] = nkept;
        raw[l] = nraw;
        free(lvl);
        free(resp);
        free(culled);
    }
    return ok ? total : -1;
}

int orc_frame_ex(const uint8_t* img, int W0, int H0, int pitch, int levels, int cap, int cell_cap, int detector,
                 const int32_t* pattern, orc_feature* feats, int max_feats, int* kept, int* raw) {
    return orc_frame_fc(img, W0, H0, pitch, levels, cap, cell_cap, detector, 0, pattern, feats, max_feats, kept, raw);
}

int orc_frame(const uint8_t* img, int W0, int H0, int pitch, int levels, int cap,
              const int32_t* pattern, orc_feature* feats, int max_feats, int* kept, int* raw) {
    return orc_frame_ex(img, W0, H0, pitch, levels, cap, 0, 0, pattern, feats, max_feats, kept, raw);
}

/* --------------------------------------------------------------- match -- */

typedef struct {
    const orc_feature* f;
    uint32_t lod;
    int idx; /* index within its level */
    float px, py;
} cand_t;

static void to_lod0(const orc_feature* f, uint32_t lod, float* px, float* py) {
    /* match_features_cpu.cpp:58-64: f32 scale iterated lod times */
    float scale = 1.0f;
    for (uint32_t i = 0; i < lod; ++i) scale *= (float)1.2;
    *px = (float)(uint32_t)f->x * scale;
    *py = (float)(uint32_t)f->y * scale;
}

static int cmp_cand_x(const void* a, const void* b) {
    const float xa = ((const cand_t*)a)->px, xb = ((const cand_t*)b)->px;
    return (xa > xb) - (xa < xb);
}

static uint32_t hamming(const uint32_t* a, const uint32_t* b) {
    uint32_t d = 0;
    for (int k = 0; k < 8; ++k) d += (uint32_t)__builtin_popcount(a[k] ^ b[k]);
    return d;
}

/* FindMatchesInLod (match_features_cpu.cpp:66-150).  Queries are level `lod`
 * of q; the pool is levels lod, lod-1, lod+1 of p.  match_out[i] receives the
 * pool candidate index (into pool) or -1. */
static void find_in_lod(const orc_feature* q, int nq, uint32_t lod, const cand_t* pool_sorted,
                        int npool, float max_dx, float max_dy, int* match_out) {
    for (int i = 0; i < nq; ++i) match_out[i] = -1;
    if (npool < 2) return;
    for (int i = 0; i < nq; ++i) {
        float cx, cy;
        to_lod0(&q[i], lod, &cx, &cy);
        uint32_t best = 0xffffffffu, second = 0xffffffffu;
        int best_idx = -1;
        const float lo = cx - max_dx, hi = cx + max_dx;
        /* lower_bound on x */
        int first = 0, count = npool;
        while (count > 0) {
            const int step = count / 2;
            if (pool_sorted[first + step].px < lo) {
                first += step + 1;
                count -= step + 1;
            } else {
                count = step;
            }
        }
        for (int k = first; k < npool; ++k) {
            const cand_t* c = &pool_sorted[k];
            if (c->px > hi) break;
            if (fabsf(cy - c->py) > max_dy) continue;
            const uint32_t d = hamming(q[i].descriptor, c->f->descriptor);
            if (d < best) {
                second = best;
                best = d;
                best_idx = k;
            } else if (d < second) {
                second = d;
            }
        }
        if (best_idx >= 0 && (float)best < 0.85f * (float)second) match_out[i] = best_idx;
    }
}

/* Build the sorted pool (levels lod, lod-1, lod+1) of a feature set. */
static int build_pool(const orc_feature* f, const int* off, int levels, int lod, cand_t* pool) {
    int n = 0;
    const int order[3] = {lod, lod - 1, lod + 1};
    for (int k = 0; k < 3; ++k) {
        const int l = order[k];
        if (l < 0 || l >= levels) continue;
        for (int i = off[l]; i < off[l + 1]; ++i) {
            pool[n].f = &f[i];
            pool[n].lod = (uint32_t)l;
            pool[n].idx = i - off[l];
            to_lod0(&f[i], (uint32_t)l, &pool[n].px, &pool[n].py);
            ++n;
        }
    }
    qsort(pool, (size_t)n, sizeof(cand_t), cmp_cand_x);
    return n;
}

int orc_match(const orc_feature* a, const int* a_off, const orc_feature* b, const int* b_off,
              int levels, int W0, int H0, int32_t* out, int max_out) {
    /* match_features_cpu.cpp:76-77 */
    const float max_dx = 0.1f * (float)(uint32_t)W0;
    const float max_dy = 0.1f * (float)(uint32_t)H0;
    const int na = a_off[levels], nb = b_off[levels];
    cand_t* pool = (cand_t*)malloc(sizeof(cand_t) * (size_t)(na > nb ? na : nb) + sizeof(cand_t));
    /* b_to_a: for each b (global index), the matched a as (lod, idx) packed, or -1 */
    int* b_to_a = (int*)malloc(sizeof(int) * (size_t)(nb + 1));
    int* tmp = (int*)malloc(sizeof(int) * (size_t)((na > nb ? na : nb) + 1));
    for (int i = 0; i < nb; ++i) b_to_a[i] = -1;
    /* direction 1 (match_features_cpu.cpp:188-194): queries b level l, pool adj(a, l) */
    for (int l = 0; l < levels; ++l) {
        const int np = build_pool(a, a_off, levels, l, pool);
        const int nq = b_off[l + 1] - b_off[l];
        find_in_lod(&b[b_off[l]], nq, (uint32_t)l, pool, np, max_dx, max_dy, tmp);
        for (int i = 0; i < nq; ++i) {
            if (tmp[i] < 0) continue;
            const cand_t* c = &pool[tmp[i]];
            b_to_a[b_off[l] + i] = a_off[c->lod] + c->idx;
        }
    }
    /* direction 2 + mutual check (match_features_cpu.cpp:196-205) */
    int n = 0;
    for (int l = 0; l < levels; ++l) {
        const int np = build_pool(b, b_off, levels, l, pool);
        const int nq = a_off[l + 1] - a_off[l];
        find_in_lod(&a[a_off[l]], nq, (uint32_t)l, pool, np, max_dx, max_dy, tmp);
        for (int i = 0; i < nq; ++i) {
            if (tmp[i] < 0) continue;
            const cand_t* c = &pool[tmp[i]];
            const int gb = b_off[c->lod] + c->idx;
            if (b_to_a[gb] != a_off[l] + i) continue;
            if (n >= max_out) {
                n = -1;
                goto done;
            }
            out[4 * n + 0] = l;
            out[4 * n + 1] = i;
            out[4 * n + 2] = (int32_t)c->lod;
            out[4 * n + 3] = c->idx;
            ++n;
        }
    }
done:
    free(pool);
    free(b_to_a);
    free(tmp);
    return n;
}

/* ------------------------------------------------------ brute force -- */

int orc_match_bruteforce(const orc_feature* a, int na, const orc_feature* b, int nb, float ratio, int32_t* a2b) {
    int n = 0;
    for (int i = 0; i < na; ++i) {
        uint32_t best = UINT32_MAX, second = UINT32_MAX;
        int idx = -1;
        if (nb >= 2) {
            for (int j = 0; j < nb; ++j) {
                uint32_t d = 0;
                for (int w = 0; w < 8; ++w) d += (uint32_t)__builtin_popcount(a[i].descriptor[w] ^ b[j].descriptor[w]);
                if (d < best) {
                    second = best;
                    best = d;
                    idx = j;
                } else if (d < second) {
                    second = d;
                }
            }
        }
        a2b[i] = (idx >= 0 && (float)best < ratio * (float)second) ? idx : -1;
        n += a2b[i] >= 0;
    }
    return n;
}

/* ----------------------------------------------------- RANSAC scoring -- */
/* Sampson distance of wslam/src/pose_estimate_cpu/ransac_cpu.cpp:183-196 in
 * double, in the evaluation order written in the CUDA file (left to right,
 * no contraction); inlier iff d < threshold (ClassifyInliers, :198-210). */
static int sampson_inlier(const double* F, double xp, double yp, double xc, double yc, double thr) {
    const double fx0 = (F[0] * xp + F[1] * yp) + F[2];
    const double fx1 = (F[3] * xp + F[4] * yp) + F[5];
    const double fx2 = (F[6] * xp + F[7] * yp) + F[8];
    const double ft0 = (F[0] * xc + F[3] * yc) + F[6];
    const double ft1 = (F[1] * xc + F[4] * yc) + F[7];
    const double num = (xc * fx0 + yc * fx1) + fx2;
    const double den = ((fx0 * fx0 + fx1 * fx1) + ft0 * ft0) + ft1 * ft1;
    if (den < 1e-12) return 0;
    return (num * num) / den < thr;
}

void orc_sampson_counts(const double* fmats, int n_hyp, const double* prev_xy, const double* curr_xy, int n,
                        double thr, int* counts, uint32_t* masks) {
    const int words = (n + 31) / 32;
    for (int h = 0; h < n_hyp; ++h) {
        int c = 0;
        for (int w = 0; masks && w < words; ++w) masks[(size_t)h * words + w] = 0u;
        for (int i = 0; i < n; ++i) {
            const int in = sampson_inlier(fmats + (size_t)h * 9, prev_xy[2 * i], prev_xy[2 * i + 1], curr_xy[2 * i],
                                          curr_xy[2 * i + 1], thr);
            c += in;
            if (in && masks) masks[(size_t)h * words + i / 32] |= 1u << (i % 32);
        }
        counts[h] = c;
    }
}

/* ------------------------------------------------------------ exports -- */

float orc_atan2f(float y, float x) { return uslam_atan2f(y, x); }

void orc_sincosf(float a, float* s, float* c) { uslam_sincosf(a, s, c); }
