/*
 * oracle.h — CPU restatement of the uni_slam feature front-end (TEST
 * INFRASTRUCTURE ONLY).
 *
 * This library is the parity checker for the CUDA path.  Only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it;
 * the product library never links or calls it.
 *
 * Parity status:
 *  - Matcher (orc_match): PINNED.  It is checked against the reference's own
 *    wslam/src/pose_estimate_cpu/match_features_cpu.cpp, compiled unmodified
 *    with shim headers (oracle/Makefile, oracle/ref_harness.cpp), on random
 *    feature sets, and against golden vectors made from that build.
 *  - cfg detection profile (orc_detect_cfg) and the brute-force matcher
 *    (orc_match_bruteforce): defined here, no reference counterpart; pinned
 *    by numpy statements of the same definitions in the tests.
 *  - Pyramid / detect / cull / describe: PARITY UNPINNED.  They restate the
 *    WGSL shaders (resources/*.wgsl) line by line, but the reference cannot
 *    execute them anywhere (Dawn is not built, and there is no graphics stack)
 *    and the reference ships no golden vectors for them.  Implementation-
 *    defined WGSL arithmetic is fixed by include/uslam_canon.h and by the
 *    canonical f32 bilinear formula written out in oracle.c.
 */
#ifndef USLAM_ORACLE_H
#define USLAM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same layout as the reference's gpumodels::Feature (wslam/src/models.hpp:31-69). */
typedef struct orc_feature {
    float x;
    float y;
    uint32_t strength;
    float orientation;
    uint32_t descriptor[8];
} orc_feature;

/* Level dimensions: w_l = (uint32)(W0 / pow(1.2, l)) (wslam/src/common.cpp:41-45). */
void orc_level_dims(int W0, int H0, int levels, uint32_t* w_out, uint32_t* h_out);

/* One pyramid level as f32: level 0 is u8/255 (data/src/provider_base.cpp:121-124);
 * level l >= 1 is one bilinear tap of LOD0 (resources/create_pyramid.wgsl:5-14). */
void orc_pyramid_level(const uint8_t* img, int W0, int H0, int pitch, uint32_t w, uint32_t h,
                       int is_lod0, float* out);

/* FAST-style response map (resources/detect_corners.wgsl:35-89). */
void orc_detect(const float* lvl, uint32_t w, uint32_t h, uint32_t* resp);

/* Literal simulation of the horizontal and vertical cull dispatches
 * (resources/cull_corners.wgsl:22-109, wslam/src/feature_detect/cull_corners.cpp:332-353).
 * out[p] for p < w*h is the culled strength (0 = not a keypoint). */
void orc_cull(const uint32_t* resp, uint32_t w, uint32_t h, int W0, int H0, uint32_t* out);

/* G(x, y) for every pixel of a level (the blur cache the kernels precompute). */
void orc_blur_level(const float* lvl, uint32_t w, uint32_t h, float* out);

/* Orientation + 256-bit descriptor of one keypoint
 * (resources/generate_features.wgsl:80-172). */
void orc_describe(const float* lvl, uint32_t w, uint32_t h, int x, int y, const int32_t* pattern,
                  float* theta_out, uint32_t desc_out[8]);

/* Blurred sample G(P) of generate_features.wgsl:149-172 for an integer point. */
float orc_gauss_tap9(const float* lvl, uint32_t w, uint32_t h, uint32_t px, uint32_t py);

/* Whole frame: pyramid, detect, cull, describe, per-level cap keeping the
 * first `cap` keypoints in (y, x) order.  feats receives the kept features
 * level by level; kept[l] and raw[l] receive per-level counts.  Returns the
 * total number of kept features, or -1 if max_feats is too small. */
int orc_frame(const uint8_t* img, int W0, int H0, int pitch, int levels, int cap,
              const int32_t* pattern, orc_feature* feats, int max_feats, int* kept, int* raw);
/* As orc_frame; cell_cap > 0 selects per-cell caps: each level is cut into
 * 32x32 cells from its origin, cells visited in row-major order and pixels
 * within a cell in (y, x) order; the first cell_cap keypoints of each cell
 * are kept, and the level cap keeps the first `cap` of that sequence. */
int orc_frame_ex(const uint8_t* img, int W0, int H0, int pitch, int levels, int cap, int cell_cap, int detector,
                 const int32_t* pattern, orc_feature* feats, int max_feats, int* kept, int* raw);
/* As orc_frame_ex with a per-frame cap (no reference counterpart; the
 * reference caps per level only, common.hpp:47): frame_cap > 0 fills the
 * levels in order, level l keeping the first min(cap, frame_cap - features
 * kept by levels 0..l-1) of its order, so the frame keeps the first
 * frame_cap features in (level, y, x) order (or (level, cell, y, x) order
 * with cell caps).  frame_cap = 0: no per-frame cap. */
int orc_frame_fc(const uint8_t* img, int W0, int H0, int pitch, int levels, int cap, int cell_cap, int detector,
                 int frame_cap, const int32_t* pattern, orc_feature* feats, int max_feats, int* kept, int* raw);
/* The `cfg` detection profile on one level (detector = 1 of orc_frame_ex):
 * FAST 9-of-16 with wrap-around at 20/255, score = sum of (|p - c| - 20/255)
 * over the qualifying points, 3x3 NMS (ties to the first pixel in raster
 * order), pixels within 3 of the edge excluded.  out[p] = arc length (9..16)
 * of a surviving corner, else 0.  No reference counterpart. */
void orc_detect_cfg(const float* lvl, uint32_t w, uint32_t h, uint32_t* out);

/* Matcher restated from wslam/src/pose_estimate_cpu/match_features_cpu.cpp:27-207.
 * a = previous (reference) set, b = current set; a_off/b_off hold levels+1
 * offsets into the feature arrays.  W0, H0 set the spatial window
 * (0.1*W0, 0.1*H0).  out receives 4 ints per match
 * (lod_a, idx_a, lod_b, idx_b), sorted by (lod_a, idx_a); returns the match
 * count or -1 if max_out is too small. */
int orc_match(const orc_feature* a, const int* a_off, const orc_feature* b, const int* b_off,
              int levels, int W0, int H0, int32_t* out, int max_out);

/* Brute-force top-2 matcher (the benchmark's stress matcher; the reference
 * has no such mode, so this is pinned by its own definition only): every
 * feature of a (na, all levels flattened) against every feature of b (nb);
 * per query the best and second-best Hamming distances (scan rule of
 * match_features_cpu.cpp:108-140, from UINT32_MAX), accepted iff
 * f32(best) < ratio * f32(second); no window, no cross-check; nb < 2 gives no
 * match (match_features_cpu.cpp:80-82).  a2b[i] receives the flat index into
 * b of query i's match, or -1.  Returns the number of matches. */
int orc_match_bruteforce(const orc_feature* a, int na, const orc_feature* b, int nb, float ratio, int32_t* a2b);

/* RANSAC scoring (no GPU counterpart in the reference): counts[h] = number of
 * correspondences whose Sampson distance to fundamental matrix h (row-major
 * 3x3 double) is below thr (ransac_cpu.cpp:183-210), in the evaluation order
 * documented with the CUDA kernel; masks (or NULL) receive the inlier bits. */
void orc_sampson_counts(const double* fmats, int n_hyp, const double* prev_xy, const double* curr_xy, int n,
                        double thr, int* counts, uint32_t* masks);

/* The shared canonical transcendentals (include/uslam_canon.h), exported so
 * the tests can measure their accuracy against a double-precision libm. */
float orc_atan2f(float y, float x);
void orc_sincosf(float a, float* s, float* c);

#ifdef __cplusplus
}
#endif

#endif
