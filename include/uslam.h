/*
 * uslam.h — C ABI of the GB300 feature front-end (pyramid, FAST-style detect,
 * cull, rotated BRIEF, windowed mutual Hamming matching).
 *
 * It replaces, for the reference uni_slam:
 *   - the four GPU passes of the feature-detect stage
 *     (wslam/src/feature_detect/feature_detect.cpp:54-67: FillPyramidPass,
 *     PassDetectCorners, CullCornersPass, GenerateFeaturesPass),
 *   - the feature readback/decode of LoadDataCPUPass
 *     (wslam/src/pose_estimate_cpu/load_features_cpu.cpp:54-187),
 *   - the CPU matcher MatchFeaturesCPU
 *     (wslam/src/pose_estimate_cpu/match_features_cpu.cpp:152-268).
 *
 * Plain pointers and sizes only.  Every call returns a uslam_status; on
 * failure uslam_last_error(ctx) holds a message.  No call throws.  A context
 * and everything created from it belong to one host thread at a time, except
 * a server, whose submit / wait / result / release may come from several
 * threads (see uslam_server_submit).
 */
#ifndef USLAM_H
#define USLAM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum uslam_status {
    USLAM_OK = 0,
    USLAM_INVALID_ARG = 1, /* bad size, null pointer, out-of-range index */
    USLAM_OOM = 2,         /* device or pinned-host allocation refused */
    USLAM_TIMEOUT = 3,     /* a bounded wait ran out (uslam_*_sync with timeout) */
    USLAM_CUDA_ERROR = 4,  /* a CUDA runtime call failed */
    USLAM_CAPACITY = 5,    /* caller buffer or admission budget too small */
    USLAM_NOT_READY = 6,   /* no reference feature set yet (the reference's STAGE_STOP) */
    USLAM_KERNEL_CHECK = 7 /* a kernel's own bounds check tripped (error word set) */
} uslam_status;

typedef struct uslam_ctx uslam_ctx;
typedef struct uslam_batch uslam_batch;
typedef struct uslam_frontend uslam_frontend;

/* Same 48-byte layout as the reference's gpumodels::Feature
 * (wslam/src/models.hpp:31-69): coords, FAST strength, orientation (rad),
 * 256-bit descriptor (bit i of the BRIEF test i is word i/32, bit i%32). */
typedef struct uslam_feature {
    float x;
    float y;
    uint32_t strength;
    float orientation;
    uint32_t descriptor[8];
} uslam_feature;

/* One mutual match: feature idx_a of level lod_a of the previous (reference)
 * set and feature idx_b of level lod_b of the current set.  The reference
 * keeps these in MatchResult[lod_a] keyed by the current feature
 * (match_features_cpu.cpp:195-205). */
typedef struct uslam_match {
    int32_t lod_a;
    int32_t idx_a;
    int32_t lod_b;
    int32_t idx_b;
} uslam_match;

typedef struct uslam_params {
    int device;          /* CUDA device ordinal */
    int levels;          /* pyramid levels; reference: 6 (wslam/include/wslam/common.hpp:43) */
    int max_width;       /* largest accepted frame width (<= 8192) */
    int max_height;      /* largest accepted frame height */
    int cap_per_level;   /* features kept per level; 0 = W0*H0/250 (common.hpp:47) */
    /* 256 BRIEF tests, (ax, ay, bx, by) int32 each: the reference's
     * gpumodels::BRIEFTestSet uploaded by GenerateFeaturesPass::writeConstantValues
     * (wslam/src/feature_detect/generate_features.cpp:450-493). */
    const int32_t* brief_pattern;
    /* 0: the reference's windowed mutual matcher (match_features_cpu.cpp:66-207);
     * 1: brute-force top-2 over all features of both frames, Lowe test
     *    best < ratio * second, no window and no cross-check (XOR + popcount
     *    on the integer pipes);
     * 2: the same brute-force top-2 with the distances from the tensor cores
     *    (popc(a & b) as an FP8 0/1 dot product, exact): identical results;
     * 3: matcher 0 (the same match lists) with the in-window distances of
     *    the batch path taken from tensor-core tiles (k_win_mma) where every
     *    level holds at most 60000 features; slower than matcher 0 on the
     *    752x480 workload, kept as an option. */
    int matcher;
    float ratio;  /* Lowe ratio of matchers 1 and 2 (the windowed matchers 0 and 3 use the reference's 0.85) */
    /* 0: a level's keypoints in (y, x) order, the first cap_per_level kept.
     * 1..1024: per-cell caps -- each level is cut into 32x32 cells from its
     * origin; the first cell_cap keypoints of each cell in (y, x) order are
     * kept, listed cell by cell (cells in row-major order), and the level cap
     * then keeps the first cap_per_level of that list.  No reference
     * counterpart: the reference keeps whichever keypoints win its atomic
     * append (generate_features.wgsl:67-70). */
    int cell_cap;
    /* 0: the reference's detector (FAST response, resources/detect_corners.wgsl,
     *    and its cull, resources/cull_corners.wgsl).
     * 1: the `cfg` profile, no reference counterpart: FAST 9-of-16 with
     *    wrap-around, a circle point brighter iff p - c > 20/255 or darker iff
     *    c - p > 20/255; pixels within 3 of a level edge are never corners;
     *    score = sum of (|p - c| - 20/255) over the qualifying points in
     *    circle order; 3x3 non-maximum suppression on the score, a tie going
     *    to the first pixel in raster order; strength = the arc length. */
    int detector;
    /* 0: no per-frame cap (the reference caps per level only, common.hpp:47).
     * > 0: the levels are filled in order, level l keeping the first
     * min(cap_per_level, frame_cap - features kept by levels 0..l-1) of its
     * order, so a frame keeps the first frame_cap features in (level, y, x)
     * order (or (level, cell, y, x) with cell_cap).  No reference counterpart. */
    int frame_cap;
    /* How the describe stage reads the blur cache (identical records):
     * 0: per-test gathers from global memory (k_describe);
     * 1: batches of 8 frames or more stage the cache box of every 32-row x
     *    128-column chunk in shared memory by one TMA load and read the tests
     *    from there (k_describe_tiled); measured no faster on 752x480 frames
     *    and slower on sparse 4K levels, so not the default. */
    int describe_form;
} uslam_params;

/* ---- context ---------------------------------------------------------- */

/* Replaces the Dawn device + pass initialisation (compute/src/gpu.cpp:284-553,
 * every Pass::initialize of the feature-detect stage). */
uslam_status uslam_create(const uslam_params* params, uslam_ctx** out);
void uslam_destroy(uslam_ctx* ctx);
/* The message of the context's last failed call.  The pointer is a copy for
 * the calling thread, valid until that thread calls uslam_last_error again. */
const char* uslam_last_error(const uslam_ctx* ctx);
const char* uslam_status_string(uslam_status s);
/* Level dimensions w_l = (uint32)(W0 / pow(1.2, l)) (wslam/src/common.cpp:41-45). */
uslam_status uslam_level_dims(int width, int height, int levels, int* w_out, int* h_out);

/* Host-only: the data-independent coverage of the reference's two cull
 * dispatches for a level of size w x h of a W0 x H0 frame
 * (resources/cull_corners.wgsl:22-109 with the dispatch of
 * wslam/src/feature_detect/cull_corners.cpp:332-353), as a bitmap of
 * ceil(w*h/32) words: bit p set iff pixel p survives culling whenever its
 * response is > 0 (row 0 additionally needs the 1x3 first arg-max, applied
 * on the device).  Needs no GPU. */
uslam_status uslam_cull_coverage(int W0, int H0, int w, int h, uint32_t* bits_out);

/* ---- detect tile shapes and the autotuner ------------------------------
 * k_detect is built for several tile shapes; every shape computes the same
 * values, so the choice per resolution class changes speed only.  A batch or
 * server created afterwards uses the shape stored for each frame size
 * (default: shape 0).  No reference counterpart (the WGSL passes use fixed
 * 16x16 / 64-wide workgroups). */
uslam_status uslam_tile_shapes(int* n_out, int* tile_w, int* tile_h);
uslam_status uslam_set_tile_shape(uslam_ctx* ctx, int width, int height, int shape);
uslam_status uslam_get_tile_shape(const uslam_ctx* ctx, int width, int height, int* shape);
/* Time the detect kernel in every shape on n_frames copies of a
 * representative frame (median of `reps` launches), store the fastest for
 * width x height and return it in *shape_out; ms_out (n entries from
 * uslam_tile_shapes, or NULL) receives each shape's median time.  Allocates
 * a temporary batch; synchronous. */
uslam_status uslam_autotune(uslam_ctx* ctx, int width, int height, const uint8_t* img, int pitch, int n_frames,
                            int reps, int* shape_out, float* ms_out);

/* ---- single-frame export set ---------------------------------------------
 * A device-resident feature set (replaces one FeatureSet of the reference,
 * wslam/src/models.hpp, produced by the four feature-detect passes), a
 * one-shot detect + describe into it, a host copy of it, and a match between
 * two sets (the reference's MatchFeaturesCPU, match_features_cpu.cpp:217-268,
 * with the context's matcher).  Synchronous.  Sets of one context share its
 * device; a set belongs to one host thread at a time. */
typedef struct uslam_featset uslam_featset;
uslam_status uslam_featset_create(uslam_ctx* ctx, int width, int height, uslam_featset** out);
void uslam_featset_destroy(uslam_featset* set);
/* u8 frame (pitch in bytes) of the set's size. */
uslam_status uslam_detect_describe(uslam_ctx* ctx, const uint8_t* img, int width, int height, int pitch,
                                   uslam_featset* out);
/* f32 frame in [0, 1] (pitch in floats), the reference's FrameBW: exact for
 * values u8 / 255 (data/src/provider_base.cpp:121-124); other values round to
 * the nearest 1/255. */
uslam_status uslam_detect_describe_f32(uslam_ctx* ctx, const float* img, int width, int height, int pitch,
                                       uslam_featset* out);
/* Host copy: features level by level in the set's order; kept/raw receive
 * `levels` counts each. */
uslam_status uslam_featset_features(uslam_featset* set, uslam_feature* out, int max_out, int* kept, int* raw);
/* Matches of prev (the reference set) against curr, both from frames of the
 * same size; out may be NULL to ask for the count. */
uslam_status uslam_match_sets(uslam_ctx* ctx, const uslam_featset* prev, const uslam_featset* curr, uslam_match* out,
                              int max_out, int* n_out);

/* ---- RANSAC hypothesis scoring (the stage after matching) ----------------
 * No counterpart as a GPU pass in the reference: RansacCPU
 * (wslam/src/pose_estimate_cpu/ransac_cpu.cpp) scores one fundamental matrix
 * per iteration on the host (SampsonDistance :173-188, ClassifyInliers
 * :190-203).  This scores n_hyp matrices (row-major 3x3 doubles, the
 * reference's convention: prev = point of the first image, curr = second)
 * against n_matches correspondences in LOD-0 pixels (x, y doubles):
 * counts[h] = number of matches with Sampson distance < threshold (px^2;
 * the reference's default 3.84).  masks (NULL or n_hyp * ceil(n / 32) words)
 * receives the inlier bitmask of every hypothesis (bit i of word i / 32).
 * Double precision, no contraction, a fixed evaluation order written in
 * ransac.cu.  Host buffers; synchronous. */
uslam_status uslam_ransac_score(uslam_ctx* ctx, const double* fmats, int n_hyp, const double* prev_xy,
                                const double* curr_xy, int n_matches, double threshold, int* counts,
                                uint32_t* masks);

/* ---- two-view triangulation (the pass after RANSAC) ---------------------
 * TriangulateCPU::execute (wslam/src/pose_estimate_cpu/triangulate_cpu.cpp:342-513)
 * for n_pairs independent frame pairs in one call.  Pair p's rows are
 * offsets[p] .. offsets[p + 1] - 1 of px: (prev_x, prev_y, curr_x, curr_y),
 * the LOD-0 pixels of its RANSAC inliers (util::ToLod0Pixel of the two
 * features).  The reference visits the rows per level in the order of its
 * flat_map keys, so rows in that order give the same results.  Per pair:
 * the rays are undistorted (bit-exact), the essential matrix is re-fitted on
 * all rays, the four (R, t) of its decomposition are scored by cheirality,
 * and the best pose's points pass the depth range and the reprojection
 * filter.  results[p] receives the TriangulationResult fields
 * (wslam/src/models.hpp:163-184); landmarks (NULL or 4 doubles per row:
 * x, y, z in the current camera, mean reprojection error) and keep (NULL or
 * one byte per row) mark the rows that became landmarks; other rows are 0.
 * opts NULL means the reference's defaults (uslam_tri_default_opts).  Pose
 * and points agree with the reference to rounding (its SVDs are computed
 * by other algorithms), see triangulate.cu.  Host buffers; synchronous. */
typedef struct uslam_camera {
    double fu, fv, cu, cv; /* intrinsics, LOD-0 pixels (CamSensorParams::intrinsics) */
    double k1, k2, p1, p2; /* radial-tangential distortion (distortion_coefficients) */
} uslam_camera;

typedef struct uslam_tri_opts {
    double max_reprojection_px; /* 4.0 */
    double min_depth;           /* 1e-3 */
    double max_depth;           /* 1e3 */
    double undistort_tolerance; /* 1e-9 */
    int min_inliers;            /* 8 (values below 8 are refused) */
    int undistort_iterations;   /* 20 */
} uslam_tri_opts;

typedef struct uslam_tri_result {
    double rotation[9];    /* row-major, p_curr = R p_prev + t; identity when no pose */
    double translation[3]; /* unit norm */
    double mean_reprojection_error_px;
    double rotation_angle_rad;
    int input_matches;
    int landmark_count;
    int cheirality_passes;
    int pose_recovered;
} uslam_tri_result;

void uslam_tri_default_opts(uslam_tri_opts* opts);
/* util::PixelToNormalised (wslam/src/map/map_helpers_lods.hpp:110-120), the
 * undistortion CollectInliers applies to every inlier pixel
 * (triangulate_cpu.cpp:218-247): n pixels (x, y doubles) -> n calibrated
 * rays, equal to the reference's bit for bit.  Host buffers; synchronous. */
uslam_status uslam_pixel_to_normalised(uslam_ctx* ctx, const uslam_camera* cam, int iterations, double tolerance,
                                       const double* px, int n, double* out);
uslam_status uslam_triangulate(uslam_ctx* ctx, const uslam_camera* cam, const uslam_tri_opts* opts, int n_pairs,
                               const int* offsets, const double* px, uslam_tri_result* results, double* landmarks,
                               uint8_t* keep);

/* ---- batched form: a work table over many frames and frame pairs -------- */

/* Plan a batch of n_frames frames (any mix of sizes) and n_pairs matches
 * (pair k matches frame pair_prev[k] (reference set) against frame
 * pair_curr[k]).  Allocates every device buffer up front.  At most 4096
 * (frame, level) segments and, with the windowed matcher, 2048 (pair, level)
 * segments: USLAM_CAPACITY beyond. */
uslam_status uslam_batch_create(uslam_ctx* ctx, int n_frames, const int* widths, const int* heights,
                                int n_pairs, const int* pair_prev, const int* pair_curr, uslam_batch** out);
void uslam_batch_destroy(uslam_batch* b);
/* Device address and row pitch of a frame's LOD0 input buffer (u8), for
 * callers that keep frames resident in HBM. */
uslam_status uslam_batch_input_device(uslam_batch* b, int frame, uint8_t** dev_ptr, int* pitch);
/* Pinned host staging buffer of a frame's input (row pitch as above). */
uslam_status uslam_batch_input_host(uslam_batch* b, int frame, uint8_t** host_ptr, int* pitch);
/* Asynchronous host->device copy of every frame from the pinned staging. */
uslam_status uslam_batch_upload(uslam_batch* b);
/* Copy caller frames (any host memory, given pitch) into the pinned staging. */
uslam_status uslam_batch_set_frame(uslam_batch* b, int frame, const uint8_t* img, int pitch);
/* Launch detect + describe of every frame and match of every pair (one CUDA
 * graph replay: about nine kernel launches for the whole batch, whatever its
 * size; a batch of 16 or more frames runs them once for each half of its
 * frames, the halves side by side on two streams). Asynchronous. */
uslam_status uslam_batch_run(uslam_batch* b);
/* Asynchronous device->host copy of every frame's features and every pair's
 * matches into pinned staging (read them with the getters below). */
uslam_status uslam_batch_download(uslam_batch* b);
/* Wait for the batch (timeout_ms <= 0: no limit); checks kernel error words. */
uslam_status uslam_batch_sync(uslam_batch* b, int timeout_ms);
/* Features of a frame, level by level in (y, x) order, from the staging
 * (after download + sync).  kept/raw receive `levels` counts each. */
uslam_status uslam_batch_features(uslam_batch* b, int frame, uslam_feature* out, int max_out, int* kept,
                                  int* raw);
uslam_status uslam_batch_matches(uslam_batch* b, int pair, uslam_match* out, int max_out, int* n_out);
/* Parity getters (synchronous, read device memory directly). */
uslam_status uslam_batch_pyramid_level(uslam_batch* b, int frame, int level, float* out);
uslam_status uslam_batch_keypoint_map(uslam_batch* b, int frame, int level, uint8_t* out);
/* The extended blur cache of a level: (h + M + 1) rows of (w + M + 1)
 * floats, M from uslam_blur_margin; row/column w + M (h + M) hold the value
 * every negative x (y) takes. */
uslam_status uslam_batch_blur_level(uslam_batch* b, int frame, int level, float* out);
uslam_status uslam_blur_margin(const uslam_ctx* ctx, int* margin);
/* Issue later upload/run/download calls on a caller's cudaStream_t (NULL:
 * the batch's own stream), so callers can record their own events around them. */
uslam_status uslam_batch_set_stream(uslam_batch* b, void* cuda_stream);
/* Per-stage timing: launch the batch's stages `iters` times without the
 * graph and without the fork, with CUDA events between them on the batch
 * stream, and return the mean milliseconds per launch in kernel_ms[0..6]:
 * pyramid (k_pyramid, one launch per tile shape), detect (k_detect, one
 * launch per tile shape), blur-cache border
 * (k_blur_border), compaction (k_band_count + k_band_write + k_xsort),
 * describe (k_describe), match (k_match, k_bruteforce with matcher 1, k_bf_mma with matcher 2) and
 * mutual check / emit (k_mutual).  Synchronous. */
uslam_status uslam_batch_profile(uslam_batch* b, int iters, float* kernel_ms);
/* Test hook for the kernels' bounded waits (no reference counterpart): the
 * number of polls of the first mbarrier wait of k_detect's tile load
 * (detect_polls) and of the tensor-core brute-force matcher's first
 * query-tile load (match_polls, matcher 2); -1 restores a kernel's own limit.
 * A wait that runs out records USLAM_ERR_TMA_TIMEOUT in the batch's error word
 * (uslam_batch_sync then returns USLAM_KERNEL_CHECK) after the copy in flight
 * has landed (that drain keeps the full limit); the batch stays usable.  Takes
 * effect from the next run. */
uslam_status uslam_batch_set_first_wait(uslam_batch* b, int detect_polls, int match_polls);
/* Bytes moved by upload and download per call (for end-to-end accounting). */
uslam_status uslam_batch_io_bytes(uslam_batch* b, size_t* h2d, size_t* d2h);

/* ---- plain per-frame form: the reference's pass sequence ---------------- */

/* One camera stream of fixed frame size holding FeatureSet(0) (current) and
 * FeatureSet(1) (reference) on the device, with the reference's rotation rule
 * (LoadDataCPUPass::shiftFeatureSets, load_features_cpu.cpp:111-142). */
uslam_status uslam_frontend_create(uslam_ctx* ctx, int width, int height, uslam_frontend** out);
void uslam_frontend_destroy(uslam_frontend* fe);
/* Process one frame: upload (img == NULL: the frame is already in the input
 * buffer returned by uslam_frontend_input_device), detect + describe into
 * FeatureSet(0) and, when a reference set exists, match FeatureSet(1) ->
 * FeatureSet(0).  advance_reference mirrors the "gen:feat:refadv" marker:
 * the previous current set becomes the reference before this frame is
 * stored.  Returns USLAM_NOT_READY (features computed, no matching) when no
 * reference exists yet.  The frame is copied into a pinned staging buffer
 * and uploaded by an asynchronous copy on the frontend's stream (the u8
 * upload of FillPyramidPass::writeBaseLayer, fill_pyramid.cpp:221-269); the
 * new feature set and matches are copied back behind the work, so the
 * feature and match getters below read host memory.  Synchronous: returns
 * when the frame's work and copies are complete. */
uslam_status uslam_frontend_process(uslam_frontend* fe, const uint8_t* img, int pitch, int advance_reference);
/* The same for the reference's f32 FrameBW pixels in [0, 1] (pitch in
 * floats), uploaded as f32 the way FillPyramidPass::writeBaseLayer uploads
 * them: the rows are copied into a pinned f32 staging buffer, one
 * asynchronous copy takes them to the device, and a kernel recovers each byte
 * as p * 255 clamped to [0, 255] (NaN to 0), rounded half to even -- exact
 * for the u8 / 255 values data::getLocalFrame stores
 * (data/src/provider_base.cpp:121-124). */
uslam_status uslam_frontend_process_f32(uslam_frontend* fe, const float* img, int pitch, int advance_reference);
uslam_status uslam_frontend_input_device(uslam_frontend* fe, uint8_t** dev_ptr, int* pitch);
/* which = 0: current set, 1: reference set.  After uslam_frontend_process
 * these read the copies that came back with the frame; after
 * uslam_frontend_enqueue they first copy the outputs back (synchronous). */
uslam_status uslam_frontend_features(uslam_frontend* fe, int which, uslam_feature* out, int max_out, int* kept,
                                     int* raw);
uslam_status uslam_frontend_matches(uslam_frontend* fe, uslam_match* out, int max_out, int* n_out);
/* Asynchronous form of uslam_frontend_process for a frame already in device
 * memory (dev_img, row pitch; NULL: the frontend's input buffer): enqueue the
 * copy and the frame's work and return.  *matched tells whether a match was
 * enqueued.  Wait with uslam_frontend_sync. */
uslam_status uslam_frontend_enqueue(uslam_frontend* fe, const uint8_t* dev_img, int pitch, int advance_reference,
                                    int* matched);
uslam_status uslam_frontend_sync(uslam_frontend* fe);

/* ---- served form: many camera streams, continuous batching -------------- */

typedef struct uslam_server uslam_server;

typedef struct uslam_server_params {
    int n_sizes;              /* frame size classes served */
    const int* widths;        /* [n_sizes] */
    const int* heights;       /* [n_sizes] */
    size_t hbm_budget_bytes;  /* device memory for frame slots, shared equally by the size classes */
    int max_batch;            /* most frames one launch takes (max_batch x levels <= 2048) */
} uslam_server_params;

/* Frame slots (pyramid, features, keyframe pair scratch) are carved from the
 * budget; admission is by free slot.  A dispatcher thread launches the
 * queued frames as one batch whenever fewer than two launches are in flight,
 * on two alternating streams.  Each stream's keyframe features stay in their
 * slot on the device (the counterpart of FeatureSet(1),
 * load_features_cpu.cpp:111-142) and every new frame is matched against it. */
uslam_status uslam_server_create(uslam_ctx* ctx, const uslam_server_params* params, uslam_server** out);
void uslam_server_destroy(uslam_server* server);
uslam_status uslam_server_open_stream(uslam_server* server, int width, int height, int* stream_id);
/* Copy a frame into a free slot and queue it.  promote_keyframe: this frame
 * becomes the stream's keyframe for the frames submitted after it (a
 * stream's first frame always does).  USLAM_CAPACITY: no free slot of that
 * size right now (admission refused; retry later).  Different streams may
 * submit from different threads at the same time (the frame copy runs
 * outside the server's lock); the frames of one stream come from one thread
 * at a time, in order. */
uslam_status uslam_server_submit(uslam_server* server, int stream, const uint8_t* img, int pitch,
                                 int promote_keyframe, uint64_t* ticket);
/* Wait until the request has finished (timeout_ms <= 0: no limit).  After a
 * failed launch or a tripped kernel check the server launches nothing more:
 * requests in flight and queued finish with that status (USLAM_CUDA_ERROR or
 * USLAM_KERNEL_CHECK), uslam_server_result returns it for them (they have no
 * results; release them as usual), and submit refuses new frames with it. */
uslam_status uslam_server_wait(uslam_server* server, uint64_t ticket, int timeout_ms);
/* Features of the frame (as uslam_batch_features) and its mutual matches
 * against the keyframe it was submitted against (lod_a/idx_a = keyframe).
 * latency_ms = submit to completion seen by the dispatcher.  Returns
 * USLAM_NOT_READY (features filled, no matches) for a stream's first frame. */
uslam_status uslam_server_result(uslam_server* server, uint64_t ticket, uslam_feature* feats, int max_feats, int* kept,
                                 int* raw, uslam_match* matches, int max_matches, int* n_matches, double* latency_ms);
/* Give the request's slot back (it stays held while it is a keyframe). */
uslam_status uslam_server_release(uslam_server* server, uint64_t ticket);
uslam_status uslam_server_stats(uslam_server* server, uint64_t* launches, uint64_t* frames, int* max_batch_seen,
                                int* slots_total);
/* Test hook for the served form's failure path (no reference counterpart),
 * as uslam_batch_set_first_wait: the polls of the first mbarrier wait of
 * k_detect's tile load in every slot (-1 restores the kernel's own limit).
 * A wait that runs out trips the launch's kernel check without any fault.
 * Call with no request in flight. */
uslam_status uslam_server_set_first_wait(uslam_server* server, int detect_polls);

/* ---- matcher for callers that cannot allocate ---------------------------- */

/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * when they need a match (a runtime that owns all device memory through its
 * own pool, a real-time loop that must not take allocator locks or risk an
 * allocation failure mid-frame, a context whose memory budget is fixed): the
 * same mutual windowed match as the batch and frontend paths, of feature set
 * prev (the reference set) against curr, allocating nothing.
 *
 * Inputs and outputs are the caller's device memory: prev_feats/curr_feats
 * hold the features level after level in (y, x) order (the layout
 * uslam_batch_features returns), prev_kept/curr_kept (host arrays of
 * `levels` ints) the per-level counts; out receives levels blocks of
 * out_cap_per_level uslam_match entries (block l = matches whose previous
 * feature lies in level l, in that feature's order) and out_counts the
 * per-level match counts.  out_cap_per_level must be at least the previous
 * set's largest level count.  The feature arrays must be 16-byte aligned
 * (the matcher reads each descriptor as two 16-byte vectors; a sub-pointer
 * into a caller's pool must keep that alignment), out and out_counts 4-byte
 * aligned; other pointers return USLAM_INVALID_ARG before any device work.
 *
 * Each feature's x and y must be integers (as f32) inside its level
 * (0 <= x < w_l, 0 <= y < h_l), as every detector of this library and of the
 * reference produces them.  The counts and sizes are checked on the host and
 * the records by a kernel before anything indexes by them: a record outside
 * its level empties both sets for the rest of the call (nothing indexes by
 * it) and the call returns USLAM_INVALID_ARG.
 *
 * Scratch comes from a file-scope device array of 4 MiB that every GPU which
 * loads the library holds until the process exits; a call whose scratch need
 * exceeds it returns USLAM_CAPACITY.  The first call on a device looks up
 * that array's device address (cudaGetSymbolAddress), and so does the first
 * call after the device's context was reset; make that first call before any
 * stream capture.  All calls share the array: calls that overlap on the GPU
 * (different streams or threads at the same time) race and must not be
 * issued.  The call makes `device` current while it runs and restores the
 * caller's current device before it returns.  It enqueues on `stream` (a
 * cudaStream_t; NULL = the default stream), waits once at the end, and
 * returns after the work is complete.  err
 * (optional, err_len bytes) receives a message on failure. */
uslam_status uslam_match_noalloc(int device, int width, int height, int levels, const uslam_feature* prev_feats,
                                 const int* prev_kept, const uslam_feature* curr_feats, const int* curr_kept,
                                 uslam_match* out, uint32_t* out_counts, int out_cap_per_level, void* stream,
                                 char* err, size_t err_len);

#ifdef __cplusplus
}
#endif

#endif /* USLAM_H */
