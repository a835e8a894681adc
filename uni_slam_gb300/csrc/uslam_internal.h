// uslam_internal.h — device-side data layout shared by the kernels and the
// host runtime of the GB300 feature front-end.
//
// HBM layout of one frame slot (all sub-buffers 256-byte aligned, carved out
// of one arena allocation per batch):
//   img      u8   [H0][img_pitch]          LOD0 input (the H2D boundary)
//   lvl[l]   f32  [h_l][lvl_pitch_l]       pyramid level l (l = 0: u8/255), written by
//                                          k_pyramid; the source of k_detect's TMA tile
//                                          loads, so lvl_pitch_l = w_l rounded up to 4
//                                          floats (16-byte rows) and the base is 256-byte
//                                          aligned
//   tmaps    CUtensorMap [levels][USLAM_NUM_TILE_SHAPES]  2D tiled maps over lvl[l], one per tile
//                                          shape (box = tile + halo, widened to TW + 16
//                                          columns), 128 bytes each
//   blur[l]  f32  [h_l + M + 1][bl_pitch_l] 9-tap blurred sample G(P) of level l for
//                                          every integer point a BRIEF test can reach:
//                                          x in [0, w_l + M) plus one sentinel column
//                                          (index w_l + M) for every negative x (all
//                                          negative u32-wrapped x convert to the same
//                                          f32, 2^32); rows likewise.  M = pattern
//                                          radius + 2, bl_pitch_l = w_l + M + 1.
//   kpmap[l] u8   [h_l][kp_pitch_l]        culled FAST strength (0 = no keypoint)
//   bands[l] u32  [ceil(h_l / 32)][2]      raw and kept keypoint counts per 32-row band
//   feats[l] Feature[cap]                  gpumodels::Feature records, (y, x) order
//   xorder[l] u32 [B][cap]                 per band b of the frame height (B =
//                                          USLAM_MATCH_BANDS): indices of the features
//                                          whose LOD-0 y lies in the band widened by the
//                                          window half-height + 2, sorted by x (the
//                                          matcher's candidate lists)
//   colstart[l] u32 [B][w_l + 1] + [B + 1] first xorder slot of each column per band,
//                                          then the band offsets into qorder
//   qorder[l] u32 [cap]                    feature indices grouped by band (of their own
//                                          LOD-0 y), sorted by x within a band (queries)
//   counts   u32  [2][levels]              kept (<= cap) and raw keypoint counts
#pragma once

#include <stdint.h>
#include <vector_types.h>

#define USLAM_MAX_LEVELS 12
#define USLAM_MATCH_BANDS 3  // horizontal bands of the frame for the matcher's lists
#define USLAM_MAX_MATCH_SEGS 2048  // (pair, level) segments of one k_match launch

// Device copy of one frame's geometry and buffer addresses.
struct FrameDev {
    const uint8_t* img;
    int W0, H0, img_pitch, levels, cap;
    int w[USLAM_MAX_LEVELS];
    int h[USLAM_MAX_LEVELS];
    int kp_pitch[USLAM_MAX_LEVELS];
    int bl_pitch[USLAM_MAX_LEVELS];  // blur cache row pitch (floats): w + margin + 1
    int lvl_pitch[USLAM_MAX_LEVELS]; // pyramid level row pitch (floats): w rounded up to 4
    int margin;                      // blur cache margin M beyond the level
    int cell_cap;                    // > 0: keypoints kept per 32x32 cell (cell order); 0: (y, x) order
    int frame_cap;                   // > 0: features kept per frame, levels filled in order; 0: none
    // polls of the first mbarrier wait of k_detect's tile load and of the
    // tensor-core brute-force matcher's first query-tile load (-1: the
    // kernels' own limits); a test hook of uslam_batch_set_first_wait
    int detect_first_wait, match_first_wait;
    float* lvl[USLAM_MAX_LEVELS];
    const void* tmaps;  // CUtensorMap [levels][USLAM_NUM_TILE_SHAPES] over lvl (device, 64-byte aligned)
    float* blur[USLAM_MAX_LEVELS];
    uint8_t* kpmap[USLAM_MAX_LEVELS];
    uint32_t* bands[USLAM_MAX_LEVELS];       // per 32-row band: raw and kept keypoint counts
    const uint32_t* mask[USLAM_MAX_LEVELS];  // combined cull coverage bitmap
    uint32_t* feats[USLAM_MAX_LEVELS];       // 12 u32 (48 B) per feature
    uint32_t* xorder[USLAM_MAX_LEVELS];
    uint32_t* colstart[USLAM_MAX_LEVELS];
    uint32_t* qorder[USLAM_MAX_LEVELS];
    uint32_t* kept;  // [levels]
    uint32_t* raw;   // [levels]
    // tensor-core brute-force matcher (matcher 2; null otherwise): the frame's
    // descriptors over all levels (level-major flat order), written by
    // k_describe.  bf8 row f = 256 FP8 E4M3 values (bit k of the descriptor
    // -> 0x50 = 8.0 or 0x00), in 8-row groups of 2048 bytes: byte k of row f
    // at (f / 8) * 2048 + (k / 16) * 128 + (f % 8) * 16 + k % 16 (the K-major
    // no-swizzle core-matrix layout of tcgen05 operands); bfext row f = 32
    // E4M3 values (the popcount split into 16 integers <= 16, 256, f % 32
    // split into two integers <= 16, 1, zeros) in 8-row groups of 256 bytes
    // (same layout, K = 32); bfpop[f] = popcount; bfid[f] = packed (level,
    // index).  Rows are allocated up to a multiple of 256.
    uint8_t* bf8;
    uint8_t* bfext;
    uint32_t* bfpop;
    int32_t* bfid;
    // windowed matcher on the tensor cores (the batch path of matcher 0; null
    // otherwise): the frame's descriptors as operand rows in the bf8 layout.
    // wq8: the query order of each level (level l from row l * wq_rows), each
    // band's queries starting at a multiple of 128 rows; wc8 / wcext: the
    // candidate lists (list b of level l from row (USLAM_MATCH_BANDS l + b) *
    // wc_rows), with the extension rows of the bfext layout (row index within
    // its 32-row group = list position % 32); wcy: the candidate's y in its
    // level; wcid: packed (level, index).
    uint32_t* winv[USLAM_MAX_LEVELS];  // per level: query-order position of feature i at [i], its position
                                       // in candidate list b (or ~0) at [cap (1 + b) + i] (written by k_xsort)
    uint8_t* wq8;
    uint8_t* wc8;
    uint8_t* wcext;
    uint16_t* wcy;
    int32_t* wcid;
    int wq_rows, wc_rows;
};

// One frame pair to match: prev = reference set (a), curr = current set (b).
struct PairDev {
    int prev, curr;         // frame indices in the batch
    int32_t* a2b;           // [levels * cap_prev]: prev feature -> packed curr feature or -1
    int32_t* b2a;           // [levels * cap_curr] (the tensor-core windowed matcher)
    // k_match's search of each curr feature b (levels * cap_curr entries of
    // 16 bytes): .x = packed (level, index) and .y = distance of its nearest
    // prev feature, .z = its second-smallest distance; all ones = none.
    // Merged by atomic minima (.x/.y as one 64-bit word); null with the
    // other matchers.
    uint4* bacc;
    int32_t* matches;       // 4 ints per match (lod_a, idx_a, lod_b, idx_b)
    uint32_t* match_count;  // [levels] matches whose a lies in that level
    int max_matches_per_level;
    float max_dx, max_dy;   // 0.1f * W0, 0.1f * H0 of the frame size
    // brute-force matcher split over the train set: bf_splits partial top-2
    // records (best key, second key, best id, unused) per query, at
    // bf_part[(split * levels * cap_prev + level * cap_prev + index) * 4];
    // unused (nullptr, 1) when the train set is not split
    uint32_t* bf_part;
    int bf_splits;
    float bf_ratio;
};

// K1 work item: one TW x TH tile of one level of one frame.
struct TileItem {
    uint16_t frame;
    uint8_t level;
    uint8_t pad;
    uint16_t tx, ty;
};

// Segment tables for the persistent describe / match kernels.
struct SegDev {
    int frame;
    int level;
};

// Compaction work item: one 32-row band (a row of 32x32 cells) of one level.
// As a describe item (k_describe_tiled) pad2 is the chunk: columns
// pad2 * KDT_CW .. + KDT_CW - 1 of the band.
struct BandItem {
    uint16_t frame;
    uint8_t level;
    uint8_t pad;
    uint16_t band;
    uint16_t pad2;
};

#define USLAM_ERR_SMEM_RANGE 1u
#define USLAM_ERR_MATCH_OVERFLOW 2u
#define USLAM_ERR_TMA_TIMEOUT 4u  // a tile load did not complete within the wait limit

// k_detect tile staging: halo of HX columns and HY rows (HY_CFG with the cfg
// profile, whose 3x3 NMS needs the FAST score one pixel beyond the tile); the
// TMA box starts XPAD columns left of the tile (a 32-byte aligned x for every
// tile width) and is TW + 2 XPAD columns wide.
#define USLAM_TILE_HX 5
#define USLAM_TILE_HY 3
#define USLAM_TILE_HY_CFG 4
#define USLAM_TILE_XPAD 8
#define USLAM_TMAP_BYTES 128
#define USLAM_NUM_TILE_SHAPES 5  // k_detect tile shapes (kTileShapes of the runtime)
// Tensor maps per level of a frame: one per k_detect tile shape over the
// level, then one over the level's blur cache (k_describe_tiled's box).
#define USLAM_TMAPS_PER_LEVEL (USLAM_NUM_TILE_SHAPES + 1)
// k_describe_tiled: columns of a describe item (a chunk of a 32-row band).
#define KDT_CW 128

// Packed match-partner encoding: level in the top 8 bits, index in the low 24.
#define USLAM_PACK(l, i) (((int32_t)(l) << 24) | (int32_t)(i))
#define USLAM_PACK_LEVEL(p) ((int)((uint32_t)(p) >> 24))
#define USLAM_PACK_INDEX(p) ((int)((uint32_t)(p) & 0xffffffu))
