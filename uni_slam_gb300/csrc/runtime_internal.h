// runtime_internal.h — host-runtime internals shared by the batch runtime
// (runtime.cu) and the serving loop (server.cu): kernel launchers, level
// dimensions, the cull coverage bitmap and the device context.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/uslam.h"
#include "uslam_internal.h"

namespace uslam {
struct MatchSegDev {
    int pair;
    int dir;
    int level;
};
cudaError_t init_constants();
cudaError_t launch_detect(const FrameDev*, const TileItem*, int, int, int, uint32_t*, cudaStream_t);
cudaError_t launch_pyramid(const FrameDev*, const TileItem*, int, int, cudaStream_t);
cudaError_t launch_compact_banded(const FrameDev*, const BandItem*, int, const SegDev*, int, int, cudaStream_t);
cudaError_t launch_blur_border(const FrameDev*, const SegDev*, int, int, cudaStream_t);
cudaError_t launch_describe(const FrameDev*, const SegDev*, int, const int32_t*, int, bool, bool, cudaStream_t);
// k_describe_tiled over describe items (one per KDT_CW-column chunk of every
// 32-row band); describe_tiled_smem(margin) = its dynamic shared memory, 0 if
// the box does not fit a TMA box (then k_describe runs instead).
cudaError_t launch_describe_tiled(const FrameDev*, const BandItem*, int, const int32_t*, bool, bool, int, uint32_t*,
                                  cudaStream_t);
size_t describe_tiled_smem(int margin);
// Frames of a batch (or server launch) from which describe_form 1 runs
// k_describe_tiled (one frame measured 0.09 ms longer than with k_describe).
constexpr int kTiledDescribeFrames = 8;
cudaError_t set_describe_tiled_smem(int margin);
// k_match over num_sms x its resident CTAs; _dyn: its warps claim query groups from next_group
cudaError_t launch_match(const FrameDev*, const PairDev*, const void* segs, int nseg, int num_sms, cudaStream_t);
cudaError_t launch_match_dyn(const FrameDev*, const PairDev*, const void* segs, int nseg, int num_sms,
                             uint32_t* claim, uint8_t* gbucket, cudaStream_t);
size_t match_claim_words(size_t max_groups);  // u32 words of one claim block
cudaError_t launch_mutual(const FrameDev*, const PairDev*, const SegDev*, int, uint32_t*, cudaStream_t);
cudaError_t launch_bacc_init(const FrameDev*, const PairDev*, const SegDev*, int, cudaStream_t);
cudaError_t launch_mutual_reset(const FrameDev*, const PairDev*, const SegDev*, int, uint32_t*, uint32_t*,
                                cudaStream_t);
cudaError_t launch_emit(const FrameDev*, const PairDev*, const SegDev*, int, uint32_t*, cudaStream_t);
cudaError_t launch_bruteforce(const FrameDev*, const PairDev*, const SegDev*, int, float, int, cudaStream_t);
cudaError_t launch_bf_mma(const FrameDev*, const PairDev*, const SegDev*, int, float, int, uint32_t*, cudaStream_t);
cudaError_t set_compact_smem(int max_w);
cudaError_t set_bf_mma_smem();
cudaError_t launch_frame_from_f32(const float* src, int W, int H, uint8_t* dst, int dpitch, cudaStream_t st);
// the windowed matcher on the tensor cores (win_tc.cu)
cudaError_t set_win_mma_smem();
int win_units_per_seg(int cap);
size_t win_unit_bytes();
cudaError_t launch_win_match(const FrameDev*, const PairDev*, const void*, int, int, void*, int, uint32_t*,
                             cudaStream_t);
constexpr int kWinMaxCap = 60000;  // list positions and tile columns stay within 16 bits
// Tile shapes (width, height) that k_detect is instantiated for; the index
// is the `shape` argument of launch_detect.  Every shape computes the same
// values (the arithmetic is per pixel), so the choice affects speed only.
constexpr int kNumTileShapes = USLAM_NUM_TILE_SHAPES;
constexpr int kTileShapes[kNumTileShapes][2] = {{64, 32}, {128, 32}, {64, 16}, {32, 32}, {128, 16}};
constexpr int kMaxSegs = 4096;
constexpr int kMaxWidth = 8192;
}  // namespace uslam

using namespace uslam;

namespace uslam_rt {

inline size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Operand rows of a frame for the tensor-core matcher: every kept feature of
// the frame (at most levels x cap, or frame_cap), rounded up to 256.
inline size_t tc_rows(const FrameDev& F) {
    size_t n = static_cast<size_t>(F.levels) * static_cast<size_t>(F.cap > 0 ? F.cap : 1);
    if (F.frame_cap > 0) n = std::min(n, static_cast<size_t>(F.frame_cap));
    return round_up(n, 256);
}

// A context's last error message.  Calls on one server may fail on several
// host threads at once (submitting threads, result readers), so a write and
// a reader's copy each take the lock.
class ErrText {
   public:
    ErrText& operator=(const std::string& msg) {
        std::lock_guard<std::mutex> g(mu_);
        text_ = msg;
        return *this;
    }
    std::string get() const {
        std::lock_guard<std::mutex> g(mu_);
        return text_;
    }

   private:
    mutable std::mutex mu_;
    std::string text_;
};

inline uslam_status set_err(ErrText* dst, uslam_status s, const std::string& msg) {
    if (dst) *dst = msg;
    return s;
}

// Level dims (wslam/src/common.cpp:41-45).
inline void level_dims(int W0, int H0, int levels, int* w, int* h) {
    for (int l = 0; l < levels; ++l) {
        const double factor = l == 0 ? 1.0 : std::pow(1.2, static_cast<double>(l));
        w[l] = static_cast<int>(static_cast<uint32_t>(static_cast<double>(W0) / factor));
        h[l] = static_cast<int>(static_cast<uint32_t>(static_cast<double>(H0) / factor));
    }
}

inline uint32_t ceil_div_u(uint32_t n, uint32_t d) { return (n + d - 1u) / d; }

// Coverage of the reference's cull passes for one level, as a bitmap.
// main_horizontal (resources/cull_corners.wgsl:22-57) with dispatch
// ceil(ceil(W0/3)/64) x H0 x levels workgroups of 64 (cull_corners.cpp:332-341)
// writes H[9*gx + y*w] = S for every start >= w (the regional loop is empty
// there because end = min(start+3, w) <= start); in row 0 it keeps the first
// arg-max of [9k, min(9k+3, w)).  main_vertical (:60-109) with dispatch
// ceil(W0/64) x ceil(H0/3) copies H at start + k*w, k < min((W0*H0 - start)/w, 3),
// start = 3*gx + 3*gy*w, and at start itself in every case.  A keypoint is a pixel whose final value is > 0, so:
//   bit(p) = V(p) && (p < w ? p % 9 < 3 : H(p)),
// with the row-0 arg-max applied in the kernel.
inline std::vector<uint32_t> build_cull_mask(int W0, int H0, int w, int h) {
    const uint64_t n = static_cast<uint64_t>(w) * static_cast<uint64_t>(h);
    const uint64_t blk = static_cast<uint64_t>(W0) * static_cast<uint64_t>(H0);
    std::vector<uint8_t> mh(n, 0), mv(n, 0);
    const uint32_t gx_h = ceil_div_u(ceil_div_u(W0, 3), 64) * 64;
    const uint32_t gy_h = static_cast<uint32_t>(H0);
    const uint32_t gx_v = ceil_div_u(W0, 64) * 64;
    const uint32_t gy_v = ceil_div_u(H0, 3);
    for (uint32_t y = 0; y < gy_h; ++y)
        for (uint32_t gx = 0; gx < gx_h; ++gx) {
            const uint64_t s = 9ull * gx + static_cast<uint64_t>(y) * w;
            if (s < n && s >= static_cast<uint64_t>(w)) mh[s] = 1;
        }
    for (uint32_t gy = 0; gy < gy_v; ++gy)
        for (uint32_t gx = 0; gx < gx_v; ++gx) {
            const uint64_t s = 3ull * gx + 3ull * gy * static_cast<uint64_t>(w);
            if (s >= n) continue;
            // didFindMax starts as src[start] > 0, so V[start] = H[start] even
            // when the loop below is empty (cull_corners.wgsl:83-97)
            mv[s] = 1;
            uint64_t cnt = (blk - s) / static_cast<uint64_t>(w);
            if (cnt > 3) cnt = 3;
            for (uint64_t k = 0; k < cnt; ++k) {
                const uint64_t i = s + k * static_cast<uint64_t>(w);
                if (i < n) mv[i] = 1;
            }
        }
    std::vector<uint32_t> bits((n + 31) / 32, 0u);
    for (uint64_t p = 0; p < n; ++p) {
        const bool keep = mv[p] && (p < static_cast<uint64_t>(w) ? (p % 9) < 3 : mh[p] != 0);
        if (keep) bits[p >> 5] |= 1u << (p & 31);
    }
    return bits;
}

// Append the detect tiles of one frame for tile shape `shape`.
inline void append_tiles(std::vector<TileItem>* out, int frame, const FrameDev& F, int shape) {
    const int tw = kTileShapes[shape][0], th = kTileShapes[shape][1];
    for (int l = 0; l < F.levels; ++l) {
        const int nx = (F.w[l] + tw - 1) / tw, ny = (F.h[l] + th - 1) / th;
        for (int ty = 0; ty < ny; ++ty)
            for (int tx = 0; tx < nx; ++tx) {
                TileItem t{};
                t.frame = static_cast<uint16_t>(frame);
                t.level = static_cast<uint8_t>(l);
                t.tx = static_cast<uint16_t>(tx);
                t.ty = static_cast<uint16_t>(ty);
                out->push_back(t);
            }
    }
}

// Tiles grouped by shape: tiles[begin[s] .. begin[s+1]) use shape s.
struct ShapedTiles {
    std::vector<TileItem> by_shape[kNumTileShapes];
    std::vector<TileItem> flat;
    int begin[kNumTileShapes + 1] = {0};
    void finish() {
        flat.clear();
        for (int s = 0; s < kNumTileShapes; ++s) {
            begin[s] = static_cast<int>(flat.size());
            flat.insert(flat.end(), by_shape[s].begin(), by_shape[s].end());
        }
        begin[kNumTileShapes] = static_cast<int>(flat.size());
    }
};

// One k_pyramid launch per tile shape present.
inline cudaError_t launch_pyramid_shaped(const FrameDev* frames, const TileItem* d_tiles, const int* begin,
                                         cudaStream_t st) {
    for (int s = 0; s < kNumTileShapes; ++s) {
        const int n = begin[s + 1] - begin[s];
        if (n <= 0) continue;
        const cudaError_t e = launch_pyramid(frames, d_tiles + begin[s], n, s, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}
// One k_detect launch per tile shape present (after every pyramid level is written).
inline cudaError_t launch_detect_only_shaped(const FrameDev* frames, const TileItem* d_tiles, const int* begin,
                                             int detector, uint32_t* err, cudaStream_t st) {
    for (int s = 0; s < kNumTileShapes; ++s) {
        const int n = begin[s + 1] - begin[s];
        if (n <= 0) continue;
        const cudaError_t e = launch_detect(frames, d_tiles + begin[s], n, s, detector, err, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}
// One k_pyramid launch, then one k_detect launch, per tile shape present
// (every pyramid level is written before any tile of that shape reads it).
inline cudaError_t launch_detect_shaped(const FrameDev* frames, const TileItem* d_tiles, const int* begin,
                                        int detector, uint32_t* err, cudaStream_t st) {
    const cudaError_t e = launch_pyramid_shaped(frames, d_tiles, begin, st);
    if (e != cudaSuccess) return e;
    for (int s = 0; s < kNumTileShapes; ++s) {
        const int n = begin[s + 1] - begin[s];
        if (n <= 0) continue;
        const cudaError_t e = launch_detect(frames, d_tiles + begin[s], n, s, detector, err, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Row pitch (floats) of a pyramid level buffer: 16-byte rows for TMA.
inline int lvl_pitch_of(int w) { return static_cast<int>(round_up(static_cast<size_t>(w), 4)); }

// Encode the tensor maps of k_detect's tile loads for one frame whose level
// buffers F.lvl[] are set: per level and tile shape a 2D f32 map over
// [h][w] (row pitch lvl_pitch) with box (TW + 2 XPAD) x (TH + 2 HY), HY of
// the detector.  out holds levels * kNumTileShapes maps of USLAM_TMAP_BYTES.
uslam_status encode_tile_maps(const FrameDev& F, int detector, void* out, ErrText* err);

struct ResClass {
    int W0 = 0, H0 = 0;
    std::vector<uint32_t*> d_mask;
};

}  // namespace uslam_rt

using namespace uslam_rt;

struct uslam_ctx {
    int device = 0;
    int levels = 6;
    int max_w = 0, max_h = 0;
    int cap_override = 0;
    int num_sms = 0;
    int margin = 0;  // blur-cache margin: BRIEF pattern radius + 2
    int matcher = 0;      // 0 windowed mutual (reference), 1 brute-force top-2
    bool win_tc = false;  // matcher 0 asked for with the distances from the tensor cores (matcher 3)
    float ratio = 0.8f;   // Lowe ratio of the brute-force matcher
    int frame_cap = 0;    // > 0: features kept per frame, levels filled in order
    int describe_form = 0;  // 1: k_describe_tiled in batches of kTiledDescribeFrames frames or more
    int cell_cap = 0;     // > 0: keypoints kept per 32x32 cell of a level, cell order
    int detector = 0;     // 0 reference FAST + cull, 1 cfg profile (FAST 9-of-16 at 20/255 + 3x3 NMS)
    std::map<std::pair<int, int>, int> tile_shape;  // per resolution class (autotuned or set)
    std::map<std::pair<int, int>, uslam_batch*> match_batches;  // uslam_match: a 2-frame batch per frame size
    void* ransac_buf = nullptr;  // uslam_ransac_score scratch, grown on demand
    size_t ransac_bytes = 0;
    std::mutex ransac_mu;
    void* tri_buf = nullptr;  // uslam_triangulate scratch, grown on demand
    size_t tri_bytes = 0;
    std::mutex tri_mu;
    int shape_for(int W0, int H0) const {
        auto it = tile_shape.find(std::make_pair(W0, H0));
        return it == tile_shape.end() ? 0 : it->second;
    }
    int32_t* d_pattern = nullptr;
    ErrText err;
    std::map<std::pair<int, int>, ResClass> classes;

    uslam_status cuda_fail(cudaError_t e, const char* what) {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return USLAM_CUDA_ERROR;
    }
    // Masks of a resolution class, built and uploaded on first use.
    uslam_status masks_for(int W0, int H0, const int* w, const int* h, std::vector<uint32_t*>* out) {
        auto key = std::make_pair(W0, H0);
        auto it = classes.find(key);
        if (it == classes.end()) {
            ResClass rc;
            rc.W0 = W0;
            rc.H0 = H0;
            for (int l = 0; l < levels; ++l) {
                const std::vector<uint32_t> bits = build_cull_mask(W0, H0, w[l], h[l]);
                uint32_t* d = nullptr;
                cudaError_t e = cudaMalloc(&d, bits.size() * sizeof(uint32_t));
                if (e != cudaSuccess) {
                    for (auto* p : rc.d_mask) cudaFree(p);
                    err = std::string("cull mask allocation: ") + cudaGetErrorString(e);
                    return e == cudaErrorMemoryAllocation ? USLAM_OOM : USLAM_CUDA_ERROR;
                }
                e = cudaMemcpy(d, bits.data(), bits.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
                if (e != cudaSuccess) {
                    cudaFree(d);
                    for (auto* p : rc.d_mask) cudaFree(p);
                    return cuda_fail(e, "cull mask upload");
                }
                rc.d_mask.push_back(d);
            }
            it = classes.emplace(key, std::move(rc)).first;
        }
        *out = it->second.d_mask;
        return USLAM_OK;
    }
};
