// ref_harness.cpp — C entry point around the reference's own matcher
// (TEST INFRASTRUCTURE ONLY).
//
// The reference source wslam/src/pose_estimate_cpu/match_features_cpu.cpp is
// included unmodified (the Makefile puts its directory on the include path;
// the shim headers in oracle/ref_shims stand in for Dawn-dependent headers).
// Including the .cpp makes its anonymous-namespace impl::FindMatches
// (match_features_cpu.cpp:152-207) callable from this translation unit.
#include "match_features_cpu.cpp"

#include <cstring>
#include <map>

namespace {
struct RefGpuFeature {  // gpumodels::Feature layout (wslam/src/models.hpp:31-69)
    float x;
    float y;
    uint32_t strength;
    float orientation;
    uint32_t descriptor[8];
};

wslam::FeatureSet ToSet(const RefGpuFeature* f, const int* off) {
    wslam::FeatureSet set;
    for (uint32_t lod = 0; lod < wslam::GPUConst::levels_of_detail; ++lod) {
        for (int i = off[lod]; i < off[lod + 1]; ++i) {
            // FromGpuModel (wslam/src/models.hpp:113-120)
            wslam::Feature g{};
            g.x = static_cast<uint32_t>(f[i].x);
            g.y = static_cast<uint32_t>(f[i].y);
            g.lod = lod;
            g.strength = f[i].strength;
            g.orientation = f[i].orientation;
            std::memcpy(g.descriptor.data(), f[i].descriptor, sizeof(f[i].descriptor));
            set.at(lod).push_back(g);
        }
    }
    return set;
}
}  // namespace

extern "C" int ref_levels() { return static_cast<int>(wslam::GPUConst::levels_of_detail); }
extern "C" int ref_frame_width() { return static_cast<int>(wslam::GPUConst::frame_width); }
extern "C" int ref_frame_height() { return static_cast<int>(wslam::GPUConst::frame_height); }

// prev = a (FeatureSet(1)), curr = b (FeatureSet(0)), as MatchFeaturesCPU::execute
// calls FindMatches(**prev, **curr) (match_features_cpu.cpp:253).  out receives
// (lod_a, idx_a, lod_b, idx_b) per match sorted by (lod_a, idx_a).
extern "C" int ref_find_matches(const RefGpuFeature* a, const int* a_off, const RefGpuFeature* b,
                                const int* b_off, int32_t* out, int max_out) {
    const auto set_a = ToSet(a, a_off);
    const auto set_b = ToSet(b, b_off);
    const wslam::MatchResult result = impl::FindMatches(set_a, set_b);
    // feature -> index within its level (features are unique within a set)
    std::map<wslam::Feature, int> index_a, index_b;
    for (uint32_t lod = 0; lod < wslam::GPUConst::levels_of_detail; ++lod) {
        for (size_t i = 0; i < set_a[lod].size(); ++i) index_a.emplace(set_a[lod][i], static_cast<int>(i));
        for (size_t i = 0; i < set_b[lod].size(); ++i) index_b.emplace(set_b[lod][i], static_cast<int>(i));
    }
    std::vector<std::array<int32_t, 4>> rows;
    for (uint32_t lod = 0; lod < wslam::GPUConst::levels_of_detail; ++lod) {
        for (const auto& [fb, fa] : result[lod]) {
            rows.push_back({static_cast<int32_t>(lod), index_a.at(fa), static_cast<int32_t>(fb.lod),
                            index_b.at(fb)});
        }
    }
    std::sort(rows.begin(), rows.end());
    if (static_cast<int>(rows.size()) > max_out) return -1;
    for (size_t i = 0; i < rows.size(); ++i) std::memcpy(&out[4 * i], rows[i].data(), 16);
    return static_cast<int>(rows.size());
}
