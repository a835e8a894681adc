// Minimal restatement of wslam/include/wslam/common.hpp for compiling the
// reference matcher and triangulation pass: the constants they read
// (GPUConst), the AnyBag keys they use (common.hpp:124-153), and an AnyBag
// with the two members they call.  Test infrastructure.
#pragma once
#include <any>
#include <cstdint>
#include <format>
#include <optional>
#include <string>
#include <unordered_map>

#include <spdlog/spdlog.h>  // the real common.hpp reaches spdlog through anybag.hpp

#ifndef WSLAM_FRAME_WIDTH
#define WSLAM_FRAME_WIDTH 752
#endif
#ifndef WSLAM_FRAME_HEIGHT
#define WSLAM_FRAME_HEIGHT 480
#endif

class AnyBag {
   public:
    void set(const std::string& key, auto&& value) {
        data_[key] = std::make_any<std::decay_t<decltype(value)>>(std::forward<decltype(value)>(value));
    }
    template <typename T>
    std::optional<T*> getPtr(const std::string& key) {
        auto it = data_.find(key);
        if (it == data_.end()) return std::nullopt;
        T* p = std::any_cast<T>(&it->second);
        if (!p) return std::nullopt;
        return p;
    }

   private:
    std::unordered_map<std::string, std::any> data_;
};

namespace wslam {
namespace GPUConst {
constexpr uint32_t frame_width = WSLAM_FRAME_WIDTH;
constexpr uint32_t frame_height = WSLAM_FRAME_HEIGHT;
constexpr uint32_t levels_of_detail = 6;
constexpr uint32_t max_features_per_lod = frame_width * frame_height / 250;
constexpr double lod_scale_factor = 1.2;
}  // namespace GPUConst
namespace ResourceIdentifier {
inline std::string GetFeatureSetName(size_t keyframes_ago) {
    return std::format("gen:feat:-{}", keyframes_ago);
}
inline const std::string MatchedFeaturesName = "gen:feat:match";
inline const std::string RansacResultName = "gen:feat:ransac";
inline const std::string TriangulationResultName = "gen:tri";
inline std::string GetImuVecName() { return "res:imu:vec"; }
inline std::string GetCameraIntrinsicsName(uint32_t cam_idx) {
    return std::format("res:cam:intrinsics:{}", cam_idx);
}
}  // namespace ResourceIdentifier
}  // namespace wslam
