// uslam_wslam.hpp — drop-in uni_slam pipeline passes over the C ABI (header-only, C++20).
//
// Compile inside the reference tree: the includes below are the reference's
// own headers, by the names its sources use (wslam/include/wslam/common.hpp,
// wslam/src/models.hpp, compute/include/compute/{pass,stage}.hpp,
// data/include/data/provider_base.hpp).
//
//   CudaFeatureDetectPass replaces, in CreateFeatureDetectStage
//   (wslam/src/feature_detect/feature_detect.cpp:54-67), FillPyramidPass,
//   PassDetectCorners, CullCornersPass and GenerateFeaturesPass, and in
//   CreatePoseEstimateCPUStage (wslam/src/pose_estimate_cpu/pose_estimate_cpu.cpp:24-26)
//   the feature readback/decode/rotation of LoadDataCPUPass
//   (load_features_cpu.cpp:54-187).  It reads AnyBag["res:frame:0:lod:0"]
//   (data::FrameBW, f32 u8/255 pixels), consumes "gen:feat:refadv", and
//   stores "gen:feat:-0" / "gen:feat:-1" (FeatureSet) with the reference's
//   rotation rule.
//
//   CudaMatchPass replaces MatchFeaturesCPU (match_features_cpu.cpp:217-268):
//   it stores "gen:feat:match" (MatchResult), or returns the reference's
//   STAGE_STOP sentinel while no reference set exists.
//
// Both passes share one CudaFrontend (device context + FeatureSet(0)/(1) on
// the device).  Errors come back as std::optional<std::string>, as in the
// reference's Pass contract (compute/include/compute/pass.hpp:19-27).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <optional>
#include <string>
#include <vector>

#include "common.hpp"
#include "compute/pass.hpp"
#include "compute/stage.hpp"
#include "data/provider_base.hpp"
#include "models.hpp"
#include "uslam.h"

namespace wslam {

// One camera stream on the GPU: the uslam context and frontend.
class CudaFrontend {
   public:
    // brief_pattern: the 256 (ax, ay, bx, by) tests the reference compiles in
    // (generate_features.cpp:458-460, `#include "brief_tests.inc"`).
    explicit CudaFrontend(const int32_t* brief_pattern, int device = 0) : device_(device) {
        pattern_.assign(brief_pattern, brief_pattern + 1024);
    }
    CudaFrontend(const CudaFrontend&) = delete;
    CudaFrontend& operator=(const CudaFrontend&) = delete;
    ~CudaFrontend() {
        if (fe_) uslam_frontend_destroy(fe_);
        if (ctx_) uslam_destroy(ctx_);
    }

    // Context and device buffers for frames of width x height (first frame).
    std::optional<std::string> ensure(int width, int height) {
        if (fe_) {
            if (width != width_ || height != height_) return std::string("frame size changed mid-stream");
            return std::nullopt;
        }
        uslam_params p{};
        p.device = device_;
        p.levels = static_cast<int>(GPUConst::levels_of_detail);
        p.max_width = width;
        p.max_height = height;
        p.cap_per_level = 0;  // W0 * H0 / 250, GPUConst::max_features_per_lod
        p.brief_pattern = pattern_.data();
        if (uslam_status s = uslam_create(&p, &ctx_); s != USLAM_OK)
            return std::string("uslam_create: ") + uslam_status_string(s);
        if (uslam_status s = uslam_frontend_create(ctx_, width, height, &fe_); s != USLAM_OK) {
            std::string msg = std::string("uslam_frontend_create: ") + uslam_last_error(ctx_);
            uslam_destroy(ctx_);  // the next frame starts over
            ctx_ = nullptr;
            fe_ = nullptr;
            return msg;
        }
        width_ = width;
        height_ = height;
        return std::nullopt;
    }

    uslam_ctx* ctx() const { return ctx_; }
    uslam_frontend* frontend() const { return fe_; }
    int levels() const { return static_cast<int>(GPUConst::levels_of_detail); }

   private:
    int device_;
    int width_ = 0, height_ = 0;
    std::vector<int32_t> pattern_;
    uslam_ctx* ctx_ = nullptr;
    uslam_frontend* fe_ = nullptr;
};

class CudaFeatureDetectPass : public compute::Pass {
   public:
    CudaFeatureDetectPass(std::shared_ptr<CudaFrontend> gpu, AnyBag& storage)
        : gpu_(std::move(gpu)), storage_(storage) {}

    [[nodiscard]] std::string getId() const override { return "[Cuda feature detect pass]"; }
    [[nodiscard]] std::optional<std::string> initialize() override { return std::nullopt; }

    [[nodiscard]] std::optional<std::string> execute() override {
        const auto frame = storage_.getPtr<data::FrameBW>(ResourceIdentifier::GetFrameName(0));
        if (!frame) return std::string("no frame under ") + ResourceIdentifier::GetFrameName(0);
        const data::FrameBW& f = **frame;
        if (auto err = gpu_->ensure(f.width, f.height)) return err;
        // consume-once marker (common.hpp:134-142), as LoadDataCPUPass does
        const bool advance = storage_.take<bool>(ResourceIdentifier::FeatureReferenceAdvanceName).value_or(false);
        // provider_base.cpp:121-124 stored u8 / 255: the library copies the f32
        // pixels into pinned staging, uploads them as f32 (as
        // FillPyramidPass::writeBaseLayer does) and recovers each byte exactly
        // on the device
        const uslam_status s = uslam_frontend_process_f32(gpu_->frontend(), f.pixels.data(), f.width, advance ? 1 : 0);
        if (s != USLAM_OK && s != USLAM_NOT_READY)
            return std::string("uslam_frontend_process: ") + uslam_last_error(gpu_->ctx());
        auto current = download(0);
        if (!current) return std::string("feature download: ") + uslam_last_error(gpu_->ctx());
        // shiftFeatureSets (load_features_cpu.cpp:111-142), same rule as the device rotation
        const bool have_reference = storage_.has(ResourceIdentifier::GetFeatureSetName(1));
        if (!have_reference || advance) {
            if (auto prev = storage_.take<FeatureSet>(ResourceIdentifier::GetFeatureSetName(0)))
                storage_.set(ResourceIdentifier::GetFeatureSetName(1), std::move(*prev));
        }
        storage_.set(ResourceIdentifier::GetFeatureSetName(0), std::move(*current));
        return std::nullopt;
    }

   private:
    // FeatureSet from the device set (which = 0 current, 1 reference), as
    // LoadDataCPUPass::loadFeatures + FromGpuModel (models.hpp:113-120).
    std::optional<FeatureSet> download(int which) {
        const int L = gpu_->levels();
        std::vector<int> kept(L), raw(L);
        if (uslam_frontend_features(gpu_->frontend(), which, nullptr, 0, kept.data(), raw.data()) != USLAM_OK)
            return std::nullopt;
        int total = 0;
        for (int k : kept) total += k;
        std::vector<uslam_feature> buf(static_cast<size_t>(std::max(total, 1)));
        if (uslam_frontend_features(gpu_->frontend(), which, buf.data(), total, kept.data(), raw.data()) != USLAM_OK)
            return std::nullopt;
        FeatureSet set;
        size_t n = 0;
        for (int l = 0; l < L; ++l) {
            set.at(l).reserve(static_cast<size_t>(kept[l]));
            for (int i = 0; i < kept[l]; ++i, ++n) {
                const uslam_feature& g = buf[n];
                Feature c{};
                c.x = static_cast<uint32_t>(g.x);
                c.y = static_cast<uint32_t>(g.y);
                c.lod = static_cast<uint32_t>(l);
                c.strength = g.strength;
                c.orientation = g.orientation;
                std::copy(g.descriptor, g.descriptor + 8, c.descriptor.begin());
                set.at(l).push_back(c);
            }
        }
        return set;
    }

    std::shared_ptr<CudaFrontend> gpu_;
    AnyBag& storage_;
};

class CudaMatchPass : public compute::Pass {
   public:
    CudaMatchPass(std::shared_ptr<CudaFrontend> gpu, AnyBag& storage) : gpu_(std::move(gpu)), storage_(storage) {}

    [[nodiscard]] std::string getId() const override { return "[Cuda match features pass]"; }
    [[nodiscard]] std::optional<std::string> initialize() override { return std::nullopt; }

    [[nodiscard]] std::optional<std::string> execute() override {
        const auto prev = storage_.getPtr<FeatureSet>(ResourceIdentifier::GetFeatureSetName(1));
        if (!prev) return compute::kStageStopExecution;  // match_features_cpu.cpp:229-236
        const auto curr = storage_.getPtr<FeatureSet>(ResourceIdentifier::GetFeatureSetName(0));
        if (!curr) return std::string("no current feature set");
        int n = 0;
        if (uslam_frontend_matches(gpu_->frontend(), nullptr, 0, &n) != USLAM_OK)
            return std::string("uslam_frontend_matches: ") + uslam_last_error(gpu_->ctx());
        std::vector<uslam_match> buf(static_cast<size_t>(std::max(n, 1)));
        if (uslam_frontend_matches(gpu_->frontend(), buf.data(), n, &n) != USLAM_OK)
            return std::string("uslam_frontend_matches: ") + uslam_last_error(gpu_->ctx());
        // result[lod of a]: key = current-frame feature (b), value = previous (a).
        // Each level's pairs go in by ascending key with an end hint: the
        // reference's flat_map then appends instead of shifting its tail on
        // every insert, and an ordered map finds the place at once.  The
        // mutual check leaves each b at most one a, so the keys are unique
        // and the map holds the same entries as one emplace per match.
        MatchResult result;
        std::vector<std::vector<std::pair<const Feature*, const Feature*>>> by_level(result.size());
        for (int i = 0; i < n; ++i) {
            const uslam_match& m = buf[i];
            by_level.at(static_cast<size_t>(m.lod_a))
                .emplace_back(&(**curr).at(m.lod_b).at(m.idx_b), &(**prev).at(m.lod_a).at(m.idx_a));
        }
        for (size_t l = 0; l < by_level.size(); ++l) {
            auto& pairs = by_level[l];
            std::sort(pairs.begin(), pairs.end(), [](const auto& u, const auto& v) { return *u.first < *v.first; });
            auto& level = result.at(l);
            for (const auto& [b, a] : pairs) level.emplace_hint(level.end(), *b, *a);
        }
        storage_.set(ResourceIdentifier::MatchedFeaturesName, std::move(result));
        return std::nullopt;
    }

   private:
    std::shared_ptr<CudaFrontend> gpu_;
    AnyBag& storage_;
};

}  // namespace wslam
