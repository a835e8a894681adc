// Minimal restatement of the CPU feature types of wslam/src/models.hpp:86-129
// (same members, same defaulted comparisons) for compiling the reference
// matcher, and, where Eigen is on the include path, the RANSAC and
// triangulation result types of wslam/src/models.hpp:132-184 for compiling
// the reference's triangulation pass.  Test infrastructure.
#pragma once
#include <array>
#include <cassert>
#include <compare>
#include <cstdint>
#include <flat_map>
#include <vector>

#include "common.hpp"

namespace wslam {
struct Feature {
    uint32_t x;
    uint32_t y;
    uint32_t lod;
    uint32_t strength;
    float orientation;
    std::array<uint32_t, 8> descriptor;
    static constexpr size_t kDescriptorBits = 256;
    constexpr auto operator<=>(const Feature&) const = default;
    constexpr bool operator==(const Feature&) const = default;
};
using FeatureSet = std::array<std::vector<Feature>, GPUConst::levels_of_detail>;
using MatchResult = std::array<std::flat_map<Feature, Feature>, GPUConst::levels_of_detail>;
}  // namespace wslam

#if __has_include(<Eigen/Dense>)
#include <Eigen/Dense>
namespace wslam {
struct RansacStats {
    size_t total_matches = 0;
    size_t inlier_count = 0;
    size_t iterations_run = 0;
    bool model_found = false;
};
struct RansacResult {
    MatchResult inliers;
    std::array<std::array<double, 3>, 3> fundamental_matrix{};
    RansacStats stats;
};
struct Landmark {
    Eigen::Vector3d position_cam_curr;
    Feature feat_prev;
    Feature feat_curr;
    double reprojection_error_px;
};
struct TriangulationStats {
    size_t input_matches = 0;
    size_t landmark_count = 0;
    size_t cheirality_passes = 0;
    double mean_reprojection_error_px = 0.0;
    bool pose_recovered = false;
    double rotation_angle_rad = 0.0;
};
struct TriangulationResult {
    Eigen::Matrix3d rotation = Eigen::Matrix3d::Identity();
    Eigen::Vector3d translation = Eigen::Vector3d::Zero();
    std::vector<Landmark> landmarks;
    TriangulationStats stats;
};
}  // namespace wslam
#endif
