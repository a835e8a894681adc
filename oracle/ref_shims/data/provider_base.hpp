// Minimal restatement of the sensor types of data/include/data/provider_base.hpp:27-76
// (same members) for compiling the reference's triangulation pass.  Test infrastructure.
#pragma once
#include <Eigen/Dense>
#include <array>
#include <cstdint>
#include <string>

namespace wslam::data {
struct CamSensorParams {
    Eigen::Matrix4d T_BS;
    uint32_t rate_hz;
    std::array<int, 2> resolution;
    std::string camera_model;
    Eigen::Vector4d intrinsics;  // [fu, fv, cu, cv]
    std::string distortion_model;
    Eigen::Vector4d distortion_coefficients;
};

struct IMUReading {
    uint64_t timestamp;
    Eigen::Matrix<float, 6, 1> vals;
    [[nodiscard]] float wx() const { return vals[0]; }
    [[nodiscard]] float wy() const { return vals[1]; }
    [[nodiscard]] float wz() const { return vals[2]; }
};
}  // namespace wslam::data
