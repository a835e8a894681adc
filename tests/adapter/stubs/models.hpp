// Test stand-in for wslam/src/models.hpp (CPU feature types, same members).
#pragma once
#include <array>
#include <compare>
#include <cstdint>
#include <map>
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
    constexpr auto operator<=>(const Feature&) const = default;
    constexpr bool operator==(const Feature&) const = default;
};
using FeatureSet = std::array<std::vector<Feature>, GPUConst::levels_of_detail>;
using MatchResult = std::array<std::map<Feature, Feature>, GPUConst::levels_of_detail>;
}  // namespace wslam
