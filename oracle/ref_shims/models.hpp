// Minimal restatement of the CPU feature types of wslam/src/models.hpp:86-129
// (same members, same defaulted comparisons) for compiling the reference
// matcher.  Test infrastructure.
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
