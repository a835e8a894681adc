// Test stand-in for data::FrameBW (data/include/data/provider_base.hpp:57-62).
#pragma once
#include <cstdint>
#include <vector>
namespace data {
struct FrameBW {
    uint64_t timestamp;
    std::vector<float> pixels;
    uint16_t width;
    uint16_t height;
};
}  // namespace data
