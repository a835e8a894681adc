// Drives CudaFeatureDetectPass + CudaMatchPass the way the reference's stages
// run them, over frames from a file, and writes every frame's FeatureSet(0)
// and MatchResult for the Python test to compare.
//   adapter_main <pattern.bin> <frames.bin> <out.bin>
// frames.bin: int32 n, width, height, then n records of (int32 advance, u8[h*w]).
// out.bin per frame: int32 status(0 ok / 1 stage stop), int32 nfeat[6],
// features (x, y, lod, strength u32, orientation f32, desc u32[8]),
// int32 nmatch, nmatch x (lod_b, x_b, y_b, lod_a, x_a, y_a) int32.
#include <cstdio>
#include <fstream>
#include <iostream>

#include "uslam_wslam.hpp"

int main(int argc, char** argv) {
    if (argc != 4) return 2;
    std::ifstream pf(argv[1], std::ios::binary);
    std::vector<int32_t> pattern(1024);
    pf.read(reinterpret_cast<char*>(pattern.data()), 4096);
    std::ifstream ff(argv[2], std::ios::binary);
    int32_t hdr[3];
    ff.read(reinterpret_cast<char*>(hdr), sizeof hdr);
    const int n = hdr[0], w = hdr[1], h = hdr[2];
    std::ofstream of(argv[3], std::ios::binary);
    auto put = [&](int32_t v) { of.write(reinterpret_cast<const char*>(&v), 4); };

    AnyBag storage;
    auto gpu = std::make_shared<wslam::CudaFrontend>(pattern.data());
    wslam::CudaFeatureDetectPass detect(gpu, storage);
    wslam::CudaMatchPass match(gpu, storage);
    if (detect.initialize() || match.initialize()) return 3;
    for (int i = 0; i < n; ++i) {
        int32_t adv;
        ff.read(reinterpret_cast<char*>(&adv), 4);
        std::vector<uint8_t> img(static_cast<size_t>(w) * h);
        ff.read(reinterpret_cast<char*>(img.data()), img.size());
        data::FrameBW frame{static_cast<uint64_t>(i), {}, static_cast<uint16_t>(w), static_cast<uint16_t>(h)};
        frame.pixels.resize(img.size());
        for (size_t k = 0; k < img.size(); ++k) frame.pixels[k] = static_cast<float>(img[k]) / 255.0f;
        storage.set(wslam::ResourceIdentifier::GetFrameName(0), std::move(frame));
        if (adv) storage.set(wslam::ResourceIdentifier::FeatureReferenceAdvanceName, true);
        if (auto e = detect.execute()) {
            std::cerr << "detect: " << *e << "\n";
            return 4;
        }
        const auto me = match.execute();
        const bool stop = me && *me == wslam::compute::kStageStopExecution;
        if (me && !stop) {
            std::cerr << "match: " << *me << "\n";
            return 5;
        }
        put(stop ? 1 : 0);
        const auto& cur = **storage.getPtr<wslam::FeatureSet>(wslam::ResourceIdentifier::GetFeatureSetName(0));
        for (const auto& lv : cur) put(static_cast<int32_t>(lv.size()));
        for (const auto& lv : cur)
            for (const auto& f : lv) of.write(reinterpret_cast<const char*>(&f), sizeof f);
        if (stop) {
            put(0);
            continue;
        }
        const auto& mr = **storage.getPtr<wslam::MatchResult>(wslam::ResourceIdentifier::MatchedFeaturesName);
        int32_t nm = 0;
        for (const auto& m : mr) nm += static_cast<int32_t>(m.size());
        put(nm);
        for (const auto& m : mr)
            for (const auto& [b, a] : m) {
                put(b.lod); put(b.x); put(b.y); put(a.lod); put(a.x); put(a.y);
            }
    }
    return 0;
}
