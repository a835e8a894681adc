// Times CudaFeatureDetectPass + CudaMatchPass the way the reference's stages
// run them: per frame a FrameBW of f32 pixels (u8 / 255, the reference's
// data::getLocalFrame rule) in AnyBag, the detect pass, then the match pass,
// with the FeatureSet and MatchResult outputs built in AnyBag.  Frames are
// reused cyclically; a keyframe advance every `advance_every` frames.
//   adapter_bench <pattern.bin> <frames.bin> <warmup> <frames_timed> <advance_every>
// frames.bin as for adapter_main (advance flags ignored).  Prints one JSON
// line: timed frames, seconds, frames/s, features and matches seen.
#include <chrono>
#include <cstdio>
#include <fstream>
#include <iostream>

#include "uslam_wslam.hpp"

int main(int argc, char** argv) {
    if (argc != 6) return 2;
    std::ifstream pf(argv[1], std::ios::binary);
    std::vector<int32_t> pattern(1024);
    pf.read(reinterpret_cast<char*>(pattern.data()), 4096);
    std::ifstream ff(argv[2], std::ios::binary);
    int32_t hdr[3];
    ff.read(reinterpret_cast<char*>(hdr), sizeof hdr);
    const int n = hdr[0], w = hdr[1], h = hdr[2];
    const int warmup = std::atoi(argv[3]), timed = std::atoi(argv[4]), advance_every = std::atoi(argv[5]);
    std::vector<std::vector<float>> frames(n);
    for (int i = 0; i < n; ++i) {
        int32_t adv;
        ff.read(reinterpret_cast<char*>(&adv), 4);
        std::vector<uint8_t> img(static_cast<size_t>(w) * h);
        ff.read(reinterpret_cast<char*>(img.data()), img.size());
        frames[i].resize(img.size());
        for (size_t k = 0; k < img.size(); ++k) frames[i][k] = static_cast<float>(img[k]) / 255.0f;
    }
    AnyBag storage;
    auto gpu = std::make_shared<wslam::CudaFrontend>(pattern.data());
    wslam::CudaFeatureDetectPass detect(gpu, storage);
    wslam::CudaMatchPass match(gpu, storage);
    if (detect.initialize() || match.initialize()) return 3;
    long long feats = 0, matches = 0;
    double seconds = 0.0, detect_s = 0.0;
    for (int i = 0; i < warmup + timed; ++i) {
        // the frame's pixels are copied into the FrameBW outside the time, as
        // the sensor loader pass would have stored them before this stage
        data::FrameBW frame{static_cast<uint64_t>(i), frames[i % n], static_cast<uint16_t>(w),
                            static_cast<uint16_t>(h)};
        storage.set(wslam::ResourceIdentifier::GetFrameName(0), std::move(frame));
        if (advance_every > 0 && i % advance_every == 0)
            storage.set(wslam::ResourceIdentifier::FeatureReferenceAdvanceName, true);
        const auto t0 = std::chrono::steady_clock::now();
        if (auto e = detect.execute()) {
            std::cerr << "detect: " << *e << "\n";
            return 4;
        }
        const auto td = std::chrono::steady_clock::now();
        const auto me = match.execute();
        const auto t1 = std::chrono::steady_clock::now();
        const bool stop = me && *me == wslam::compute::kStageStopExecution;
        if (me && !stop) {
            std::cerr << "match: " << *me << "\n";
            return 5;
        }
        if (i >= warmup) {
            seconds += std::chrono::duration<double>(t1 - t0).count();
            detect_s += std::chrono::duration<double>(td - t0).count();
            const auto& cur = **storage.getPtr<wslam::FeatureSet>(wslam::ResourceIdentifier::GetFeatureSetName(0));
            for (const auto& lv : cur) feats += static_cast<long long>(lv.size());
            if (!stop) {
                const auto& mr = **storage.getPtr<wslam::MatchResult>(wslam::ResourceIdentifier::MatchedFeaturesName);
                for (const auto& m : mr) matches += static_cast<long long>(m.size());
            }
        }
    }
    std::printf(
        "{\"frames\": %d, \"seconds\": %.6f, \"frames_per_s\": %.3f, \"detect_pass_ms\": %.4f, "
        "\"match_pass_ms\": %.4f, \"features\": %lld, \"matches\": %lld}\n",
        timed, seconds, timed / seconds, 1e3 * detect_s / timed, 1e3 * (seconds - detect_s) / timed, feats, matches);
    return 0;
}
