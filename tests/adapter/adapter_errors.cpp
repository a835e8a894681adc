// Error paths of CudaFeatureDetectPass / CudaMatchPass that need no GPU work:
// each line printed is "<case>: <result>", where the result is "ok" for
// std::nullopt and the returned string otherwise.
//   adapter_errors <pattern.bin>
#include <fstream>
#include <iostream>

#include "uslam_wslam.hpp"

namespace {
void show(const char* name, const std::optional<std::string>& r) {
    std::cout << name << ": " << (r ? *r : std::string("ok")) << "\n";
}
}  // namespace

int main(int argc, char** argv) {
    if (argc != 2) return 2;
    std::ifstream pf(argv[1], std::ios::binary);
    std::vector<int32_t> pattern(1024);
    pf.read(reinterpret_cast<char*>(pattern.data()), 4096);

    AnyBag storage;
    auto gpu = std::make_shared<wslam::CudaFrontend>(pattern.data());
    wslam::CudaFeatureDetectPass detect(gpu, storage);
    wslam::CudaMatchPass match(gpu, storage);
    std::cout << "ids: " << detect.getId() << " | " << match.getId() << "\n";
    show("init", detect.initialize() ? detect.initialize() : match.initialize());
    // match_features_cpu.cpp:229-236: no reference set yet -> the stage sentinel
    show("match_without_reference", match.execute());
    // a reference set but no current set
    storage.set(wslam::ResourceIdentifier::GetFeatureSetName(1), wslam::FeatureSet{});
    show("match_without_current", match.execute());
    // no frame in the bag
    show("detect_without_frame", detect.execute());
    // a frame: runs on a GPU, or reports the failed context creation without one
    data::FrameBW frame{0, {}, 64, 48};
    frame.pixels.assign(64 * 48, 0.5f);
    storage.set(wslam::ResourceIdentifier::GetFrameName(0), std::move(frame));
    show("detect_with_frame", detect.execute());
    return 0;
}
