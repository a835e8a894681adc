// ref_ransac_harness.cpp — a C entry point around the reference's own RANSAC
// inlier test (TEST INFRASTRUCTURE ONLY).
//
// wslam/src/pose_estimate_cpu/ransac_cpu.cpp is included unmodified (the
// Makefile puts its directory, wslam/src and the Eigen bundled with the
// reference's gtsam on the include path; oracle/ref_shims stands in for the
// Dawn- and spdlog-dependent headers).  Including the .cpp makes its
// anonymous-namespace helpers callable: SampsonDistance (:183-196) and
// ClassifyInliers (:198-210).
#include "ransac_cpu.cpp"

#include <cstring>

// For each of n_hyp row-major 3x3 matrices: the inlier count, the inlier
// bitmask (bit i of word i / 32) and, if dist is not NULL, the Sampson
// distance of every correspondence, all from the reference's functions.
extern "C" void ref_sampson_classify(const double* fmats, int n_hyp, const double* prev_xy, const double* curr_xy,
                                     int n, double threshold, int* counts, uint32_t* masks, double* dist) {
    std::vector<impl::FlatMatch> m(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) {
        m[i].prev = Eigen::Vector2d(prev_xy[2 * i], prev_xy[2 * i + 1]);
        m[i].curr = Eigen::Vector2d(curr_xy[2 * i], curr_xy[2 * i + 1]);
    }
    const int words = (n + 31) / 32;
    for (int h = 0; h < n_hyp; ++h) {
        Eigen::Matrix3d f;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) f(r, c) = fmats[static_cast<size_t>(h) * 9 + 3 * r + c];
        const std::vector<size_t> in = impl::ClassifyInliers(f, m, threshold);
        counts[h] = static_cast<int>(in.size());
        uint32_t* mk = masks + static_cast<size_t>(h) * words;
        std::memset(mk, 0, sizeof(uint32_t) * static_cast<size_t>(words));
        for (size_t i : in) mk[i / 32] |= 1u << (i % 32);
        if (dist)
            for (int i = 0; i < n; ++i)
                dist[static_cast<size_t>(h) * n + i] = impl::SampsonDistance(f, m[i].prev, m[i].curr);
    }
}
