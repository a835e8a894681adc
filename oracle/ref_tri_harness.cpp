// ref_tri_harness.cpp — C entry points around the reference's own triangulation
// pass (TEST INFRASTRUCTURE ONLY).
//
// wslam/src/pose_estimate_cpu/triangulate_cpu.cpp is included unmodified (the
// Makefile puts its directory, wslam/src and the Eigen bundled with the
// reference's gtsam on the include path; oracle/ref_shims stands in for the
// Dawn- and spdlog-dependent headers).  Including the .cpp makes its
// anonymous-namespace helpers callable, so the oracle can be pinned stage by
// stage as well as through TriangulateCPU::execute().
#include "triangulate_cpu.cpp"

#include <cstring>

namespace {
wslam::data::CamSensorParams MakeCam(const double* cam) {
    wslam::data::CamSensorParams c{};
    c.intrinsics = Eigen::Vector4d(cam[0], cam[1], cam[2], cam[3]);
    c.distortion_coefficients = Eigen::Vector4d(cam[4], cam[5], cam[6], cam[7]);
    return c;
}

wslam::Feature MakeFeature(uint32_t x, uint32_t y, uint32_t lod, uint32_t tag) {
    wslam::Feature f{};
    f.x = x;
    f.y = y;
    f.lod = lod;
    f.strength = tag;  // carries the input index through the pass
    return f;
}
}  // namespace

// util::PixelToNormalised (wslam/src/map/map_helpers_lods.hpp:110-120).
extern "C" void ref_pixel_to_normalised(double px, double py, const double* cam, uint32_t iters,
                                        double tol, double* out) {
    const auto c = MakeCam(cam);
    const Eigen::Vector2d r = wslam::map::util::PixelToNormalised(
        Eigen::Vector2d(px, py), c.intrinsics, c.distortion_coefficients, iters, tol);
    out[0] = r.x();
    out[1] = r.y();
}

// impl::FitEssentialMatrix (triangulate_cpu.cpp:77-140); E row-major.
extern "C" int ref_fit_essential(const double* xy_prev, const double* xy_curr, int n, double* e_out) {
    std::vector<Eigen::Vector2d> p, q;
    for (int i = 0; i < n; ++i) {
        p.emplace_back(xy_prev[2 * i], xy_prev[2 * i + 1]);
        q.emplace_back(xy_curr[2 * i], xy_curr[2 * i + 1]);
    }
    const auto e = impl::FitEssentialMatrix(p, q);
    if (!e) return 0;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) e_out[3 * r + c] = (*e)(r, c);
    return 1;
}

// impl::DecomposeEssential (triangulate_cpu.cpp:149-172): 4 x (R row-major, t).
extern "C" void ref_decompose_essential(const double* e_in, double* out) {
    Eigen::Matrix3d e;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) e(r, c) = e_in[3 * r + c];
    const auto cands = impl::DecomposeEssential(e);
    for (int k = 0; k < 4; ++k) {
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) out[12 * k + 3 * r + c] = cands[k].r(r, c);
        for (int r = 0; r < 3; ++r) out[12 * k + 9 + r] = cands[k].t(r);
    }
}

// impl::TriangulatePoint (triangulate_cpu.cpp:180-207); pose = R row-major, t.
extern "C" int ref_triangulate_point(const double* pose, const double* xy_prev, const double* xy_curr,
                                     double* out) {
    Eigen::Matrix3d r;
    for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c) r(i, c) = pose[3 * i + c];
    const Eigen::Vector3d t(pose[9], pose[10], pose[11]);
    const auto p = impl::TriangulatePoint(r, t, Eigen::Vector2d(xy_prev[0], xy_prev[1]),
                                          Eigen::Vector2d(xy_curr[0], xy_curr[1]));
    if (!p) return 0;
    out[0] = p->x();
    out[1] = p->y();
    out[2] = p->z();
    return 1;
}

// TriangulateCPU::execute (triangulate_cpu.cpp:342-513) through the pass's
// own AnyBag interface.  corr: n rows of (lod, prev_x, prev_y, curr_x, curr_y),
// each current feature unique within its level.  cam: fu, fv, cu, cv, k1, k2,
// p1, p2.  opts: max_reprojection_px, min_depth, max_depth, min_inliers,
// undistort_iterations, undistort_tolerance.
// pose_out: R row-major, t.  stats_out: input_matches, landmark_count,
// cheirality_passes, mean_reprojection_error_px, pose_recovered,
// rotation_angle_rad.  keep[i] / lm[4 i..4 i + 3] (x, y, z in the current
// camera, reprojection error) for each input row that became a landmark.
extern "C" int ref_triangulate(const uint32_t* corr, int n, const double* cam, const double* opts,
                               double* pose_out, double* stats_out, int* keep, double* lm) {
    AnyBag storage;
    wslam::RansacResult ransac{};
    for (int i = 0; i < n; ++i) {
        const uint32_t* c = corr + 5 * i;
        const auto prev = MakeFeature(c[1], c[2], c[0], static_cast<uint32_t>(i));
        const auto curr = MakeFeature(c[3], c[4], c[0], static_cast<uint32_t>(i));
        if (!ransac.inliers.at(c[0]).emplace(curr, prev).second) return -1;
    }
    ransac.stats.total_matches = static_cast<size_t>(n);
    ransac.stats.inlier_count = static_cast<size_t>(n);
    ransac.stats.model_found = true;
    storage.set(wslam::ResourceIdentifier::RansacResultName, std::move(ransac));
    storage.set(wslam::ResourceIdentifier::GetCameraIntrinsicsName(0), MakeCam(cam));

    wslam::TriangulateCPU::Opts o{};
    o.max_reprojection_px = opts[0];
    o.min_depth = opts[1];
    o.max_depth = opts[2];
    o.min_inliers = static_cast<size_t>(opts[3]);
    o.undistort_iterations = static_cast<uint32_t>(opts[4]);
    o.undistort_tolerance = opts[5];
    wslam::TriangulateCPU pass(storage, o);
    if (pass.initialize() || pass.execute()) return -2;
    auto res = storage.getPtr<wslam::TriangulationResult>(wslam::ResourceIdentifier::TriangulationResultName);
    if (!res) return -3;
    const auto& t = **res;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) pose_out[3 * r + c] = t.rotation(r, c);
    for (int r = 0; r < 3; ++r) pose_out[9 + r] = t.translation(r);
    stats_out[0] = static_cast<double>(t.stats.input_matches);
    stats_out[1] = static_cast<double>(t.stats.landmark_count);
    stats_out[2] = static_cast<double>(t.stats.cheirality_passes);
    stats_out[3] = t.stats.mean_reprojection_error_px;
    stats_out[4] = t.stats.pose_recovered ? 1.0 : 0.0;
    stats_out[5] = t.stats.rotation_angle_rad;
    std::memset(keep, 0, sizeof(int) * static_cast<size_t>(n));
    for (const auto& l : t.landmarks) {
        const int i = static_cast<int>(l.feat_curr.strength);
        keep[i] = 1;
        lm[4 * i + 0] = l.position_cam_curr.x();
        lm[4 * i + 1] = l.position_cam_curr.y();
        lm[4 * i + 2] = l.position_cam_curr.z();
        lm[4 * i + 3] = l.reprojection_error_px;
    }
    return static_cast<int>(t.landmarks.size());
}
