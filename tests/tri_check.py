"""Shared checks of triangulation results against the reference's
(TriangulateCPU, wslam/src/pose_estimate_cpu/triangulate_cpu.cpp), used by the
oracle pins and the GPU parity tests.  Tolerances are stated in
test_oracle_triangulate.py."""
from __future__ import annotations

import numpy as np

OPT_KEYS = ("max_reprojection_px", "min_depth", "max_depth", "min_inliers", "undistort_iterations",
            "undistort_tolerance")


def case_opts(opts: np.ndarray) -> dict:
    o = dict(zip(OPT_KEYS, (float(v) for v in opts)))
    o["min_inliers"] = int(o["min_inliers"])
    o["undistort_iterations"] = int(o["undistort_iterations"])
    return o


def unit_sign(m: np.ndarray) -> np.ndarray:
    m = m / np.linalg.norm(m)
    return m * np.sign(m.flat[np.argmax(np.abs(m))])


def check_against_reference(res: dict, pose, stats, keep, lm, tag: str):
    """The TriangulationResult of res (oracle or GPU) against the reference's."""
    assert res["input_matches"] == int(stats[0]), tag
    assert res["landmark_count"] == int(stats[1]), tag
    assert res["cheirality_passes"] == int(stats[2]), tag
    assert bool(res["pose_recovered"]) == bool(stats[4]), tag
    np.testing.assert_allclose(res["rotation"], np.asarray(pose[:9]).reshape(3, 3), rtol=0, atol=1e-9, err_msg=tag)
    np.testing.assert_allclose(res["translation"], pose[9:12], rtol=0, atol=1e-9, err_msg=tag)
    assert abs(res["rotation_angle_rad"] - stats[5]) <= 1e-9, tag
    assert abs(res["mean_reprojection_error_px"] - stats[3]) <= 1e-9 * max(1.0, abs(stats[3])), tag
    k = np.asarray(keep).astype(bool)
    assert np.array_equal(np.asarray(res["keep"]).astype(bool), k), tag
    got = np.asarray(res["landmarks"])[k]
    want = np.asarray(lm)[k]
    scale = np.maximum(1.0, np.abs(want[:, 2:3]))
    assert np.all(np.abs(got[:, :3] - want[:, :3]) <= 1e-8 * scale), tag
    assert np.all(np.abs(got[:, 3] - want[:, 3]) <= 1e-8 * np.maximum(1.0, want[:, 3])), tag
    assert np.all(np.asarray(res["landmarks"])[~k] == 0.0), tag
