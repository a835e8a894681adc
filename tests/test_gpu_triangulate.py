"""Batched two-view triangulation on the GPU (uslam_triangulate,
uslam_pixel_to_normalised) against the reference's own TriangulateCPU
(golden vectors from triangulate_cpu.cpp) and the oracle restatement, with
the tolerances stated in test_oracle_triangulate.py: rays bit-exact, pose
1e-9, landmarks 1e-8 x max(1, |z|), counts and keep masks exact."""
import os

import numpy as np
import pytest

from oracle import triangulate as T
from tri_check import case_opts, check_against_reference
from uni_slam_gb300 import Context, USlamError, synth

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "triangulate_cases.npz")


@pytest.fixture(scope="module")
def ctx(brief_pattern):
    with Context(brief_pattern, levels=6, max_width=752, max_height=480) as c:
        yield c


def test_rays_bit_exact(ctx):
    g = np.load(GOLDEN)
    rays = ctx.pixel_to_normalised(g["undistort/px"], g["undistort/cam"], 20, 1e-9)
    assert np.array_equal(rays.view(np.uint64), g["undistort/rays"].view(np.uint64))
    # every pixel of two of the golden scenes, both views, other iteration limits
    for name in ("mixed_800", "two_undistort_iters"):
        rows, cam, o = g[f"{name}/rows"], g[f"{name}/cam"], case_opts(g[f"{name}/opts"])
        px = rows[:, 1:5].astype(np.float64).reshape(-1, 2)
        want = T.pixel_to_normalised(px, cam, o["undistort_iterations"], o["undistort_tolerance"])
        got = ctx.pixel_to_normalised(px, cam, o["undistort_iterations"], o["undistort_tolerance"])
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), name


def test_golden_cases_batched(ctx):
    """All golden scenes in as few calls as their options allow (one call per
    distinct option set), each pair against the reference's result."""
    g = np.load(GOLDEN)
    names = sorted({k.split("/")[0] for k in g.files if not k.startswith("undistort/")})
    groups = {}
    for name in names:
        groups.setdefault(tuple(g[f"{name}/opts"]), []).append(name)
    for opts, group in groups.items():
        o = case_opts(np.array(opts))
        cam = g[f"{group[0]}/cam"]
        assert all(np.array_equal(g[f"{n}/cam"], cam) for n in group)
        res = ctx.triangulate([g[f"{n}/rows"][:, 1:5].astype(np.float64) for n in group], cam, o)
        for name, r in zip(group, res):
            check_against_reference(r, g[f"{name}/pose"], g[f"{name}/stats"], g[f"{name}/keep"],
                                    g[f"{name}/landmarks"], name)


def test_many_pairs_against_oracle(ctx):
    """24 seeded scenes of mixed sizes (including empty, 7-row and 8-row
    pairs) in one call, each against the oracle."""
    parts, cam = [], synth.SCENE_CAMERA
    sizes = [1500, 0, 7, 8, 33, 640, 1200, 300] * 3
    for k, n in enumerate(sizes):
        rows, _, _, _ = synth.two_view_scene(seed=500 + k, n=max(n, 1), outlier_frac=0.01 * (k % 3),
                                             rot_sigma=0.01 + 0.01 * (k % 4))
        parts.append(rows[:n, 1:5].astype(np.float64))
    res = ctx.triangulate(parts, cam)
    assert len(res) == len(parts)
    for k, (px, r) in enumerate(zip(parts, res)):
        want = T.triangulate(px, cam)
        pose = np.concatenate([want["rotation"].ravel(), want["translation"]])
        stats = [want["input_matches"], want["landmark_count"], want["cheirality_passes"],
                 want["mean_reprojection_error_px"], want["pose_recovered"], want["rotation_angle_rad"]]
        check_against_reference(r, pose, stats, want["keep"], want["landmarks"], f"pair {k} n={len(px)}")


def test_deterministic_and_single_pair(ctx):
    rows, cam, _, _ = synth.two_view_scene(seed=77, n=1000, outlier_frac=0.01)
    px = rows[:, 1:5].astype(np.float64)
    a = ctx.triangulate(px, cam)
    b = ctx.triangulate([px, px], cam)
    for r in b:
        assert np.array_equal(r["landmarks"].view(np.uint64), a["landmarks"].view(np.uint64))
        assert np.array_equal(r["rotation"].view(np.uint64), a["rotation"].view(np.uint64))
        assert r["landmark_count"] == a["landmark_count"]


def test_edge_calls(ctx):
    cam = synth.SCENE_CAMERA
    assert ctx.triangulate([], cam) == []
    r = ctx.triangulate(np.zeros((5, 4)), cam)
    assert r["input_matches"] == 5 and r["landmark_count"] == 0 and not r["pose_recovered"]
    assert np.array_equal(r["rotation"], np.eye(3))
    with pytest.raises(USlamError):
        ctx.triangulate(np.zeros((10, 4)), cam, {"min_inliers": 4})
    assert ctx.pixel_to_normalised(np.zeros((0, 2)), cam).shape == (0, 2)
