"""The triangulation oracle (oracle/triangulate.py) pinned against the
reference's own TriangulateCPU: golden vectors made by the unmodified
triangulate_cpu.cpp (tests/golden/make_triangulate_golden.py), and, where
oracle/_ref/libref_triangulate.so was built, fresh scenes run through it.

Tolerances (binary64 throughout):
  rays (PixelToNormalised)       bit-exact: same operations in the same order;
  essential matrix               1e-9 after normalising scale and sign (the SVDs
                                 are LAPACK here, Eigen's JacobiSVD there);
  pose (R, t), rotation angle    1e-9 absolute;
  landmarks                      1e-8 x max(1, |z|) (DLT points far from the
                                 cameras amplify the rounding of the null vector);
  mean reprojection error        1e-9 relative;
  counts and the keep mask       exact.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

from oracle import triangulate as T
from tri_check import OPT_KEYS, case_opts, check_against_reference, unit_sign

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "triangulate_cases.npz")
REF_LIB = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libref_triangulate.so")


def golden_cases():
    g = np.load(GOLDEN)
    names = sorted({k.split("/")[0] for k in g.files if k != "undistort" and not k.startswith("undistort/")})
    return g, names


def test_undistort_golden_bit_exact():
    g = np.load(GOLDEN)
    rays = T.pixel_to_normalised(g["undistort/px"], g["undistort/cam"], 20, 1e-9)
    assert np.array_equal(rays.view(np.uint64), g["undistort/rays"].view(np.uint64))


@pytest.mark.parametrize("name", golden_cases()[1])
def test_oracle_matches_reference_golden(name):
    g, _ = golden_cases()
    rows, cam, opts = g[f"{name}/rows"], g[f"{name}/cam"], case_opts(g[f"{name}/opts"])
    px = rows[:, 1:5].astype(np.float64)
    res = T.triangulate(px, cam, opts)
    check_against_reference(res, g[f"{name}/pose"], g[f"{name}/stats"], g[f"{name}/keep"],
                            g[f"{name}/landmarks"], name)
    if len(rows) >= opts["min_inliers"]:
        xp = T.pixel_to_normalised(px[:, 0:2], cam, opts["undistort_iterations"], opts["undistort_tolerance"])
        xc = T.pixel_to_normalised(px[:, 2:4], cam, opts["undistort_iterations"], opts["undistort_tolerance"])
        e = T.fit_essential(xp, xc)
        np.testing.assert_allclose(unit_sign(e), unit_sign(g[f"{name}/essential"].reshape(3, 3)), atol=1e-9)
        # the four candidates as a set (their order follows each SVD's sign conventions)
        want = g[f"{name}/candidates"]
        got = np.array([np.concatenate([r.ravel(), t]) for r, t in T.decompose_essential(e)])
        for w in want:
            assert np.min(np.abs(got - w).max(1)) <= 1e-9, name


def test_below_min_inliers_is_empty():
    res = T.triangulate(np.zeros((7, 4)), np.array([400.0, 400, 300, 200, 0, 0, 0, 0]))
    assert res["input_matches"] == 7 and res["landmark_count"] == 0 and not res["pose_recovered"]
    assert np.array_equal(res["rotation"], np.eye(3)) and np.array_equal(res["translation"], np.zeros(3))


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference triangulation not built (make -C oracle)")
@pytest.mark.parametrize("seed", range(4))
def test_oracle_matches_reference_fresh(seed):
    from uni_slam_gb300 import synth
    lib = C.CDLL(REF_LIB)
    rows, cam, _, _ = synth.two_view_scene(seed=900 + seed, n=200 + 150 * seed, outlier_frac=0.01 * (seed % 2))
    opts = np.array([float(T.DEFAULT_OPTS[k]) for k in OPT_KEYS])
    n = len(rows)
    pose, st, keep, lm = np.zeros(12), np.zeros(6), np.zeros(n, np.int32), np.zeros((n, 4))
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    assert lib.ref_triangulate(p(rows), C.c_int(n), p(cam), p(opts), p(pose), p(st), p(keep), p(lm)) >= 0
    res = T.triangulate(rows[:, 1:5].astype(np.float64), cam)
    check_against_reference(res, pose, st, keep, lm, f"seed {seed}")
