"""Regenerate tests/golden/triangulate_cases.npz (run where the reference
checkout is present, after `make -C oracle`).

Every case is a seeded two-view scene (uni_slam_gb300.synth.two_view_scene)
passed through the reference's own triangulation pass,
wslam/src/pose_estimate_cpu/triangulate_cpu.cpp compiled unmodified with the
Eigen bundled in its gtsam (oracle/_ref/libref_triangulate.so, see
oracle/ref_tri_harness.cpp).  Stored per case: the rows, camera and options,
TriangulationResult (pose, stats, per-row keep and landmarks), the
reference's essential matrix and four pose candidates for those rays, and
for 256 pixels the reference's PixelToNormalised.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import triangulate as T  # noqa: E402
from uni_slam_gb300 import synth  # noqa: E402

LIB = os.path.join(REPO, "oracle", "_ref", "libref_triangulate.so")
OPT_KEYS = ("max_reprojection_px", "min_depth", "max_depth", "min_inliers", "undistort_iterations",
            "undistort_tolerance")

# name -> (two_view_scene kwargs, option overrides)
CASES = {
    "mixed_300": (dict(seed=301, n=300, outlier_frac=0.01), {}),
    "mixed_800": (dict(seed=305, n=800, outlier_frac=0.01), {}),
    "clean_500": (dict(seed=310, n=500), {}),
    "minimal_8": (dict(seed=103, n=8), {}),
    "below_min_7": (dict(seed=103, n=7), {}),
    "pure_rotation": (dict(seed=105, n=300, baseline=0.0), {}),
    "strict_opts": (dict(seed=104, n=500, outlier_frac=0.01), dict(max_reprojection_px=1.0, min_depth=5.0,
                                                                    max_depth=20.0)),
    "far_points": (dict(seed=106, n=400, depth=(100.0, 900.0)), {}),
    "two_undistort_iters": (dict(seed=108, n=300, outlier_frac=0.01), dict(undistort_iterations=2)),
    "tiny_baseline": (dict(seed=109, n=300, baseline=0.01), {}),
    "wide_rotation": (dict(seed=204, n=500, rot_sigma=0.05), {}),
}


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def main():
    lib = C.CDLL(LIB)
    lib.ref_pixel_to_normalised.argtypes = [C.c_double, C.c_double, C.c_void_p, C.c_uint32, C.c_double, C.c_void_p]
    out = {}
    for name, (kw, ov) in CASES.items():
        rows, cam, _, _ = synth.two_view_scene(**kw)
        o = dict(T.DEFAULT_OPTS, **ov)
        opts = np.array([float(o[k]) for k in OPT_KEYS])
        n = len(rows)
        pose, st = np.zeros(12), np.zeros(6)
        keep, lm = np.zeros(n, np.int32), np.zeros((n, 4))
        rc = lib.ref_triangulate(_p(rows), C.c_int(n), _p(cam), _p(opts), _p(pose), _p(st), _p(keep), _p(lm))
        assert rc >= 0, (name, rc)
        rays = np.zeros((n, 4))
        one = np.zeros(2)
        for i in range(n):
            for j, (x, y) in enumerate(((rows[i, 1], rows[i, 2]), (rows[i, 3], rows[i, 4]))):
                lib.ref_pixel_to_normalised(float(x), float(y), _p(cam), int(o["undistort_iterations"]),
                                            float(o["undistort_tolerance"]), _p(one))
                rays[i, 2 * j:2 * j + 2] = one
        e = np.zeros(9)
        cands = np.zeros(48)
        fit = 0
        if n >= 8:
            xp, xc = np.ascontiguousarray(rays[:, 0:2]), np.ascontiguousarray(rays[:, 2:4])
            fit = lib.ref_fit_essential(_p(xp), _p(xc), C.c_int(n), _p(e))
            if fit:
                lib.ref_decompose_essential(_p(e), _p(cands))
        out[f"{name}/rows"] = rows
        out[f"{name}/cam"] = cam
        out[f"{name}/opts"] = opts
        out[f"{name}/pose"] = pose
        out[f"{name}/stats"] = st
        out[f"{name}/keep"] = keep.astype(np.uint8)
        out[f"{name}/landmarks"] = lm
        out[f"{name}/essential"] = e
        out[f"{name}/candidates"] = cands.reshape(4, 12)
        print(f"{name}: n={n} landmarks={int(st[1])} cheirality={int(st[2])} fit={fit}")
    # undistortion pins over the whole frame
    rs = np.random.default_rng(7)
    px = np.concatenate([rs.uniform(0, [752, 480], (240, 2)),
                         np.array([[0, 0], [751, 0], [0, 479], [751, 479], [376, 240], [375.5, 239.5],
                                   [0, 240], [751, 240], [376, 0], [376, 479], [100.25, 50.75], [700, 400],
                                   [1, 1], [750, 478], [10, 470], [740, 12]], float)])
    ref = np.zeros_like(px)
    one = np.zeros(2)
    for i, (x, y) in enumerate(px):
        lib.ref_pixel_to_normalised(float(x), float(y), _p(synth.SCENE_CAMERA), 20, 1e-9, _p(one))
        ref[i] = one
    out["undistort/px"] = px
    out["undistort/cam"] = synth.SCENE_CAMERA.copy()
    out["undistort/rays"] = ref
    np.savez_compressed(os.path.join(HERE, "triangulate_cases.npz"), **out)


if __name__ == "__main__":
    main()
