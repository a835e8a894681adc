"""Regenerate tests/golden/ransac_cases.npz (run where the reference
checkout is present, after `make -C oracle`).

Every case is a seeded two-view scene (tests/test_oracle_ransac.two_view:
a true fundamental matrix, exact correspondences and planted outliers) plus
random and degenerate matrices, scored by the reference's own inlier test,
SampsonDistance and ClassifyInliers of
wslam/src/pose_estimate_cpu/ransac_cpu.cpp compiled unmodified with the
Eigen bundled in its gtsam (oracle/_ref/libref_ransac.so, see
oracle/ref_ransac_harness.cpp).  Stored per case: the matrices, the
correspondences, the threshold, and the reference's counts, inlier masks and
Sampson distances.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from test_oracle_ransac import two_view  # noqa: E402

# name -> (scene seed, random matrices, threshold)
CASES = {
    "scene0_thr3.84": (0, 12, 3.84),
    "scene1_thr1": (1, 12, 1.0),
    "scene2_thr3.84": (2, 12, 3.84),
    "scene3_thr10": (3, 12, 10.0),
}


def main():
    ref = oracle.ref_sampson()
    if ref is None:
        raise SystemExit("oracle/_ref/libref_ransac.so is missing: run `make -C oracle` with the reference checkout")
    out = {}
    for name, (seed, n_rand, thr) in CASES.items():
        rs = np.random.RandomState(1000 + seed)
        F, p, q = two_view(np.random.RandomState(seed))
        near = F + rs.normal(scale=1e-9, size=(3, 3))  # many distances close to the threshold's scale
        Fs = np.concatenate([F[None], near[None], rs.normal(size=(n_rand, 3, 3)), np.zeros((1, 3, 3))])
        counts, masks, dist = ref(Fs, p, q, thr)
        out[f"{name}/F"] = Fs.reshape(-1, 9)
        out[f"{name}/prev"] = p
        out[f"{name}/curr"] = q
        out[f"{name}/thr"] = np.array([thr])
        out[f"{name}/counts"] = counts
        out[f"{name}/masks"] = masks
        out[f"{name}/dist"] = dist
    np.savez_compressed(os.path.join(HERE, "ransac_cases.npz"), **out)
    print(f"wrote {len(CASES)} cases")


if __name__ == "__main__":
    main()
