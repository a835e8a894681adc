"""numpy restatement of the reference's CPU triangulation pass — TEST
INFRASTRUCTURE ONLY (tests/ and the CPU-baseline leg of bench.py).

Follows TriangulateCPU::execute (wslam/src/pose_estimate_cpu/triangulate_cpu.cpp:342-513)
step by step:

  CollectInliers       triangulate_cpu.cpp:218-247  LOD-0 pixels -> calibrated rays
  PixelToNormalised    wslam/src/map/map_helpers_lods.hpp:110-120 (+ UndistortNormalised :41-76)
  FitEssentialMatrix   triangulate_cpu.cpp:77-140   normalised 8-point on all rays
  NormalisingTransform triangulate_cpu.cpp:48-73
  DecomposeEssential   triangulate_cpu.cpp:149-172  four (R, t) candidates
  TriangulatePoint     triangulate_cpu.cpp:180-207  linear DLT, right null vector of a 4x4
  ScoreCandidate       triangulate_cpu.cpp:257-278  points in front of both cameras
  landmark filter      triangulate_cpu.cpp:444-488  depth range + mean reprojection error
  ProjectToPixel       triangulate_cpu.cpp:34-45 with DistortNormalised (map_helpers_lods.hpp:16-29)
  ComputeRotationAngle map_helpers_lods.hpp:33-36

Rows are taken in the caller's order; the reference visits them per level in
the order of its flat_map keys (the current feature), so callers that compare
against the reference pass rows sorted by (level, current x, current y).

The undistortion repeats the reference's double operations in the same order,
so its rays equal the reference's bit for bit.  The SVD steps use LAPACK
(numpy) where the reference uses Eigen's JacobiSVD: the null vectors agree to
rounding, up to sign, and the candidate order of DecomposeEssential may differ
by the sign conventions of the two SVDs (the set of four poses is the same),
so the pose chosen agrees whenever the best cheirality count is unique.
"""
from __future__ import annotations

import math

import numpy as np

DEFAULT_OPTS = {
    # TriangulateCPU::Opts (wslam/src/pose_estimate_cpu/triangulate_cpu.hpp:30-54)
    "max_reprojection_px": 4.0,
    "min_depth": 1e-3,
    "max_depth": 1e3,
    "min_inliers": 8,
    "undistort_iterations": 20,
    "undistort_tolerance": 1e-9,
}

SQRT2 = 1.4142135623730951  # std::numbers::sqrt2


def undistort_normalised(dist: np.ndarray, d, max_iters: int, tol: float) -> np.ndarray:
    """UndistortNormalised (map_helpers_lods.hpp:45-76) for every row of dist (n, 2)."""
    dist = np.asarray(dist, np.float64)
    k1, k2, p1, p2 = (float(v) for v in d)
    xy = dist.copy()
    active = np.ones(len(xy), bool)
    for _ in range(int(max_iters)):
        if not active.any():
            break
        x, y = xy[active, 0], xy[active, 1]
        r2 = x * x + y * y
        radial = 1.0 + k1 * r2 + k2 * r2 * r2
        dx_tan = 2.0 * p1 * x * y + p2 * (r2 + 2.0 * x * x)
        dy_tan = p1 * (r2 + 2.0 * y * y) + 2.0 * p2 * x * y
        nx = (dist[active, 0] - dx_tan) / radial
        ny = (dist[active, 1] - dy_tan) / radial
        ex, ey = nx - x, ny - y
        step = np.sqrt(ex * ex + ey * ey)
        xy[active, 0] = nx
        xy[active, 1] = ny
        idx = np.flatnonzero(active)
        active[idx[step < tol]] = False
    return xy


def pixel_to_normalised(px: np.ndarray, cam, max_iters: int, tol: float) -> np.ndarray:
    """PixelToNormalised (map_helpers_lods.hpp:110-120); cam = fu, fv, cu, cv, k1, k2, p1, p2."""
    px = np.asarray(px, np.float64)
    fu, fv, cu, cv = (float(v) for v in cam[:4])
    dist = np.stack([(px[:, 0] - cu) / fu, (px[:, 1] - cv) / fv], 1)
    return undistort_normalised(dist, cam[4:8], max_iters, tol)


def distort_normalised(xy: np.ndarray, d) -> np.ndarray:
    """DistortNormalised (map_helpers_lods.hpp:16-29)."""
    k1, k2, p1, p2 = (float(v) for v in d)
    x, y = xy[:, 0], xy[:, 1]
    r2 = x * x + y * y
    radial = 1.0 + k1 * r2 + k2 * r2 * r2
    dx = 2.0 * p1 * x * y + p2 * (r2 + 2.0 * x * x)
    dy = p1 * (r2 + 2.0 * y * y) + 2.0 * p2 * x * y
    return np.stack([x * radial + dx, y * radial + dy], 1)


def project_to_pixel(p: np.ndarray, cam) -> np.ndarray:
    """ProjectToPixel (triangulate_cpu.cpp:34-45): NaN where z <= 0."""
    z = p[:, 2]
    with np.errstate(divide="ignore", invalid="ignore"):
        xy = np.stack([p[:, 0] / z, p[:, 1] / z], 1)
    xd = distort_normalised(xy, cam[4:8])
    out = np.stack([cam[0] * xd[:, 0] + cam[2], cam[1] * xd[:, 1] + cam[3]], 1)
    out[z <= 0.0] = np.nan
    return out


def normalising_transform(points: np.ndarray) -> np.ndarray:
    """NormalisingTransform (triangulate_cpu.cpp:48-73), sums taken in row order."""
    n = float(len(points))
    c = np.array([np.cumsum(points[:, 0])[-1], np.cumsum(points[:, 1])[-1]]) / n
    d = points - c
    mean_dist = np.cumsum(np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]))[-1] / n
    scale = SQRT2 / mean_dist if mean_dist > 1e-12 else 1.0
    t = np.eye(3)
    t[0, 0] = scale
    t[1, 1] = scale
    t[0, 2] = -scale * c[0]
    t[1, 2] = -scale * c[1]
    return t


def fit_essential(prev: np.ndarray, curr: np.ndarray):
    """FitEssentialMatrix (triangulate_cpu.cpp:77-140); None where it fails."""
    tp, tc = normalising_transform(prev), normalising_transform(curr)
    p = prev @ tp[:2, :2].T + tp[:2, 2]
    q = curr @ tc[:2, :2].T + tc[:2, 2]
    xp, yp, xc, yc = p[:, 0], p[:, 1], q[:, 0], q[:, 1]
    a = np.stack([xc * xp, xc * yp, xc, yc * xp, yc * yp, yc, xp, yp, np.ones_like(xp)], 1)
    v = np.linalg.svd(a, full_matrices=len(a) < 9)[2][8]
    e_norm = v.reshape(3, 3)
    u, s, vt = np.linalg.svd(e_norm)
    avg = 0.5 * (s[0] + s[1])
    e_clean = u @ np.diag([avg, avg, 0.0]) @ vt
    e_final = tc.T @ e_clean @ tp
    if not np.all(np.isfinite(e_final)):
        return None
    return e_final


def decompose_essential(e: np.ndarray):
    """DecomposeEssential (triangulate_cpu.cpp:149-172): [(R1, t), (R1, -t), (R2, t), (R2, -t)]."""
    u, _, vt = np.linalg.svd(e)
    v = vt.T.copy()
    u = u.copy()
    if np.linalg.det(u) < 0.0:
        u[:, 2] *= -1.0
    if np.linalg.det(v) < 0.0:
        v[:, 2] *= -1.0
    w = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    r1 = u @ w @ v.T
    r2 = u @ w.T @ v.T
    t = u[:, 2].copy()
    return [(r1, t), (r1, -t), (r2, t), (r2, -t)]


def triangulate_points(r: np.ndarray, t: np.ndarray, xy_prev: np.ndarray, xy_curr: np.ndarray) -> np.ndarray:
    """TriangulatePoint (triangulate_cpu.cpp:180-207) for every row: (n, 3), NaN where it fails."""
    n = len(xy_prev)
    p2 = np.concatenate([r, t[:, None]], 1)
    a = np.zeros((n, 4, 4))
    a[:, 0, 0] = -1.0
    a[:, 0, 2] = xy_prev[:, 0]
    a[:, 1, 1] = -1.0
    a[:, 1, 2] = xy_prev[:, 1]
    a[:, 2, :] = xy_curr[:, 0, None] * p2[2] - p2[0]
    a[:, 3, :] = xy_curr[:, 1, None] * p2[2] - p2[1]
    x = np.linalg.svd(a)[2][:, 3, :]
    w = x[:, 3]
    with np.errstate(divide="ignore", invalid="ignore"):
        p = x[:, :3] / w[:, None]
    bad = (np.abs(w) < 1e-12) | ~np.all(np.isfinite(p), 1)
    p[bad] = np.nan
    return p


def rotation_angle(r: np.ndarray) -> float:
    """ComputeRotationAngle (map_helpers_lods.hpp:33-36)."""
    trace = min(max((r[0, 0] + r[1, 1]) + r[2, 2], -1.0), 3.0)
    return math.acos(min(max(0.5 * (trace - 1.0), -1.0), 1.0))


def triangulate(px: np.ndarray, cam, opts: dict | None = None) -> dict:
    """TriangulateCPU::execute for one frame pair.

    px: (n, 4) LOD-0 pixels (prev_x, prev_y, curr_x, curr_y) of the RANSAC
    inliers.  Returns the TriangulationResult fields plus per-row ``keep`` and
    ``landmarks`` (x, y, z in the current camera, reprojection error) and the
    per-candidate cheirality counts ``in_front``.
    """
    o = dict(DEFAULT_OPTS, **(opts or {}))
    px = np.asarray(px, np.float64).reshape(-1, 4)
    n = len(px)
    cam = np.asarray(cam, np.float64)
    res = {
        "rotation": np.eye(3), "translation": np.zeros(3), "input_matches": n, "landmark_count": 0,
        "cheirality_passes": 0, "mean_reprojection_error_px": 0.0, "pose_recovered": False,
        "rotation_angle_rad": 0.0, "keep": np.zeros(n, bool), "landmarks": np.zeros((n, 4)),
        "in_front": np.zeros(4, np.int64), "best": -1,
    }
    if n < o["min_inliers"]:
        return res
    it, tol = int(o["undistort_iterations"]), float(o["undistort_tolerance"])
    xy_prev = pixel_to_normalised(px[:, 0:2], cam, it, tol)
    xy_curr = pixel_to_normalised(px[:, 2:4], cam, it, tol)
    e = fit_essential(xy_prev, xy_curr)
    if e is None:
        return res
    cands = decompose_essential(e)
    best, best_count, best_pts = 0, 0, None
    for k, (r, t) in enumerate(cands):
        p = triangulate_points(r, t, xy_prev, xy_curr)
        pc = p @ r.T + t
        count = int(np.count_nonzero((p[:, 2] > 0.0) & (pc[:, 2] > 0.0)))
        res["in_front"][k] = count
        if count > best_count:
            best, best_count, best_pts = k, count, p
    res["cheirality_passes"] = best_count
    if best_count == 0:
        return res
    r, t = cands[best]
    res["best"] = best
    res["rotation"], res["translation"] = r, t
    res["rotation_angle_rad"] = rotation_angle(r)
    p_prev = best_pts
    p_curr = p_prev @ r.T + t
    ok = np.all(np.isfinite(p_prev), 1)
    with np.errstate(invalid="ignore"):
        ok &= ~((p_prev[:, 2] < o["min_depth"]) | (p_prev[:, 2] > o["max_depth"])
                | (p_curr[:, 2] < o["min_depth"]) | (p_curr[:, 2] > o["max_depth"]))
    rp = project_to_pixel(np.where(ok[:, None], p_prev, 1.0), cam)
    rc = project_to_pixel(np.where(ok[:, None], p_curr, 1.0), cam)
    ok &= np.all(np.isfinite(rp), 1) & np.all(np.isfinite(rc), 1)
    dp, dc = rp - px[:, 0:2], rc - px[:, 2:4]
    err = 0.5 * (np.sqrt(dp[:, 0] * dp[:, 0] + dp[:, 1] * dp[:, 1]) + np.sqrt(dc[:, 0] * dc[:, 0] + dc[:, 1] * dc[:, 1]))
    with np.errstate(invalid="ignore"):
        ok &= ~(err > o["max_reprojection_px"])
    res["keep"] = ok
    res["landmarks"][ok, :3] = p_curr[ok]
    res["landmarks"][ok, 3] = err[ok]
    res["landmark_count"] = int(ok.sum())
    res["pose_recovered"] = bool(ok.any())
    if ok.any():
        res["mean_reprojection_error_px"] = float(np.cumsum(err[ok])[-1] / ok.sum())
    return res
