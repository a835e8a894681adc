"""Seeded synthetic camera frames standing in for EuRoC (not available here).

Generators:
  * ``warped_pair``  — one 752x480 frame pair: background 128, 200 rectangles
    (sides U[8,80], intensity U[0,255]), 50 checkerboard patches of 8x8 cells
    (cell side U{2..6}, two intensities U[0,255]), additive N(0, 4^2) noise
    blurred with a sigma=1 Gaussian, clamp to u8.  Frame 2 is frame 1's
    noiseless content warped by a homography (rotation U[-5,5] deg, translation
    U[-10,10] px, scale U[0.97,1.03] about the centre) with fresh noise.
  * ``plane_sequence`` — consecutive 752x480 frames of a camera flying over
    a textured plane (a 4096x4096 texture of the same recipe, element counts
    scaled by area), translation 2-5 cm and rotation 0.5-2 deg per frame,
    bilinear homography rendering, N(0, 3^2) noise.
  * ``scene_frame`` — one frame of any size from the same recipe with counts
    scaled by area (the uneven-size batch).

The legacy ``numpy.random.RandomState`` stream is used: it is frozen across
numpy versions, so a seed names the same frame everywhere.
"""
from __future__ import annotations

import hashlib

import numpy as np

BASE_W, BASE_H = 752, 480


def _gauss_kernel(sigma: float) -> np.ndarray:
    r = int(np.ceil(3 * sigma))
    x = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-0.5 * (x / sigma) ** 2)
    return k / k.sum()


def _blur(img: np.ndarray, sigma: float) -> np.ndarray:
    k = _gauss_kernel(sigma)
    r = len(k) // 2
    p = np.pad(img, ((0, 0), (r, r)), mode="reflect")
    out = np.zeros_like(img)
    for i, kv in enumerate(k):
        out += kv * p[:, i:i + img.shape[1]]
    p = np.pad(out, ((r, r), (0, 0)), mode="reflect")
    out2 = np.zeros_like(img)
    for i, kv in enumerate(k):
        out2 += kv * p[i:i + img.shape[0], :]
    return out2


def _content(rs: np.random.RandomState, w: int, h: int, n_rect: int, n_check: int) -> np.ndarray:
    img = np.full((h, w), 128.0, dtype=np.float64)
    for _ in range(n_rect):
        rw, rh = rs.randint(8, 81), rs.randint(8, 81)
        x0 = rs.randint(-rw // 2, w - rw // 2)
        y0 = rs.randint(-rh // 2, h - rh // 2)
        val = rs.randint(0, 256)
        img[max(y0, 0):max(min(y0 + rh, h), 0), max(x0, 0):max(min(x0 + rw, w), 0)] = val
    for _ in range(n_check):
        cell = rs.randint(2, 7)
        side = 8 * cell
        x0 = rs.randint(-side // 2, w - side // 2)
        y0 = rs.randint(-side // 2, h - side // 2)
        v0, v1 = rs.randint(0, 256), rs.randint(0, 256)
        yy, xx = np.mgrid[0:side, 0:side]
        pat = np.where(((yy // cell) + (xx // cell)) % 2 == 0, v0, v1).astype(np.float64)
        ys, xs = max(y0, 0), max(x0, 0)
        ye, xe = min(y0 + side, h), min(x0 + side, w)
        if ye > ys and xe > xs:
            img[ys:ye, xs:xe] = pat[ys - y0:ye - y0, xs - x0:xe - x0]
    return img


def _noise(rs: np.random.RandomState, w: int, h: int, sigma: float, blur_sigma: float | None) -> np.ndarray:
    n = rs.normal(0.0, sigma, size=(h, w))
    return _blur(n, blur_sigma) if blur_sigma else n


def _to_u8(img: np.ndarray) -> np.ndarray:
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


def _bilinear(src: np.ndarray, sx: np.ndarray, sy: np.ndarray, fill: float) -> np.ndarray:
    h, w = src.shape
    x0 = np.floor(sx).astype(np.int64)
    y0 = np.floor(sy).astype(np.int64)
    ax = sx - x0
    ay = sy - y0
    valid = (x0 >= 0) & (y0 >= 0) & (x0 + 1 < w) & (y0 + 1 < h)
    x0c = np.clip(x0, 0, w - 2)
    y0c = np.clip(y0, 0, h - 2)
    v = ((1 - ax) * (1 - ay) * src[y0c, x0c] + ax * (1 - ay) * src[y0c, x0c + 1]
         + (1 - ax) * ay * src[y0c + 1, x0c] + ax * ay * src[y0c + 1, x0c + 1])
    return np.where(valid, v, fill)


def warp_homography(src: np.ndarray, Hm: np.ndarray, fill: float = 128.0) -> np.ndarray:
    """out(x, y) = src(H^-1 (x, y, 1)) with bilinear sampling."""
    h, w = src.shape
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    Hi = np.linalg.inv(Hm)
    d = Hi[2, 0] * xx + Hi[2, 1] * yy + Hi[2, 2]
    sx = (Hi[0, 0] * xx + Hi[0, 1] * yy + Hi[0, 2]) / d
    sy = (Hi[1, 0] * xx + Hi[1, 1] * yy + Hi[1, 2]) / d
    return _bilinear(src, sx, sy, fill)


def random_similarity(rs: np.random.RandomState, w: int, h: int) -> np.ndarray:
    ang = np.deg2rad(rs.uniform(-5.0, 5.0))
    tx, ty = rs.uniform(-10.0, 10.0), rs.uniform(-10.0, 10.0)
    s = rs.uniform(0.97, 1.03)
    cx, cy = (w - 1) / 2.0, (h - 1) / 2.0
    c, sn = np.cos(ang) * s, np.sin(ang) * s
    A = np.array([[c, -sn, 0.0], [sn, c, 0.0], [0.0, 0.0, 1.0]])
    T0 = np.array([[1.0, 0.0, -cx], [0.0, 1.0, -cy], [0.0, 0.0, 1.0]])
    T1 = np.array([[1.0, 0.0, cx + tx], [0.0, 1.0, cy + ty], [0.0, 0.0, 1.0]])
    return T1 @ A @ T0


def _counts(w: int, h: int, n_rect: int, n_check: int, scale_by_area: bool) -> tuple[int, int]:
    if not scale_by_area:
        return n_rect, n_check
    f = (w * h) / float(BASE_W * BASE_H)
    return max(1, int(round(n_rect * f))), max(1, int(round(n_check * f)))


def scene_frame(seed: int, w: int = BASE_W, h: int = BASE_H, n_rect: int = 200, n_check: int = 50,
                 scale_by_area: bool = True) -> np.ndarray:
    rs = np.random.RandomState(seed)
    nr, nc = _counts(w, h, n_rect, n_check, scale_by_area)
    content = _content(rs, w, h, nr, nc)
    return _to_u8(content + _noise(rs, w, h, 4.0, 1.0))


def warped_pair(seed: int, w: int = BASE_W, h: int = BASE_H, n_rect: int = 200, n_check: int = 50,
                 scale_by_area: bool = True) -> tuple[np.ndarray, np.ndarray]:
    rs = np.random.RandomState(seed)
    nr, nc = _counts(w, h, n_rect, n_check, scale_by_area)
    content = _content(rs, w, h, nr, nc)
    f1 = _to_u8(content + _noise(rs, w, h, 4.0, 1.0))
    Hm = random_similarity(rs, w, h)
    f2 = _to_u8(warp_homography(content, Hm) + _noise(rs, w, h, 4.0, 1.0))
    return f1, f2


class PlaneTrajectory:
    """Camera over a textured plane; frames rendered by bilinear homography."""

    def __init__(self, seed: int, w: int = BASE_W, h: int = BASE_H, tex_size: int = 4096,
                 texel_m: float = 0.004, depth_m: float = 2.0, focal_px: float = 460.0,
                 texture: np.ndarray | None = None):
        self.rs = np.random.RandomState(seed)
        self.w, self.h = w, h
        if texture is None:
            texture = plane_texture(self.rs, tex_size)
        self.tex = texture
        tex_size = texture.shape[0]
        self.texel_m = texel_m
        self.tex_size = tex_size
        self.K = np.array([[focal_px, 0.0, (w - 1) / 2.0], [0.0, focal_px, (h - 1) / 2.0], [0.0, 0.0, 1.0]])
        # camera centre above the plane's middle, looking down the -z axis
        self.c = np.array([0.0, 0.0, depth_m])
        self.R = np.diag([1.0, -1.0, -1.0])  # world -> camera
        self.dir = self.rs.uniform(0, 2 * np.pi)

    def _step(self):
        rs = self.rs
        self.dir += rs.uniform(-0.3, 0.3)
        dist = rs.uniform(0.02, 0.05)
        dz = rs.uniform(-0.2, 0.2) * dist
        self.c = self.c + np.array([dist * np.cos(self.dir), dist * np.sin(self.dir), dz])
        ang = np.deg2rad(rs.uniform(0.5, 2.0))
        axis = np.array([rs.uniform(-0.3, 0.3), rs.uniform(-0.3, 0.3), 1.0])
        axis /= np.linalg.norm(axis)
        Kx = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
        dR = np.eye(3) + np.sin(ang) * Kx + (1 - np.cos(ang)) * (Kx @ Kx)
        self.R = dR @ self.R

    def render(self) -> np.ndarray:
        w, h = self.w, self.h
        yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
        rays = np.linalg.inv(self.K) @ np.stack([xx.ravel(), yy.ravel(), np.ones(w * h)])
        d = self.R.T @ rays  # world directions
        lam = -self.c[2] / d[2]
        X = self.c[0] + lam * d[0]
        Y = self.c[1] + lam * d[1]
        sx = X / self.texel_m + self.tex_size / 2.0
        sy = Y / self.texel_m + self.tex_size / 2.0
        v = _bilinear(self.tex, sx.reshape(h, w), sy.reshape(h, w), 128.0)
        v = v + self.rs.normal(0.0, 3.0, size=(h, w))
        return _to_u8(v)

    def frames(self, n: int) -> list[np.ndarray]:
        out = []
        for _ in range(n):
            out.append(self.render())
            self._step()
        return out


def plane_texture(rs: np.random.RandomState, tex_size: int = 4096) -> np.ndarray:
    """The textured plane: the frame recipe at tex_size^2, counts scaled by area."""
    nr, nc = _counts(tex_size, tex_size, 200, 50, True)
    tex = _content(rs, tex_size, tex_size, nr, nc)
    tex += _noise(rs, tex_size, tex_size, 4.0, 1.0)
    return tex


def plane_sequence(seed: int, n: int = 64, w: int = BASE_W, h: int = BASE_H,
                   texture: np.ndarray | None = None) -> list[np.ndarray]:
    return PlaneTrajectory(seed, w, h, texture=texture).frames(n)


def frame_digest(img: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(img).tobytes()).hexdigest()


# Camera of the two-view scenes: a 752x480 pinhole with radial-tangential
# distortion of the size typical for wide-angle grey-scale SLAM cameras
# (fu, fv, cu, cv, k1, k2, p1, p2).
SCENE_CAMERA = np.array([460.0, 458.0, 376.0, 240.0, -0.28, 0.07, 2e-4, 2e-5])


def two_view_scene(seed: int, n: int, w: int = BASE_W, h: int = BASE_H, noise_px: float = 0.3,
                   outlier_frac: float = 0.0, depth=(4.0, 30.0), rot_sigma: float = 0.02,
                   baseline: float = 1.0, cam: np.ndarray | None = None):
    """Seeded RANSAC-inlier correspondences of a rigid two-view scene.

    Random points in front of the first camera are seen from a second pose
    (p_curr = R p_prev + t, a small random rotation, |t| = baseline), projected
    with the distortion model, perturbed by Gaussian pixel noise and truncated
    to integer pixels (the features' u32 coordinates); outlier_frac of the
    current pixels are replaced by uniform ones.  Rows are (lod, prev_x,
    prev_y, curr_x, curr_y) with a random level, unique current pixel per
    level, sorted by (level, curr_x, curr_y): the order in which the
    reference's triangulation pass visits its inliers.  Returns
    (rows u32 (n, 5), cam, R, t).
    """
    rng = np.random.default_rng(seed)
    cam = SCENE_CAMERA if cam is None else np.asarray(cam, np.float64)
    ang = rng.normal(0.0, rot_sigma, 3)
    th = float(np.linalg.norm(ang))
    if th > 0.0:
        k = ang / th
        kx = np.array([[0.0, -k[2], k[1]], [k[2], 0.0, -k[0]], [-k[1], k[0], 0.0]])
        R = np.eye(3) + np.sin(th) * kx + (1.0 - np.cos(th)) * kx @ kx
    else:
        R = np.eye(3)
    t = rng.normal(0.0, 1.0, 3)
    t[2] *= 0.3
    t *= baseline / np.linalg.norm(t) if baseline > 0 else 0.0

    def proj(P):
        x, y = P[:, 0] / P[:, 2], P[:, 1] / P[:, 2]
        r2 = x * x + y * y
        k1, k2, p1, p2 = cam[4:8]
        rad = 1.0 + k1 * r2 + k2 * r2 * r2
        xd = x * rad + 2.0 * p1 * x * y + p2 * (r2 + 2.0 * x * x)
        yd = y * rad + p1 * (r2 + 2.0 * y * y) + 2.0 * p2 * x * y
        return np.stack([cam[0] * xd + cam[2], cam[1] * yd + cam[3]], 1)

    m = max(8 * n, 64)
    P = np.stack([rng.uniform(-8.0, 8.0, m), rng.uniform(-5.0, 5.0, m), rng.uniform(depth[0], depth[1], m)], 1)
    Q = P @ R.T + t
    a, b = proj(P), proj(Q)
    inside = (Q[:, 2] > 0.5) & np.all((a >= 0) & (a < [w, h]) & (b >= 0) & (b < [w, h]), 1)
    a, b = a[inside], b[inside]
    a = np.floor(a + rng.normal(0.0, noise_px, a.shape)).clip(0, [w - 1, h - 1])
    b = np.floor(b + rng.normal(0.0, noise_px, b.shape)).clip(0, [w - 1, h - 1])
    n_out = int(round(outlier_frac * len(b)))
    if n_out:
        idx = rng.choice(len(b), n_out, replace=False)
        b[idx] = rng.integers(0, [w, h], (n_out, 2))
    rows = np.stack([rng.integers(0, 6, len(a)), a[:, 0], a[:, 1], b[:, 0], b[:, 1]], 1).astype(np.uint32)
    _, first = np.unique(rows[:, [0, 3, 4]], axis=0, return_index=True)
    rows = rows[np.sort(first)][:n]
    rows = rows[np.lexsort((rows[:, 4], rows[:, 3], rows[:, 0]))]
    return np.ascontiguousarray(rows), cam.copy(), R, t
