"""CPU oracle of the feature front-end — TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` load this package; the product library never calls it.  See
oracle.h for what each function restates and the parity status (matcher
pinned against the reference's own compiled source; WGSL stages unpinned).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

FEATURE_DTYPE = np.dtype([
    ("x", "<f4"), ("y", "<f4"), ("strength", "<u4"), ("orientation", "<f4"), ("descriptor", "<u4", (8,)),
])

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"{LIB} missing: run `make -C oracle`")
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.orc_level_dims.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp]
        L.orc_pyramid_level.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_uint32, C.c_int, vp]
        L.orc_detect.argtypes = [vp, C.c_uint32, C.c_uint32, vp]
        L.orc_cull.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_int, C.c_int, vp]
        L.orc_describe.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_int, C.c_int, vp, vp, vp]
        L.orc_blur_level.argtypes = [vp, C.c_uint32, C.c_uint32, vp]
        L.orc_gauss_tap9.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]
        L.orc_gauss_tap9.restype = C.c_float
        L.orc_frame.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, C.c_int, vp, vp]
        L.orc_frame.restype = C.c_int
        L.orc_frame_ex.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, C.c_int,
                                   vp, vp]
        L.orc_detect_cfg.argtypes = [vp, C.c_uint32, C.c_uint32, vp]
        L.orc_detect_cfg.restype = None
        L.orc_frame_ex.restype = C.c_int
        L.orc_frame_fc.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp,
                                   C.c_int, vp, vp]
        L.orc_frame_fc.restype = C.c_int
        L.orc_match.argtypes = [vp, vp, vp, vp, C.c_int, C.c_int, C.c_int, vp, C.c_int]
        L.orc_match.restype = C.c_int
        L.orc_match_bruteforce.argtypes = [vp, C.c_int, vp, C.c_int, C.c_float, vp]
        L.orc_match_bruteforce.restype = C.c_int
        L.orc_sampson_counts.argtypes = [vp, C.c_int, vp, vp, C.c_int, C.c_double, vp, vp]
        L.orc_sampson_counts.restype = None
        L.orc_atan2f.argtypes = [C.c_float, C.c_float]
        L.orc_atan2f.restype = C.c_float
        L.orc_sincosf.argtypes = [C.c_float, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def level_dims(W0: int, H0: int, levels: int = 6):
    w = np.zeros(levels, np.uint32)
    h = np.zeros(levels, np.uint32)
    lib().orc_level_dims(W0, H0, levels, _p(w), _p(h))
    return [(int(a), int(b)) for a, b in zip(w, h)]


def pyramid_level(img: np.ndarray, level: int, levels: int = 6) -> np.ndarray:
    img = np.ascontiguousarray(img, np.uint8)
    H0, W0 = img.shape
    w, h = level_dims(W0, H0, levels)[level]
    out = np.zeros((h, w), np.float32)
    lib().orc_pyramid_level(_p(img), W0, H0, W0, w, h, int(level == 0), _p(out))
    return out


def detect(lvl: np.ndarray) -> np.ndarray:
    lvl = np.ascontiguousarray(lvl, np.float32)
    h, w = lvl.shape
    out = np.zeros((h, w), np.uint32)
    lib().orc_detect(_p(lvl), w, h, _p(out))
    return out


def cull(resp: np.ndarray, W0: int, H0: int) -> np.ndarray:
    resp = np.ascontiguousarray(resp, np.uint32)
    h, w = resp.shape
    out = np.zeros((h, w), np.uint32)
    lib().orc_cull(_p(resp), w, h, W0, H0, _p(out))
    return out


def detect_cfg(lvl: np.ndarray) -> np.ndarray:
    """cfg detection profile on one level: arc length of NMS survivors, else 0."""
    lvl = np.ascontiguousarray(lvl, np.float32)
    h, w = lvl.shape
    out = np.zeros((h, w), np.uint32)
    lib().orc_detect_cfg(_p(lvl), w, h, _p(out))
    return out


def gauss_tap9(lvl: np.ndarray, px: int, py: int) -> float:
    lvl = np.ascontiguousarray(lvl, np.float32)
    h, w = lvl.shape
    return float(lib().orc_gauss_tap9(_p(lvl), w, h, px & 0xffffffff, py & 0xffffffff))


def blur_level(lvl: np.ndarray) -> np.ndarray:
    lvl = np.ascontiguousarray(lvl, np.float32)
    h, w = lvl.shape
    out = np.zeros((h, w), np.float32)
    lib().orc_blur_level(_p(lvl), w, h, _p(out))
    return out


def describe(lvl: np.ndarray, x: int, y: int, pattern: np.ndarray):
    lvl = np.ascontiguousarray(lvl, np.float32)
    pat = np.ascontiguousarray(pattern, np.int32).reshape(-1)
    h, w = lvl.shape
    th = np.zeros(1, np.float32)
    d = np.zeros(8, np.uint32)
    lib().orc_describe(_p(lvl), w, h, x, y, _p(pat), _p(th), _p(d))
    return float(th[0]), d


def frame(img: np.ndarray, pattern: np.ndarray, levels: int = 6, cap: int | None = None, cell_cap: int = 0,
          detector: int = 0, frame_cap: int = 0):
    """Features of one frame: (features[FEATURE_DTYPE], kept[levels], raw[levels]).
    cell_cap > 0 keeps at most cell_cap keypoints per 32x32 cell, listed cell by cell;
    detector = 1 selects the cfg detection profile (FAST 9-of-16 at 20/255, 3x3 NMS);
    frame_cap > 0 keeps the first frame_cap features of the frame in (level, order
    within the level) order, on top of the per-level cap."""
    img = np.ascontiguousarray(img, np.uint8)
    H0, W0 = img.shape
    if cap is None:
        cap = W0 * H0 // 250
    pat = np.ascontiguousarray(pattern, np.int32).reshape(-1)
    dims = level_dims(W0, H0, levels)
    max_feats = max(1, sum(min(cap, w * h) for w, h in dims))
    feats = np.zeros(max_feats, FEATURE_DTYPE)
    kept = np.zeros(levels, np.int32)
    raw = np.zeros(levels, np.int32)
    n = lib().orc_frame_fc(_p(img), W0, H0, W0, levels, cap, cell_cap, detector, frame_cap, _p(pat), _p(feats),
                           max_feats, _p(kept), _p(raw))
    if n < 0:
        raise RuntimeError("orc_frame: feature buffer too small")
    return feats[:n].copy(), kept, raw


def match(feats_a, kept_a, feats_b, kept_b, W0: int, H0: int) -> np.ndarray:
    """Mutual matches (lod_a, idx_a, lod_b, idx_b) of prev=a against curr=b."""
    levels = len(kept_a)
    a = np.ascontiguousarray(feats_a, FEATURE_DTYPE)
    b = np.ascontiguousarray(feats_b, FEATURE_DTYPE)
    a_off = np.concatenate([[0], np.cumsum(kept_a)]).astype(np.int32)
    b_off = np.concatenate([[0], np.cumsum(kept_b)]).astype(np.int32)
    max_out = max(1, int(min(a_off[-1], b_off[-1])))
    out = np.zeros((max_out, 4), np.int32)
    n = lib().orc_match(_p(a), _p(a_off), _p(b), _p(b_off), levels, W0, H0, _p(out), max_out)
    if n < 0:
        raise RuntimeError("orc_match: output buffer too small")
    return out[:n].copy()


def match_bruteforce(feats_a, kept_a, feats_b, kept_b, ratio: float = 0.8) -> np.ndarray:
    """Brute-force top-2 matches (lod_a, idx_a, lod_b, idx_b) of every feature
    of a against every feature of b, in (lod_a, idx_a) order."""
    a = np.ascontiguousarray(feats_a, FEATURE_DTYPE)
    b = np.ascontiguousarray(feats_b, FEATURE_DTYPE)
    a2b = np.full(max(len(a), 1), -1, np.int32)
    lib().orc_match_bruteforce(_p(a), len(a), _p(b), len(b), ratio, _p(a2b))
    a2b = a2b[:len(a)]
    a_off = np.concatenate([[0], np.cumsum(kept_a)])
    b_off = np.concatenate([[0], np.cumsum(kept_b)])
    qa = np.nonzero(a2b >= 0)[0]
    la = np.searchsorted(a_off, qa, side="right") - 1
    tb = a2b[qa]
    lb = np.searchsorted(b_off, tb, side="right") - 1
    return np.stack([la, qa - a_off[la], lb, tb - b_off[lb]], 1).astype(np.int32).reshape(-1, 4)


def sampson_counts(fmats: np.ndarray, prev_xy: np.ndarray, curr_xy: np.ndarray, thr: float = 3.84):
    """(counts[H], masks[H, ceil(N/32)]) of the Sampson inlier test."""
    F = np.ascontiguousarray(fmats, np.float64).reshape(-1, 9)
    p = np.ascontiguousarray(prev_xy, np.float64).reshape(-1, 2)
    q = np.ascontiguousarray(curr_xy, np.float64).reshape(-1, 2)
    n = len(p)
    counts = np.zeros(len(F), np.int32)
    masks = np.zeros((len(F), max(1, (n + 31) // 32)), np.uint32)
    lib().orc_sampson_counts(_p(F), len(F), _p(p), _p(q), n, thr, _p(counts), _p(masks))
    return counts, masks[:, :(n + 31) // 32]


def atan2f(y: float, x: float) -> float:
    return float(lib().orc_atan2f(y, x))


def sincosf(a: float) -> tuple[float, float]:
    s = np.zeros(1, np.float32)
    c = np.zeros(1, np.float32)
    lib().orc_sincosf(a, _p(s), _p(c))
    return float(s[0]), float(c[0])


# --------------------------------------------------- compiled reference matcher

def ref_matcher(W0: int = 752, H0: int = 480):
    """The reference's own match_features_cpu.cpp (compiled by oracle/Makefile), or None."""
    path = os.path.join(REF_DIR, f"libref_matcher_{W0}x{H0}.so")
    if not os.path.exists(path):
        return None
    L = C.CDLL(path)
    vp = C.c_void_p
    L.ref_find_matches.argtypes = [vp, vp, vp, vp, vp, C.c_int]
    L.ref_find_matches.restype = C.c_int

    def run(feats_a, kept_a, feats_b, kept_b):
        a = np.ascontiguousarray(feats_a, FEATURE_DTYPE)
        b = np.ascontiguousarray(feats_b, FEATURE_DTYPE)
        a_off = np.concatenate([[0], np.cumsum(kept_a)]).astype(np.int32)
        b_off = np.concatenate([[0], np.cumsum(kept_b)]).astype(np.int32)
        max_out = max(1, int(min(a_off[-1], b_off[-1])))
        out = np.zeros((max_out, 4), np.int32)
        n = L.ref_find_matches(_p(a), _p(a_off), _p(b), _p(b_off), _p(out), max_out)
        if n < 0:
            raise RuntimeError("ref_find_matches: output buffer too small")
        return out[:n].copy()

    return run


def ref_sampson():
    """The reference's own RANSAC inlier test (ransac_cpu.cpp SampsonDistance
    and ClassifyInliers, compiled by oracle/Makefile), or None.  The callable
    returns (counts[H], masks[H, ceil(N/32)], distances[H, N])."""
    path = os.path.join(REF_DIR, "libref_ransac.so")
    if not os.path.exists(path):
        return None
    L = C.CDLL(path)
    vp = C.c_void_p
    L.ref_sampson_classify.argtypes = [vp, C.c_int, vp, vp, C.c_int, C.c_double, vp, vp, vp]
    L.ref_sampson_classify.restype = None

    def run(fmats, prev_xy, curr_xy, thr: float = 3.84):
        F = np.ascontiguousarray(fmats, np.float64).reshape(-1, 9)
        pp = np.ascontiguousarray(prev_xy, np.float64).reshape(-1, 2)
        q = np.ascontiguousarray(curr_xy, np.float64).reshape(-1, 2)
        n = len(pp)
        counts = np.zeros(len(F), np.int32)
        masks = np.zeros((len(F), max(1, (n + 31) // 32)), np.uint32)
        dist = np.zeros((len(F), max(1, n)), np.float64)
        L.ref_sampson_classify(_p(F), len(F), _p(pp), _p(q), n, thr, _p(counts), _p(masks), _p(dist))
        return counts, masks[:, :(n + 31) // 32], dist[:, :n]

    return run


STAGED_MATCHER = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "wslam", "src", "pose_estimate_cpu",
                              "match_features_cpu.cpp")


def ref_matcher_expected() -> bool:
    """True where the reference's matcher source is at hand (its copy staged
    in baseline/_ref travels with the repository), so oracle/_ref must hold
    the compiled matcher and the live checks against it must run."""
    return os.path.exists(STAGED_MATCHER)
