"""Python handles over the C ABI: Context, Batch (work-table form) and
Frontend (the reference's per-frame pass sequence with FeatureSet rotation).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import FEATURE_DTYPE, MATCH_DTYPE, USlamError, iptr, ptr


# stages timed by uslam_batch_profile (the compaction stage is three kernels:
# k_band_count, k_band_write, k_xsort)
KERNELS = ("k_pyramid", "k_detect", "k_blur_border", "compaction", "k_describe", "k_match", "k_mutual")


def level_dims(width: int, height: int, levels: int = 6) -> list[tuple[int, int]]:
    lib = capi.load()
    w = np.zeros(levels, np.int32)
    h = np.zeros(levels, np.int32)
    st = lib.uslam_level_dims(width, height, levels, iptr(w), iptr(h))
    if st != capi.OK:
        raise USlamError(st, "level_dims")
    return [(int(a), int(b)) for a, b in zip(w, h)]


class Context:
    """Device context: BRIEF table, level count, caps (per level and, with
    cell_cap > 0, per 32x32 cell), size limits, matcher (0: the reference's
    windowed mutual matcher, 1: brute-force top-2 with Lowe ``ratio`` on the
    integer pipes, 2: the same brute-force top-2 on the tensor cores, 3: the
    windowed matcher with its distances from tensor-core tiles) and
    detector (0: the reference's FAST + cull, 1: the cfg profile, FAST
    9-of-16 at 20/255 with 3x3 NMS); frame_cap > 0 keeps the first frame_cap
    features of a frame in (level, order within the level) order;
    describe_form 1 reads the describe tests from TMA-staged shared-memory
    boxes in batches of 8+ frames (0: per-test gathers, the default)."""

    def __init__(self, pattern: np.ndarray, levels: int = 6, max_width: int = 4096, max_height: int = 4096,
                 cap_per_level: int = 0, device: int = 0, matcher: int = 0, ratio: float = 0.8,
                 cell_cap: int = 0, detector: int = 0, frame_cap: int = 0, describe_form: int = 0):
        self.lib = capi.load()
        self._pattern = np.ascontiguousarray(pattern, dtype=np.int32).reshape(-1)
        if self._pattern.size != 1024:
            raise ValueError("pattern must hold 256 x (ax, ay, bx, by)")
        p = capi.Params(device, levels, max_width, max_height, cap_per_level,
                        self._pattern.ctypes.data_as(C.POINTER(C.c_int32)), matcher, ratio, cell_cap,
                        detector, frame_cap, describe_form)
        h = C.c_void_p()
        st = self.lib.uslam_create(C.byref(p), C.byref(h))
        if st != capi.OK:
            raise USlamError(st, "uslam_create failed")
        self.h = h
        self.levels = levels

    def blur_margin(self) -> int:
        m = C.c_int()
        self.check(self.lib.uslam_blur_margin(self.h, C.byref(m)), "blur_margin")
        return m.value

    def tile_shapes(self) -> list[tuple[int, int]]:
        n = C.c_int()
        self.check(self.lib.uslam_tile_shapes(C.byref(n), None, None), "tile_shapes")
        tw = np.zeros(n.value, np.int32)
        th = np.zeros(n.value, np.int32)
        self.check(self.lib.uslam_tile_shapes(C.byref(n), iptr(tw), iptr(th)), "tile_shapes")
        return [(int(a), int(b)) for a, b in zip(tw, th)]

    def set_tile_shape(self, width: int, height: int, shape: int):
        self.check(self.lib.uslam_set_tile_shape(self.h, width, height, shape), "set_tile_shape")

    def tile_shape(self, width: int, height: int) -> int:
        s = C.c_int()
        self.check(self.lib.uslam_get_tile_shape(self.h, width, height, C.byref(s)), "get_tile_shape")
        return s.value

    def autotune(self, frame: np.ndarray, n_frames: int = 8, reps: int = 10) -> tuple[int, list[float]]:
        """Time k_detect in every tile shape on n_frames copies of `frame`;
        store the fastest for the frame's size.  Returns (shape, per-shape ms)."""
        img = np.ascontiguousarray(frame, np.uint8)
        h, w = img.shape
        ms = np.zeros(len(self.tile_shapes()), np.float32)
        s = C.c_int()
        self.check(self.lib.uslam_autotune(self.h, w, h, ptr(img), w, n_frames, reps, C.byref(s), ptr(ms)),
                   "autotune")
        return s.value, [float(v) for v in ms]

    def match(self, prev: "FeatureSet", curr: "FeatureSet") -> np.ndarray:
        """Matches of prev (reference set) against curr (uslam_match_sets)."""
        n = C.c_int()
        self.check(self.lib.uslam_match_sets(self.h, prev.h, curr.h, None, 0, C.byref(n)), "match_sets")
        out = np.zeros(n.value, MATCH_DTYPE)
        self.check(self.lib.uslam_match_sets(self.h, prev.h, curr.h, ptr(out), out.size, C.byref(n)), "match_sets")
        return out

    def ransac_score(self, fmats: np.ndarray, prev_xy: np.ndarray, curr_xy: np.ndarray, threshold: float = 3.84,
                     masks: bool = False):
        """Inlier counts of H fundamental matrices over N correspondences
        (uslam_ransac_score); with masks=True also the inlier bitmasks."""
        F = np.ascontiguousarray(fmats, np.float64).reshape(-1, 9)
        p = np.ascontiguousarray(prev_xy, np.float64).reshape(-1, 2)
        q = np.ascontiguousarray(curr_xy, np.float64).reshape(-1, 2)
        n = len(p)
        counts = np.zeros(len(F), np.int32)
        m = np.zeros((len(F), max(1, (n + 31) // 32)), np.uint32) if masks else None
        self.check(self.lib.uslam_ransac_score(self.h, ptr(F), len(F), ptr(p), ptr(q), n, threshold, iptr(counts),
                                               ptr(m) if masks else None), "ransac_score")
        return (counts, m[:, :(n + 31) // 32]) if masks else counts

    def pixel_to_normalised(self, px, cam, iterations: int = 20, tolerance: float = 1e-9) -> np.ndarray:
        """Calibrated rays of LOD-0 pixels (uslam_pixel_to_normalised)."""
        p = np.ascontiguousarray(px, np.float64).reshape(-1, 2)
        out = np.zeros_like(p)
        c = capi.Camera(*[float(v) for v in np.asarray(cam, np.float64).reshape(8)])
        self.check(self.lib.uslam_pixel_to_normalised(self.h, C.byref(c), iterations, tolerance, ptr(p), len(p),
                                                      ptr(out)), "pixel_to_normalised")
        return out

    def triangulate(self, px, cam, opts: dict | None = None):
        """Two-view triangulation of one or many frame pairs (uslam_triangulate).

        px: one (n, 4) array of LOD-0 pixels (prev_x, prev_y, curr_x, curr_y)
        or a list of them, one per pair; cam: fu, fv, cu, cv, k1, k2, p1, p2;
        opts: TriangulateCPU::Opts fields to override.  Returns, per pair, a dict
        of the TriangulationResult fields plus ``keep`` (bool per row) and
        ``landmarks`` ((n, 4): x, y, z in the current camera, reprojection
        error; zero where not kept)."""
        single = isinstance(px, np.ndarray) and px.ndim == 2
        parts = [np.asarray(px, np.float64).reshape(-1, 4)] if single else \
            [np.asarray(a, np.float64).reshape(-1, 4) for a in px]
        offsets = np.zeros(len(parts) + 1, np.int32)
        offsets[1:] = np.cumsum([len(a) for a in parts])
        rows = np.ascontiguousarray(np.concatenate(parts) if parts else np.zeros((0, 4)), np.float64)
        c = capi.Camera(*[float(v) for v in np.asarray(cam, np.float64).reshape(8)])
        o = capi.TriOpts()
        self.lib.uslam_tri_default_opts(C.byref(o))
        for k, v in (opts or {}).items():
            setattr(o, k, v)
        res = np.zeros(len(parts), capi.TRI_RESULT_DTYPE)
        lm = np.zeros((len(rows), 4))
        keep = np.zeros(len(rows), np.uint8)
        self.check(self.lib.uslam_triangulate(self.h, C.byref(c), C.byref(o), len(parts), iptr(offsets),
                                              ptr(rows), ptr(res), ptr(lm), ptr(keep)), "triangulate")
        out = []
        for k in range(len(parts)):
            a, b = offsets[k], offsets[k + 1]
            r = res[k]
            out.append({
                "rotation": r["rotation"].reshape(3, 3).copy(), "translation": r["translation"].copy(),
                "input_matches": int(r["input_matches"]), "landmark_count": int(r["landmark_count"]),
                "cheirality_passes": int(r["cheirality_passes"]), "pose_recovered": bool(r["pose_recovered"]),
                "mean_reprojection_error_px": float(r["mean_reprojection_error_px"]),
                "rotation_angle_rad": float(r["rotation_angle_rad"]),
                "keep": keep[a:b].astype(bool), "landmarks": lm[a:b].copy(),
            })
        return out[0] if single else out

    def error(self) -> str:
        return self.lib.uslam_last_error(self.h).decode()

    def check(self, st: int, what: str, ok=(capi.OK,)):
        if st not in ok:
            raise USlamError(st, f"{what}: {self.error()}")
        return st

    def close(self):
        if self.h:
            self.lib.uslam_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Batch:
    """Work table over frames of any sizes plus frame pairs to match."""

    def __init__(self, ctx: Context, sizes: list[tuple[int, int]], pairs: list[tuple[int, int]] = ()):
        self.ctx = ctx
        self.lib = ctx.lib
        self.sizes = list(sizes)
        self.pairs = list(pairs)
        w = np.array([s[0] for s in sizes], np.int32)
        h = np.array([s[1] for s in sizes], np.int32)
        pp = np.array([p[0] for p in pairs] or [0], np.int32)
        pc = np.array([p[1] for p in pairs] or [0], np.int32)
        hb = C.c_void_p()
        ctx.check(self.lib.uslam_batch_create(ctx.h, len(sizes), iptr(w), iptr(h), len(self.pairs), iptr(pp),
                                              iptr(pc), C.byref(hb)), "batch_create")
        self.h = hb
        self.caps = []

    def set_frame(self, i: int, img: np.ndarray):
        img = np.ascontiguousarray(img, dtype=np.uint8)
        self.ctx.check(self.lib.uslam_batch_set_frame(self.h, i, ptr(img), img.shape[1]), "set_frame")

    def input_device(self, i: int) -> tuple[int, int]:
        p = C.POINTER(C.c_uint8)()
        pitch = C.c_int()
        self.ctx.check(self.lib.uslam_batch_input_device(self.h, i, C.byref(p), C.byref(pitch)), "input_device")
        return C.cast(p, C.c_void_p).value, pitch.value

    def input_host(self, i: int) -> np.ndarray:
        """Pinned staging view (H0 x pitch) of frame i's input."""
        p = C.POINTER(C.c_uint8)()
        pitch = C.c_int()
        self.ctx.check(self.lib.uslam_batch_input_host(self.h, i, C.byref(p), C.byref(pitch)), "input_host")
        h0 = self.sizes[i][1]
        return np.ctypeslib.as_array(p, shape=(h0 * pitch.value,)).reshape(h0, pitch.value)

    def upload(self):
        self.ctx.check(self.lib.uslam_batch_upload(self.h), "upload")

    def run(self):
        self.ctx.check(self.lib.uslam_batch_run(self.h), "run")

    def download(self):
        self.ctx.check(self.lib.uslam_batch_download(self.h), "download")

    def sync(self, timeout_ms: int = 0):
        self.ctx.check(self.lib.uslam_batch_sync(self.h, timeout_ms), "sync")

    def process(self, frames: list[np.ndarray]):
        for i, f in enumerate(frames):
            self.set_frame(i, f)
        self.upload()
        self.run()
        self.download()
        self.sync()

    def features(self, i: int):
        L = self.ctx.levels
        kept = np.zeros(L, np.int32)
        raw = np.zeros(L, np.int32)
        self.ctx.check(self.lib.uslam_batch_features(self.h, i, None, 0, iptr(kept), iptr(raw)), "features")
        out = np.zeros(int(kept.sum()), FEATURE_DTYPE)
        self.ctx.check(self.lib.uslam_batch_features(self.h, i, ptr(out), out.size, iptr(kept), iptr(raw)),
                       "features")
        return out, kept, raw

    def matches(self, p: int) -> np.ndarray:
        n = C.c_int()
        self.ctx.check(self.lib.uslam_batch_matches(self.h, p, None, 0, C.byref(n)), "matches")
        out = np.zeros(n.value, MATCH_DTYPE)
        self.ctx.check(self.lib.uslam_batch_matches(self.h, p, ptr(out), out.size, C.byref(n)), "matches")
        return out

    def _dims(self, i: int, level: int):
        return level_dims(self.sizes[i][0], self.sizes[i][1], self.ctx.levels)[level]

    def pyramid_level(self, i: int, level: int) -> np.ndarray:
        w, h = self._dims(i, level)
        out = np.zeros((h, w), np.float32)
        self.ctx.check(self.lib.uslam_batch_pyramid_level(self.h, i, level, ptr(out)), "pyramid_level")
        return out

    def blur_level(self, i: int, level: int, extended: bool = False) -> np.ndarray:
        """Blur cache of a level: the w x h interior, or the extended cache
        ((h + M + 1) x (w + M + 1), last row/column = negative-coordinate sentinel)."""
        w, h = self._dims(i, level)
        m = self.ctx.blur_margin()
        out = np.zeros((h + m + 1, w + m + 1), np.float32)
        self.ctx.check(self.lib.uslam_batch_blur_level(self.h, i, level, ptr(out)), "blur_level")
        return out if extended else np.ascontiguousarray(out[:h, :w])

    def keypoint_map(self, i: int, level: int) -> np.ndarray:
        w, h = self._dims(i, level)
        out = np.zeros((h, w), np.uint8)
        self.ctx.check(self.lib.uslam_batch_keypoint_map(self.h, i, level, ptr(out)), "keypoint_map")
        return out

    def set_stream(self, cuda_stream: int | None):
        self.ctx.check(self.lib.uslam_batch_set_stream(self.h, C.c_void_p(cuda_stream or 0)), "set_stream")

    def profile(self, iters: int = 5) -> dict[str, float]:
        ms = np.zeros(len(KERNELS), np.float32)
        self.ctx.check(self.lib.uslam_batch_profile(self.h, iters, ptr(ms)), "profile")
        return dict(zip(KERNELS, (float(v) for v in ms)))

    def io_bytes(self) -> tuple[int, int]:
        a = C.c_size_t()
        b = C.c_size_t()
        self.ctx.check(self.lib.uslam_batch_io_bytes(self.h, C.byref(a), C.byref(b)), "io_bytes")
        return a.value, b.value

    def close(self):
        if self.h:
            self.lib.uslam_batch_destroy(self.h)
            self.h = None


class Frontend:
    """One camera stream: FeatureSet(0)/(1) on the device, matched per frame."""

    def __init__(self, ctx: Context, width: int, height: int):
        self.ctx = ctx
        self.lib = ctx.lib
        self.width, self.height = width, height
        h = C.c_void_p()
        ctx.check(self.lib.uslam_frontend_create(ctx.h, width, height, C.byref(h)), "frontend_create")
        self.h = h

    def process(self, img: np.ndarray | None, advance_reference: bool = False) -> bool:
        """Returns True when the frame was matched against a reference set."""
        if img is None:
            st = self.lib.uslam_frontend_process(self.h, None, 0, int(advance_reference))
        else:
            img = np.ascontiguousarray(img, dtype=np.uint8)
            st = self.lib.uslam_frontend_process(self.h, ptr(img), img.shape[1], int(advance_reference))
        self.ctx.check(st, "frontend_process", ok=(capi.OK, capi.NOT_READY))
        return st == capi.OK

    def process_f32(self, img: np.ndarray, advance_reference: bool = False, pitch: int | None = None) -> bool:
        """The reference's f32 FrameBW pixels (u8 / 255) of shape (H, pitch >= W);
        returns True when the frame was matched against a reference set."""
        img = np.ascontiguousarray(img, dtype=np.float32)
        st = self.lib.uslam_frontend_process_f32(self.h, ptr(img), pitch or img.shape[1], int(advance_reference))
        self.ctx.check(st, "frontend_process_f32", ok=(capi.OK, capi.NOT_READY))
        return st == capi.OK

    def input_device(self) -> tuple[int, int]:
        p = C.POINTER(C.c_uint8)()
        pitch = C.c_int()
        self.ctx.check(self.lib.uslam_frontend_input_device(self.h, C.byref(p), C.byref(pitch)), "input_device")
        return C.cast(p, C.c_void_p).value, pitch.value

    def enqueue(self, dev_ptr: int | None = None, pitch: int = 0, advance_reference: bool = False) -> bool:
        """Enqueue a frame already in device memory (None: the input buffer)."""
        m = C.c_int()
        self.ctx.check(self.lib.uslam_frontend_enqueue(self.h, C.c_void_p(dev_ptr or 0), pitch,
                                                       int(advance_reference), C.byref(m)), "enqueue")
        return bool(m.value)

    def sync(self):
        self.ctx.check(self.lib.uslam_frontend_sync(self.h), "frontend_sync")

    def features(self, which: int = 0):
        L = self.ctx.levels
        kept = np.zeros(L, np.int32)
        raw = np.zeros(L, np.int32)
        self.ctx.check(self.lib.uslam_frontend_features(self.h, which, None, 0, iptr(kept), iptr(raw)), "features")
        out = np.zeros(int(kept.sum()), FEATURE_DTYPE)
        self.ctx.check(self.lib.uslam_frontend_features(self.h, which, ptr(out), out.size, iptr(kept), iptr(raw)),
                       "features")
        return out, kept, raw

    def matches(self) -> np.ndarray:
        n = C.c_int()
        self.ctx.check(self.lib.uslam_frontend_matches(self.h, None, 0, C.byref(n)), "matches")
        out = np.zeros(n.value, MATCH_DTYPE)
        self.ctx.check(self.lib.uslam_frontend_matches(self.h, ptr(out), out.size, C.byref(n)), "matches")
        return out

    def close(self):
        if self.h:
            self.lib.uslam_frontend_destroy(self.h)
            self.h = None


class Server:
    """Served form: camera streams, HBM-budget admission, continuous batching."""

    def __init__(self, ctx: Context, sizes: list[tuple[int, int]], hbm_budget_bytes: int = 4 << 30,
                 max_batch: int = 64):
        self.ctx = ctx
        self.lib = ctx.lib
        self._w = np.array([s[0] for s in sizes], np.int32)
        self._h = np.array([s[1] for s in sizes], np.int32)
        p = capi.ServerParams(len(sizes), iptr(self._w), iptr(self._h), hbm_budget_bytes, max_batch)
        h = C.c_void_p()
        ctx.check(self.lib.uslam_server_create(ctx.h, C.byref(p), C.byref(h)), "server_create")
        self.h = h

    def open_stream(self, width: int, height: int) -> int:
        sid = C.c_int()
        self.ctx.check(self.lib.uslam_server_open_stream(self.h, width, height, C.byref(sid)), "open_stream")
        return sid.value

    def submit(self, stream: int, img: np.ndarray, promote: bool = False) -> int | None:
        """Ticket of the queued frame, or None when admission is refused (no free slot)."""
        img = np.ascontiguousarray(img, np.uint8)
        t = C.c_uint64()
        st = self.lib.uslam_server_submit(self.h, stream, ptr(img), img.shape[1], int(promote), C.byref(t))
        if st == capi.CAPACITY:
            return None
        self.ctx.check(st, "submit")
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 0):
        self.ctx.check(self.lib.uslam_server_wait(self.h, ticket, timeout_ms), "wait")

    def result(self, ticket: int):
        """(features, kept, raw, matches or None, latency_ms)."""
        L = self.ctx.levels
        kept = np.zeros(L, np.int32)
        raw = np.zeros(L, np.int32)
        nm = C.c_int()
        lat = C.c_double()
        st = self.lib.uslam_server_result(self.h, ticket, None, 0, iptr(kept), iptr(raw), None, 0, C.byref(nm),
                                          C.byref(lat))
        self.ctx.check(st, "result", ok=(capi.OK, capi.NOT_READY))
        feats = np.zeros(int(kept.sum()), FEATURE_DTYPE)
        m = np.zeros(nm.value, MATCH_DTYPE)
        st = self.lib.uslam_server_result(self.h, ticket, ptr(feats), feats.size, iptr(kept), iptr(raw), ptr(m),
                                          m.size, C.byref(nm), C.byref(lat))
        self.ctx.check(st, "result", ok=(capi.OK, capi.NOT_READY))
        return feats, kept, raw, (m if st == capi.OK else None), lat.value

    def result_into(self, ticket: int, feats: np.ndarray, matches: np.ndarray, kept: np.ndarray,
                    raw: np.ndarray) -> tuple[int, int, float]:
        """Results of a finished request into caller buffers (one call; the
        server already holds them in host memory): (features, matches,
        server latency in ms); the counts per level land in kept / raw."""
        nm = C.c_int()
        lat = C.c_double()
        st = self.lib.uslam_server_result(self.h, ticket, ptr(feats), feats.size, iptr(kept), iptr(raw), ptr(matches),
                                          matches.size, C.byref(nm), C.byref(lat))
        self.ctx.check(st, "result", ok=(capi.OK, capi.NOT_READY))
        return int(kept.sum()), (nm.value if st == capi.OK else 0), lat.value

    def latency_ms(self, ticket: int) -> float:
        """Submit-to-completion time of a finished request (no data copied)."""
        lat = C.c_double()
        st = self.lib.uslam_server_result(self.h, ticket, None, 0, None, None, None, 0, None, C.byref(lat))
        self.ctx.check(st, "result", ok=(capi.OK, capi.NOT_READY))
        return lat.value

    def release(self, ticket: int):
        self.ctx.check(self.lib.uslam_server_release(self.h, ticket), "release")

    def stats(self) -> dict:
        a, b = C.c_uint64(), C.c_uint64()
        c, d = C.c_int(), C.c_int()
        self.ctx.check(self.lib.uslam_server_stats(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)), "stats")
        return {"launches": a.value, "frames": b.value, "max_batch_seen": c.value, "slots": d.value}

    def close(self):
        if self.h:
            self.lib.uslam_server_destroy(self.h)
            self.h = None


class FeatureSet:
    """A device-resident feature set of one frame size (uslam_featset):
    detect(frame) fills it from a u8 frame or an f32 frame in [0, 1]."""

    def __init__(self, ctx: Context, width: int, height: int):
        self.ctx, self.lib = ctx, ctx.lib
        self.width, self.height = width, height
        h = C.c_void_p()
        ctx.check(self.lib.uslam_featset_create(ctx.h, width, height, C.byref(h)), "featset_create")
        self.h = h

    def detect(self, frame: np.ndarray):
        if frame.dtype == np.float32:
            img = np.ascontiguousarray(frame, np.float32)
            fn = self.lib.uslam_detect_describe_f32
        else:
            img = np.ascontiguousarray(frame, np.uint8)
            fn = self.lib.uslam_detect_describe
        h, w = img.shape
        self.ctx.check(fn(self.ctx.h, ptr(img), w, h, w, self.h), "detect_describe")

    def features(self):
        levels = self.ctx.levels
        kept = np.zeros(levels, np.int32)
        raw = np.zeros(levels, np.int32)
        self.ctx.check(self.lib.uslam_featset_features(self.h, None, 0, iptr(kept), iptr(raw)), "featset_features")
        out = np.zeros(int(kept.sum()), FEATURE_DTYPE)
        self.ctx.check(self.lib.uslam_featset_features(self.h, ptr(out), out.size, iptr(kept), iptr(raw)),
                       "featset_features")
        return out, kept, raw

    def close(self):
        if self.h:
            self.lib.uslam_featset_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
