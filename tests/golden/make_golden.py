"""Regenerate the golden fixtures of tests/golden (run where the reference
checkout is present, after `make -C oracle`).

matcher_cases.npz — feature-set pairs and the mutual matches computed by the
reference's own wslam/src/pose_estimate_cpu/match_features_cpu.cpp, compiled
unmodified by oracle/Makefile (oracle/_ref/libref_matcher_<W>x<H>.so).
synth_digests.json — SHA-256 of seeded synthetic frames (generator pins).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

import oracle  # noqa: E402
from uni_slam_gb300 import synth  # noqa: E402

FEATURE_DTYPE = oracle.FEATURE_DTYPE


def _features(rs, dims, counts):
    feats = []
    for (w, h), n in zip(dims, counts):
        f = np.zeros(n, FEATURE_DTYPE)
        # unique (x, y) per level, sorted (y, x) like the front-end's output
        idx = rs.choice(w * h, size=n, replace=False)
        idx.sort()
        f["x"] = (idx % w).astype(np.float32)
        f["y"] = (idx // w).astype(np.float32)
        f["strength"] = rs.randint(10, 18, size=n)
        f["orientation"] = rs.uniform(-np.pi, np.pi, size=n).astype(np.float32)
        f["descriptor"] = rs.randint(0, 2**32, size=(n, 8), dtype=np.uint64).astype(np.uint32)
        feats.append(f)
    return feats


def _perturb(rs, feats, dims, flip_p, jitter, drop_p, extra):
    out = []
    for (w, h), f in zip(dims, feats):
        g = f.copy()
        keep = rs.uniform(size=len(g)) >= drop_p
        g = g[keep]
        g["x"] = np.clip(g["x"] + rs.randint(-jitter, jitter + 1, size=len(g)), 0, w - 1)
        g["y"] = np.clip(g["y"] + rs.randint(-jitter, jitter + 1, size=len(g)), 0, h - 1)
        bits = rs.uniform(size=(len(g), 256)) < flip_p
        flips = np.packbits(bits, axis=1, bitorder="little").view("<u4")
        g["descriptor"] ^= flips
        if extra:
            g = np.concatenate([g, _features(rs, [(w, h)], [extra])[0]])
        # deduplicate positions, order (y, x)
        key = g["y"].astype(np.int64) * w + g["x"].astype(np.int64)
        _, first = np.unique(key, return_index=True)
        g = g[np.sort(first)]
        key = g["y"].astype(np.int64) * w + g["x"].astype(np.int64)
        g = g[np.argsort(key, kind="stable")]
        out.append(g)
    return out


def matcher_cases():
    cases = []
    for k, (W, H) in enumerate([(752, 480), (752, 480), (752, 480), (1280, 720)]):
        rs = np.random.RandomState(1000 + k)
        dims = oracle.level_dims(W, H, 6)
        counts = [int(c) for c in rs.randint(20, 90, size=6)]
        if k == 1:
            counts[3] = 0  # an empty level
            counts[5] = 1  # a pool of size < 2 for its neighbour queries
        a = _features(rs, dims, counts)
        b = _perturb(rs, a, dims, flip_p=0.08 if k != 2 else 0.0, jitter=2, drop_p=0.2, extra=15)
        if k == 2:
            # exact duplicates of descriptors: ties on the best distance
            for lvl in b:
                if len(lvl) > 4:
                    lvl["descriptor"][1] = lvl["descriptor"][0]
        cases.append((W, H, a, b))
    return cases


def main():
    out = {}
    for k, (W, H, a, b) in enumerate(matcher_cases()):
        ref = oracle.ref_matcher(W, H)
        if ref is None:
            raise SystemExit(f"reference matcher {W}x{H} not built (make -C oracle with the reference present)")
        ka = np.array([len(x) for x in a], np.int32)
        kb = np.array([len(x) for x in b], np.int32)
        fa = np.concatenate(a)
        fb = np.concatenate(b)
        m = ref(fa, ka, fb, kb)
        out[f"c{k}_size"] = np.array([W, H], np.int32)
        out[f"c{k}_a"] = fa.view(np.uint8)
        out[f"c{k}_ka"] = ka
        out[f"c{k}_b"] = fb.view(np.uint8)
        out[f"c{k}_kb"] = kb
        out[f"c{k}_matches"] = m
        print(f"case {k}: {W}x{H} a={ka.sum()} b={kb.sum()} matches={len(m)}")
    out["n_cases"] = np.array([len(matcher_cases())], np.int32)
    np.savez_compressed(os.path.join(HERE, "matcher_cases.npz"), **out)

    digests = {}
    for seed in (0, 1, 2):
        f1, f2 = synth.warped_pair(seed)
        digests[f"warped_pair/{seed}/0"] = synth.frame_digest(f1)
        digests[f"warped_pair/{seed}/1"] = synth.frame_digest(f2)
    for seed in (0,):
        frames = synth.plane_sequence(seed, n=3)
        for i, f in enumerate(frames):
            digests[f"plane_sequence/{seed}/{i}"] = synth.frame_digest(f)
    with open(os.path.join(HERE, "synth_digests.json"), "w") as f:
        json.dump(digests, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
