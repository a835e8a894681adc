"""The BRIEF test pattern: 256 point pairs (ax, ay, bx, by).

The reference compiles its pattern in from wslam/src/feature_detect/brief_tests.inc
(the ORB learned pattern, included at generate_features.cpp:458-460) and uploads
it once as a uniform (GenerateFeaturesPass::writeConstantValues,
generate_features.cpp:450-493).  This library likewise takes the pattern as an
input of ``uslam_create``: the caller supplies the same table it already
compiles in.  The table is not part of this repository; ``stage_from_reference``
extracts it from a reference checkout into a git-ignored staging file that the
tests, smoke check and benchmark read.
"""
from __future__ import annotations

import hashlib
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
STAGED = os.path.join(HERE, "_staged", "brief_pattern.txt")
REF_RELPATH = os.path.join("wslam", "src", "feature_detect", "brief_tests.inc")


def parse_inc(text: str) -> np.ndarray:
    """Parse a C initializer list of ints (comments allowed) into (256, 4) int32."""
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    vals = [int(v) for v in re.findall(r"-?\d+", text)]
    if len(vals) != 1024:
        raise ValueError(f"expected 1024 integers in the BRIEF table, found {len(vals)}")
    return np.asarray(vals, dtype=np.int32).reshape(256, 4)


def stage_from_reference(ref_root: str) -> str | None:
    """Extract the pattern from a reference checkout; returns the staged path."""
    src = os.path.join(ref_root, REF_RELPATH)
    if not os.path.exists(src):
        return None
    with open(src, "r", encoding="utf-8") as f:
        pat = parse_inc(f.read())
    os.makedirs(os.path.dirname(STAGED), exist_ok=True)
    body = "\n".join(" ".join(str(int(v)) for v in row) for row in pat) + "\n"
    tmp = STAGED + ".tmp"
    with open(tmp, "w", encoding="utf-8") as f:
        f.write(body)
    os.replace(tmp, STAGED)
    return STAGED


def load(path: str | None = None) -> np.ndarray:
    """Load the staged pattern as a contiguous (256, 4) int32 array."""
    path = path or os.environ.get("USLAM_BRIEF_PATTERN", STAGED)
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"BRIEF pattern not staged at {path}; run __graft_entry__.build() on a machine with the "
            "reference checkout, or point USLAM_BRIEF_PATTERN at a 256x4 integer table"
        )
    arr = np.loadtxt(path, dtype=np.int32).reshape(256, 4)
    return np.ascontiguousarray(arr)


def digest(pat: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(pat, dtype="<i4").tobytes()).hexdigest()
