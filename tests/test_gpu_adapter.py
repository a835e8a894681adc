"""The C++ drop-in passes (include/uslam_wslam.hpp), compiled against
stand-ins of the reference's headers and run the way the reference's stages
run them: every frame's FeatureSet(0) and MatchResult equal the oracle's,
with the reference's FeatureSet(1) rotation and STAGE_STOP on the first frame."""
import os
import struct
import subprocess

import numpy as np
import pytest

import oracle
from uni_slam_gb300 import synth

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
FEAT = np.dtype([("x", "<u4"), ("y", "<u4"), ("lod", "<u4"), ("strength", "<u4"), ("orientation", "<f4"),
                 ("descriptor", "<u4", (8,))])


def _build(tmp_path):
    exe = str(tmp_path / "adapter_main")
    lib = os.path.join(REPO, "uni_slam_gb300")
    cmd = ["g++", "-std=c++20", "-O1", "-I", os.path.join(HERE, "adapter", "stubs"), "-I",
           os.path.join(REPO, "include"), os.path.join(HERE, "adapter", "adapter_main.cpp"), "-o", exe,
           "-L", lib, "-luslam", f"-Wl,-rpath,{lib}"]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def test_wslam_passes_match_oracle(tmp_path, brief_pattern):
    exe = _build(tmp_path)
    W, H = 752, 480
    frames = synth.plane_sequence(11, n=5)
    advance = [0, 0, 1, 0, 1]
    (tmp_path / "pattern.bin").write_bytes(np.ascontiguousarray(brief_pattern, "<i4").tobytes())
    with open(tmp_path / "frames.bin", "wb") as f:
        f.write(struct.pack("<3i", len(frames), W, H))
        for img, adv in zip(frames, advance):
            f.write(struct.pack("<i", adv))
            f.write(np.ascontiguousarray(img, np.uint8).tobytes())
    r = subprocess.run([exe, str(tmp_path / "pattern.bin"), str(tmp_path / "frames.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    buf = (tmp_path / "out.bin").read_bytes()
    pos = 0

    def take(fmt):
        nonlocal pos
        v = struct.unpack_from(fmt, buf, pos)
        pos += struct.calcsize(fmt)
        return v

    ref_set, cur_set = None, None
    for i, (img, adv) in enumerate(zip(frames, advance)):
        status, = take("<i")
        counts = np.array(take("<6i"))
        n = int(counts.sum())
        got = np.frombuffer(buf, FEAT, count=n, offset=pos)
        pos += n * FEAT.itemsize
        nm, = take("<i")
        pairs = sorted(tuple(take("<6i")) for _ in range(nm))
        exp = oracle.frame(img, brief_pattern)
        if cur_set is not None and (ref_set is None or adv):
            ref_set = cur_set
        cur_set = exp
        assert status == (1 if ref_set is None else 0), f"frame {i}"
        assert np.array_equal(counts, exp[1])
        ef = exp[0]
        lods = np.repeat(np.arange(6), exp[1])
        assert np.array_equal(got["x"], ef["x"].astype(np.uint32)) and np.array_equal(got["y"], ef["y"].astype(np.uint32))
        assert np.array_equal(got["lod"], lods) and np.array_equal(got["descriptor"], ef["descriptor"])
        assert np.array_equal(got["orientation"].view(np.uint32), ef["orientation"].view(np.uint32))
        if ref_set is None:
            assert nm == 0
            continue
        m = oracle.match(ref_set[0], ref_set[1], exp[0], exp[1], W, H)
        aoff = np.concatenate([[0], np.cumsum(ref_set[1])])
        boff = np.concatenate([[0], np.cumsum(exp[1])])
        want = sorted((lb, int(exp[0][boff[lb] + ib]["x"]), int(exp[0][boff[lb] + ib]["y"]),
                       la, int(ref_set[0][aoff[la] + ia]["x"]), int(ref_set[0][aoff[la] + ia]["y"]))
                      for la, ia, lb, ib in m)
        assert len(want) > 100
        assert pairs == want, f"frame {i}"
