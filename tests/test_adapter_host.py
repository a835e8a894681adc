"""The C++ drop-in passes (include/uslam_wslam.hpp) compile against stand-ins
of the reference's headers, link against libuslam.so, and return the
reference's Pass-contract results on the paths that need no GPU work:
STAGE_STOP while no reference set exists (match_features_cpu.cpp:229-236),
an error string for a missing current set or frame, and on a machine without
a GPU an error string from the failed context creation instead of a crash."""
import os
import subprocess

import numpy as np

from uni_slam_gb300 import capi

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _run(tmp_path, brief_pattern):
    capi.load()  # the library must exist (built by __graft_entry__.build())
    exe = str(tmp_path / "adapter_errors")
    lib = os.path.join(REPO, "uni_slam_gb300")
    subprocess.run(["g++", "-std=c++20", "-O1", "-Wall", "-Werror", "-I", os.path.join(HERE, "adapter", "stubs"),
                    "-I", os.path.join(REPO, "include"), os.path.join(HERE, "adapter", "adapter_errors.cpp"),
                    "-o", exe, "-L", lib, "-luslam", f"-Wl,-rpath,{lib}"], check=True, capture_output=True)
    pat = tmp_path / "pattern.bin"
    pat.write_bytes(np.ascontiguousarray(brief_pattern, "<i4").tobytes())
    r = subprocess.run([exe, str(pat)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    return dict(line.split(": ", 1) for line in r.stdout.splitlines())


def test_pass_error_paths(tmp_path, brief_pattern):
    out = _run(tmp_path, brief_pattern)
    assert out["ids"] == "[Cuda feature detect pass] | [Cuda match features pass]"
    assert out["init"] == "ok"
    assert out["match_without_reference"] == "STAGE_STOP"
    assert out["match_without_current"] == "no current feature set"
    assert out["detect_without_frame"] == "no frame under res:frame:0:lod:0"
    if _device_count() > 0:
        assert out["detect_with_frame"] == "ok"
    else:
        assert out["detect_with_frame"] == "uslam_create: cuda error", out["detect_with_frame"]


def _device_count() -> int:
    import torch

    return torch.cuda.device_count()
