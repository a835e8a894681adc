"""The C-ABI library loads and exports every symbol declared in include/*.h,
and its host-only entry points behave (no GPU needed)."""
import ctypes as C
import glob
import os
import re

import numpy as np

import oracle
from uni_slam_gb300 import capi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:uslam_status|void|const char\*)\s+(uslam_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    lib = capi.load()
    declared = _declared()
    assert len(declared) >= 25
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    assert declared <= set(capi.SIGNATURES), sorted(declared - set(capi.SIGNATURES))


def test_level_dims_match_oracle():
    from uni_slam_gb300 import level_dims
    for W, H in [(752, 480), (640, 480), (1280, 720), (1920, 1080), (3840, 2160), (10, 10), (33, 17)]:
        assert level_dims(W, H, 6) == oracle.level_dims(W, H, 6)


def test_status_strings_and_invalid_args():
    lib = capi.load()
    assert lib.uslam_status_string(capi.OK) == b"ok"
    assert lib.uslam_status_string(capi.TIMEOUT) == b"timeout"
    w = np.zeros(6, np.int32)
    assert lib.uslam_level_dims(0, 480, 6, capi.iptr(w), capi.iptr(w)) == capi.INVALID_ARG
    assert lib.uslam_create(None, None) == capi.INVALID_ARG
    p = capi.Params(0, 0, 752, 480, 0, None)  # zero levels, null pattern
    h = C.c_void_p()
    assert lib.uslam_create(C.byref(p), C.byref(h)) == capi.INVALID_ARG
    assert lib.uslam_cull_coverage(752, 480, 800, 480, capi.ptr(w)) == capi.INVALID_ARG
    assert lib.uslam_last_error(None) == b"null context"
