"""The matcher entry point for callers that cannot allocate device memory
(uslam_match_noalloc): through the C ABI, on caller-owned device buffers, it
must return exactly the matches of the batch path, on two calls in a row
(its shared scratch keeps the previous call's contents)."""
import ctypes as C

import numpy as np
import pytest

from uni_slam_gb300 import Batch, Context, capi, synth

pytestmark = pytest.mark.gpu


def _rows(m):
    return np.stack([m["lod_a"], m["idx_a"], m["lod_b"], m["idx_b"]], 1) if len(m) else np.zeros((0, 4), np.int32)


def test_noalloc_match_equals_batch_path(brief_pattern):
    import torch

    lib = capi.load()
    W, H, L = 752, 480, 6
    frames = []
    for seed in (21, 22):
        frames += list(synth.warped_pair(seed))
    with Context(brief_pattern, levels=L, max_width=W, max_height=H) as ctx:
        b = Batch(ctx, [(W, H)] * 4, [(0, 1), (2, 3)])
        try:
            b.process(frames)
            feats = [b.features(i) for i in range(4)]
            expected = [_rows(b.matches(p)) for p in range(2)]
        finally:
            b.close()
    stream = torch.cuda.current_stream().cuda_stream
    err = C.create_string_buffer(256)
    for call, (ia, ib) in enumerate([(0, 1), (2, 3)]):
        fa, ka, _ = feats[ia]
        fb, kb, _ = feats[ib]
        da = torch.from_numpy(fa.view(np.uint8).copy()).cuda()
        db = torch.from_numpy(fb.view(np.uint8).copy()).cuda()
        cap_out = int(ka.max())
        out = torch.full((L * cap_out * 4,), -7, dtype=torch.int32, device="cuda")
        counts = torch.zeros(L, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        ka32 = np.ascontiguousarray(ka, np.int32)
        kb32 = np.ascontiguousarray(kb, np.int32)
        st = lib.uslam_match_noalloc(0, W, H, L, C.c_void_p(da.data_ptr()), capi.iptr(ka32),
                                     C.c_void_p(db.data_ptr()), capi.iptr(kb32), C.c_void_p(out.data_ptr()),
                                     C.c_void_p(counts.data_ptr()), cap_out, C.c_void_p(stream), err, len(err))
        assert st == capi.OK, err.value.decode()
        o = out.cpu().numpy().reshape(L, cap_out, 4)
        n = counts.cpu().numpy()
        got = np.concatenate([o[l, :n[l]] for l in range(L)]) if n.sum() else np.zeros((0, 4), np.int32)
        assert len(expected[call]) > 100
        assert np.array_equal(got, expected[call]), f"call {call}"


def test_noalloc_rejects_oversize_and_bad_args():
    lib = capi.load()
    err = C.create_string_buffer(256)
    big = np.full(6, 200000, np.int32)  # scratch need far beyond the fixed maximum
    st = lib.uslam_match_noalloc(0, 752, 480, 6, C.c_void_p(1), capi.iptr(big), C.c_void_p(1), capi.iptr(big),
                                 C.c_void_p(1), C.c_void_p(1), 200000, None, err, len(err))
    assert st == capi.CAPACITY and b"fixed maximum" in err.value
    small = np.zeros(6, np.int32)
    st = lib.uslam_match_noalloc(0, 0, 480, 6, None, capi.iptr(small), None, capi.iptr(small), C.c_void_p(1),
                                 C.c_void_p(1), 1, None, err, len(err))
    assert st == capi.INVALID_ARG
