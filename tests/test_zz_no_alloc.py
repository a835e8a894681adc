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
    free_before = None
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
        if call == 1:
            # the second call: every kernel it runs is loaded, so any change of
            # the device's free memory would be an allocation by the call
            free_before = torch.cuda.mem_get_info(0)[0]
            torch_before = torch.cuda.memory_allocated(0)
        st = lib.uslam_match_noalloc(0, W, H, L, C.c_void_p(da.data_ptr()), capi.iptr(ka32),
                                     C.c_void_p(db.data_ptr()), capi.iptr(kb32), C.c_void_p(out.data_ptr()),
                                     C.c_void_p(counts.data_ptr()), cap_out, C.c_void_p(stream), err, len(err))
        assert st == capi.OK, err.value.decode()
        if call == 1:
            assert torch.cuda.mem_get_info(0)[0] == free_before, "the call allocated device memory"
            assert torch.cuda.memory_allocated(0) == torch_before
        o = out.cpu().numpy().reshape(L, cap_out, 4)
        n = counts.cpu().numpy()
        got = np.concatenate([o[l, :n[l]] for l in range(L)]) if n.sum() else np.zeros((0, 4), np.int32)
        assert len(expected[call]) > 100
        assert np.array_equal(got, expected[call]), f"call {call}"


def test_noalloc_rejects_oversize_and_bad_args():
    """Sizes beyond the fixed scratch and bad arguments are refused on the
    host, with real device buffers in every pointer argument."""
    import torch

    lib = capi.load()
    err = C.create_string_buffer(256)
    feats = torch.zeros(48 * 64, dtype=torch.uint8, device="cuda")
    out = torch.zeros(6 * 16, dtype=torch.int32, device="cuda")
    counts = torch.zeros(6, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    fp, op, cp = C.c_void_p(feats.data_ptr()), C.c_void_p(out.data_ptr()), C.c_void_p(counts.data_ptr())
    big = np.full(6, 200000, np.int32)  # scratch need far beyond the fixed maximum
    st = lib.uslam_match_noalloc(0, 752, 480, 6, fp, capi.iptr(big), fp, capi.iptr(big), op, cp, 200000, None, err,
                                 len(err))
    assert st == capi.CAPACITY and b"fixed maximum" in err.value
    small = np.zeros(6, np.int32)
    st = lib.uslam_match_noalloc(0, 0, 480, 6, fp, capi.iptr(small), fp, capi.iptr(small), op, cp, 1, None, err,
                                 len(err))
    assert st == capi.INVALID_ARG


def test_noalloc_rejects_misaligned_records():
    """A feature array that is not 16-byte aligned (a sub-pointer into a
    caller's pool, here 4 bytes in) is refused before any device work."""
    import torch

    lib = capi.load()
    err = C.create_string_buffer(256)
    feats = torch.zeros(48 * 8 + 16, dtype=torch.uint8, device="cuda")
    out = torch.zeros(6 * 4 * 4, dtype=torch.int32, device="cuda")
    counts = torch.zeros(6, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    k = np.array([2, 0, 0, 0, 0, 0], np.int32)
    base = feats.data_ptr()
    assert base % 16 == 0
    for pa, pb in ((base + 4, base), (base, base + 4)):
        st = lib.uslam_match_noalloc(0, 752, 480, 6, C.c_void_p(pa), capi.iptr(k), C.c_void_p(pb), capi.iptr(k),
                                     C.c_void_p(out.data_ptr()), C.c_void_p(counts.data_ptr()), 4, None, err,
                                     len(err))
        assert st == capi.INVALID_ARG and b"16-byte" in err.value, (st, err.value)


def _flip(d: np.ndarray, n: int, rs) -> np.ndarray:
    bits = np.unpackbits(d.view(np.uint8), bitorder="little")
    bits[rs.choice(256, n, replace=False)] ^= 1
    return np.packbits(bits, bitorder="little").view("<u4")


@pytest.mark.parametrize("d1,d2,expected", [(17, 20, 0), (16, 19, 1)])
def test_noalloc_ratio_boundary(d1, d2, expected):
    """Planted descriptors at the Lowe-ratio boundary (accept iff
    (float)best < 0.85f * (float)second, match_features_cpu.cpp:142-146):
    0.85f * 20 rounds to exactly 17.0f in f32, so best 17 against second 20
    is rejected, and 16 against 19 (16.15) accepted.  One previous feature
    a0 meets the current features b0 (distance d1) and b1 (d2) in its
    window; a far feature a1 keeps both pools at two."""
    import torch

    import oracle

    assert not np.float32(17) < np.float32(0.85) * np.float32(20)
    lib = capi.load()
    W, H, L = 752, 480, 6
    rs = np.random.RandomState(d1)
    D = rs.randint(0, 2**32, size=8, dtype=np.uint64).astype(np.uint32)
    fa = np.zeros(2, oracle.FEATURE_DTYPE)
    fa["x"], fa["y"], fa["strength"] = [100, 600], [100, 400], 12
    fa["descriptor"][0], fa["descriptor"][1] = D, ~D
    fb = np.zeros(2, oracle.FEATURE_DTYPE)
    fb["x"], fb["y"], fb["strength"] = [102, 110], [101, 104], 12
    fb["descriptor"][0], fb["descriptor"][1] = _flip(D, d1, rs), _flip(D, d2, rs)
    ka = np.array([2, 0, 0, 0, 0, 0], np.int32)
    kb = ka.copy()
    em = oracle.match(fa, ka, fb, kb, W, H)
    assert len(em) == expected
    da = torch.from_numpy(fa.view(np.uint8).copy()).cuda()
    db = torch.from_numpy(fb.view(np.uint8).copy()).cuda()
    out = torch.full((L * 2 * 4,), -7, dtype=torch.int32, device="cuda")
    counts = torch.zeros(L, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    err = C.create_string_buffer(256)
    st = lib.uslam_match_noalloc(0, W, H, L, C.c_void_p(da.data_ptr()), capi.iptr(ka), C.c_void_p(db.data_ptr()),
                                 capi.iptr(kb), C.c_void_p(out.data_ptr()), C.c_void_p(counts.data_ptr()), 2,
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream), err, len(err))
    assert st == capi.OK, err.value.decode()
    o = out.cpu().numpy().reshape(L, 2, 4)
    n = counts.cpu().numpy()
    got = np.concatenate([o[l, :n[l]] for l in range(L)]) if n.sum() else np.zeros((0, 4), np.int32)
    assert np.array_equal(got, em)


@pytest.mark.parametrize("case", [0, 1])
def test_noalloc_window_edge_pair(case):
    """The symmetric matcher computes each pair's distance once for both
    directions, and at the window's x edge the directions see different
    candidates (tests/planted.py): only the far pair may match, as in the
    oracle and the compiled reference."""
    import torch

    import oracle
    import planted

    lib = capi.load()
    fa, ka, fb, kb = planted.window_edge_sets(case)
    em = oracle.match(fa, ka, fb, kb, planted.W, planted.H)
    assert len(em) == 1
    L = planted.L
    da = torch.from_numpy(fa.view(np.uint8).copy()).cuda()
    db = torch.from_numpy(fb.view(np.uint8).copy()).cuda()
    out = torch.full((L * 2 * 4,), -7, dtype=torch.int32, device="cuda")
    counts = torch.zeros(L, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    err = C.create_string_buffer(256)
    st = lib.uslam_match_noalloc(0, planted.W, planted.H, L, C.c_void_p(da.data_ptr()), capi.iptr(ka),
                                 C.c_void_p(db.data_ptr()), capi.iptr(kb), C.c_void_p(out.data_ptr()),
                                 C.c_void_p(counts.data_ptr()), 2, C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                 err, len(err))
    assert st == capi.OK, err.value.decode()
    o = out.cpu().numpy().reshape(L, 2, 4)
    n = counts.cpu().numpy()
    got = np.concatenate([o[l, :n[l]] for l in range(L)]) if n.sum() else np.zeros((0, 4), np.int32)
    assert np.array_equal(got, em)


def test_noalloc_rejects_records_outside_level():
    """Records whose x is not an integer inside its level are refused with
    USLAM_INVALID_ARG before any kernel indexes by them (the planted values,
    x = w and x = 10.5, stay inside the sort's histogram even unchecked),
    and the next valid call succeeds."""
    import torch

    import oracle

    lib = capi.load()
    W, H, L = 752, 480, 6
    f = np.zeros(2, oracle.FEATURE_DTYPE)
    f["x"], f["y"], f["strength"] = [100, 110], [100, 104], 12
    f["descriptor"] = np.random.RandomState(3).randint(0, 2**32, size=(2, 8), dtype=np.uint64).astype(np.uint32)
    k = np.array([2, 0, 0, 0, 0, 0], np.int32)
    out = torch.zeros((L * 2 * 4,), dtype=torch.int32, device="cuda")
    counts = torch.zeros(L, dtype=torch.int32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    err = C.create_string_buffer(256)

    def call(fa, fb):
        da = torch.from_numpy(fa.view(np.uint8).copy()).cuda()
        db = torch.from_numpy(fb.view(np.uint8).copy()).cuda()
        torch.cuda.synchronize()
        return lib.uslam_match_noalloc(0, W, H, L, C.c_void_p(da.data_ptr()), capi.iptr(k), C.c_void_p(db.data_ptr()),
                                       capi.iptr(k), C.c_void_p(out.data_ptr()), C.c_void_p(counts.data_ptr()), 2,
                                       stream, err, len(err))

    for bad_x, which in ((float(W), 0), (10.5, 1)):
        g = f.copy()
        g["x"][1] = bad_x
        st = call(g, f) if which == 0 else call(f, g)
        assert st == capi.INVALID_ARG and b"inside its level" in err.value, (bad_x, st, err.value)
    assert call(f, f) == capi.OK, err.value.decode()
