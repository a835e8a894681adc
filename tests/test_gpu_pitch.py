"""Frames given with a row pitch larger than their width, the padding bytes
filled with noise, through every entry point that takes a pitch: the batch's
staging copy (uslam_batch_set_frame), the frontend from host memory
(uslam_frontend_process) and from device memory (uslam_frontend_enqueue),
the single-frame sets (uslam_detect_describe, and uslam_detect_describe_f32
with its pitch in floats), and the server (uslam_server_submit).  Every
result equals the oracle's on the unpadded frame: no padding byte is read."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from uni_slam_gb300 import Batch, Context, FeatureSet, Frontend, Server, capi, synth

pytestmark = pytest.mark.gpu

W, H, PITCH = 752, 480, 800


def _padded(img: np.ndarray, seed: int) -> np.ndarray:
    p = np.random.RandomState(seed).randint(0, 256, size=(img.shape[0], PITCH)).astype(np.uint8)
    p[:, : img.shape[1]] = img
    return p


def _mm(m):
    if len(m) == 0:
        return np.zeros((0, 4), np.int32)
    return np.stack([m["lod_a"], m["idx_a"], m["lod_b"], m["idx_b"]], 1)


def _same(got, exp):
    gf, gk, gr = got[:3]
    assert np.array_equal(gk, exp[1]) and np.array_equal(gr, exp[2])
    assert gf.tobytes() == exp[0].tobytes()


def test_padded_rows_every_entry_point(brief_pattern):
    f0, f1 = synth.warped_pair(31)
    p0, p1 = _padded(f0, 1), _padded(f1, 2)
    e0, e1 = oracle.frame(f0, brief_pattern), oracle.frame(f1, brief_pattern)
    em = oracle.match(e0[0], e0[1], e1[0], e1[1], W, H)
    assert len(em) > 100
    with Context(brief_pattern, levels=6, max_width=W, max_height=H) as c:
        lib = c.lib
        # batch: staging copy with the caller's pitch
        b = Batch(c, [(W, H), (W, H)], [(0, 1)])
        try:
            for i, p in enumerate((p0, p1)):
                c.check(lib.uslam_batch_set_frame(b.h, i, capi.ptr(p), PITCH), "set_frame")
            b.upload()
            b.run()
            b.download()
            b.sync()
            _same(b.features(0), e0)
            _same(b.features(1), e1)
            assert np.array_equal(_mm(b.matches(0)), em)
        finally:
            b.close()
        # frontend: host memory, then device memory, each with the caller's pitch
        fe = Frontend(c, W, H)
        try:
            c.check(lib.uslam_frontend_process(fe.h, capi.ptr(p0), PITCH, 0), "process", ok=(capi.OK, capi.NOT_READY))
            _same(fe.features(0), e0)
            dev = torch.from_numpy(p1).cuda()
            torch.cuda.synchronize()
            m = C.c_int()
            c.check(lib.uslam_frontend_enqueue(fe.h, C.c_void_p(dev.data_ptr()), PITCH, 0, C.byref(m)), "enqueue")
            fe.sync()
            assert m.value == 1
            _same(fe.features(0), e1)
            assert np.array_equal(_mm(fe.matches()), em)
        finally:
            fe.close()
        # frontend on the reference's f32 FrameBW pixels, padded rows (pitch in
        # floats): the bytes are recovered while staging, the results come back
        # with the frame (the reference set's too)
        fe = Frontend(c, W, H)
        try:
            q0 = (p0.astype(np.float32) / np.float32(255.0)).astype(np.float32)
            q1 = (p1.astype(np.float32) / np.float32(255.0)).astype(np.float32)
            assert not fe.process_f32(q0, pitch=PITCH)
            _same(fe.features(0), e0)
            assert fe.process_f32(q1, pitch=PITCH)
            _same(fe.features(0), e1)
            _same(fe.features(1), e0)
            assert np.array_equal(_mm(fe.matches()), em)
        finally:
            fe.close()
        # single-frame sets: u8 (pitch in bytes) and f32 (pitch in floats)
        with FeatureSet(c, W, H) as a, FeatureSet(c, W, H) as bset:
            c.check(lib.uslam_detect_describe(c.h, capi.ptr(p0), W, H, PITCH, a.h), "detect_describe")
            pf = (p1.astype(np.float32) / np.float32(255.0)).astype(np.float32)
            c.check(lib.uslam_detect_describe_f32(c.h, capi.ptr(pf), W, H, PITCH, bset.h), "detect_describe_f32")
            _same(a.features(), e0)
            _same(bset.features(), e1)
            assert np.array_equal(_mm(c.match(a, bset)), em)
        # server: the submit copy with the caller's pitch
        s = Server(c, [(W, H)], hbm_budget_bytes=1 << 30, max_batch=4)
        try:
            sid = s.open_stream(W, H)
            tickets = []
            for p in (p0, p1):
                t = C.c_uint64()
                c.check(lib.uslam_server_submit(s.h, sid, capi.ptr(p), PITCH, 0, C.byref(t)), "submit")
                tickets.append(t.value)
            for t in tickets:
                s.wait(t)
            r0, r1 = s.result(tickets[0]), s.result(tickets[1])
            _same(r0, e0)
            _same(r1, e1)
            assert r0[3] is None and np.array_equal(_mm(r1[3]), em)
            for t in tickets:
                s.release(t)
        finally:
            s.close()
