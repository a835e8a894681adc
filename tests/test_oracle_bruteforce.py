"""The oracle's brute-force top-2 matcher against a plain numpy statement of
the same rule (every query against every train descriptor, best/second-best
Hamming distance, f32 ratio test, no window, no cross-check), plus its edge
cases: ties, a train set of fewer than two features, empty sets."""
import numpy as np

import oracle


def _feats(desc):
    f = np.zeros(len(desc), oracle.FEATURE_DTYPE)
    f["descriptor"] = desc
    return f


def _numpy_top2(da, db, ratio):
    bits = np.unpackbits(da.view(np.uint8), axis=1).astype(np.int32)
    bbits = np.unpackbits(db.view(np.uint8), axis=1).astype(np.int32)
    d = (bits[:, None, :] != bbits[None, :, :]).sum(2)
    out = np.full(len(da), -1, np.int32)
    if len(db) < 2:
        return out
    for i in range(len(da)):
        order = np.argsort(d[i], kind="stable")
        best, second = d[i, order[0]], d[i, order[1]]
        if np.float32(best) < np.float32(ratio) * np.float32(second):
            out[i] = order[0]
    return out


def _flat(m, kept_a, kept_b):
    a_off = np.concatenate([[0], np.cumsum(kept_a)])
    b_off = np.concatenate([[0], np.cumsum(kept_b)])
    return {int(a_off[la] + ia): int(b_off[lb] + ib) for la, ia, lb, ib in m}


def test_matches_numpy_statement():
    rs = np.random.RandomState(7)
    db = rs.randint(0, 2**32, size=(400, 8), dtype=np.uint64).astype(np.uint32)
    da = rs.randint(0, 2**32, size=(300, 8), dtype=np.uint64).astype(np.uint32)
    # plant 150 queries as noisy copies of train descriptors (a few flipped bits)
    for i in range(150):
        da[i] = db[rs.randint(400)]
        for _ in range(rs.randint(0, 40)):
            w, bit = rs.randint(8), rs.randint(32)
            da[i, w] ^= np.uint32(1 << bit)
    kept_a, kept_b = np.array([100, 120, 80]), np.array([250, 0, 150])
    m = oracle.match_bruteforce(_feats(da), kept_a, _feats(db), kept_b, 0.8)
    exp = _numpy_top2(da, db, 0.8)
    got = _flat(m, kept_a, kept_b)
    want = {i: int(j) for i, j in enumerate(exp) if j >= 0}
    assert got == want
    assert 100 < len(want) <= 150
    # rows are in (lod_a, idx_a) order
    assert np.array_equal(m[np.lexsort((m[:, 1], m[:, 0]))], m)


def test_tied_best_fails_and_small_pools():
    rs = np.random.RandomState(3)
    q = rs.randint(0, 2**32, size=(1, 8), dtype=np.uint64).astype(np.uint32)
    twin = np.concatenate([q, q, q ^ np.uint32(0xffffffff)])
    assert len(oracle.match_bruteforce(_feats(q), [1], _feats(twin), [3])) == 0  # best == second
    assert len(oracle.match_bruteforce(_feats(q), [1], _feats(q), [1])) == 0  # one train feature
    assert len(oracle.match_bruteforce(_feats(q), [1], _feats(twin[1:]), [2])) == 1
    empty = np.zeros(0, oracle.FEATURE_DTYPE)
    assert len(oracle.match_bruteforce(empty, [0], _feats(twin), [3])) == 0
    assert len(oracle.match_bruteforce(_feats(q), [1], empty, [0])) == 0


def test_ratio_boundary_is_strict_f32():
    # best 4, second 5: 4 < 0.8 * 5 is false in f32 (0.8f * 5 rounds to 4.0)
    q = np.zeros((1, 8), np.uint32)
    b = np.zeros((2, 8), np.uint32)
    b[0, 0] = 0xF
    b[1, 0] = 0x1F
    assert np.float32(0.8) * np.float32(5) == np.float32(4.0)
    assert len(oracle.match_bruteforce(_feats(q), [1], _feats(b), [2], 0.8)) == 0
    assert len(oracle.match_bruteforce(_feats(q), [1], _feats(b), [2], 0.81)) == 1
