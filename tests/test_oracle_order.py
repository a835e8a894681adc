"""The matcher's result does not depend on the order of the features within
a level (match_features_cpu.cpp:66-150 sorts each pool by x and resolves a
tied best through the ratio test, which then rejects): the oracle, given both
sets with every level permuted, returns the same matched feature pairs."""
import numpy as np
import pytest

import oracle
from test_oracle_pins import _random_sets


def _pairs(fa, ka, fb, kb, m):
    oa = np.concatenate([[0], np.cumsum(ka)])
    ob = np.concatenate([[0], np.cumsum(kb)])
    out = set()
    for la, ia, lb, ib in m:
        a, b = fa[oa[la] + ia], fb[ob[lb] + ib]
        out.add((int(la), float(a["x"]), float(a["y"]), int(lb), float(b["x"]), float(b["y"])))
    return out


def _permute(rs, f, k):
    off = np.concatenate([[0], np.cumsum(k)])
    idx = np.concatenate([off[l] + rs.permutation(int(k[l])) for l in range(len(k))]).astype(np.int64)
    return f[idx]


@pytest.mark.parametrize("flip_p", [0.0, 0.05, 0.2])
def test_match_independent_of_feature_order(flip_p):
    rs = np.random.RandomState(int(flip_p * 100) + 3)
    W, H = 752, 480
    ref = oracle.ref_matcher(W, H)  # None without a copy of the reference matcher source
    assert ref is not None or not oracle.ref_matcher_expected()
    for trial in range(4):
        fa, ka, fb, kb = _random_sets(rs, W, H, per_level=150, flip_p=flip_p)
        base = _pairs(fa, ka, fb, kb, oracle.match(fa, ka, fb, kb, W, H))
        pa, pb = _permute(rs, fa, ka), _permute(rs, fb, kb)
        perm = _pairs(pa, ka, pb, kb, oracle.match(pa, ka, pb, kb, W, H))
        assert perm == base, f"trial {trial}"
        if ref is not None:  # the compiled reference on the permuted sets agrees
            assert _pairs(pa, ka, pb, kb, ref(pa, ka, pb, kb)) == base, f"trial {trial} (reference)"
        if flip_p == 0.0:
            assert len(base) > 0
