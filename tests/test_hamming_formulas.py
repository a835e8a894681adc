"""The integer identity the CUDA matchers rely on, checked with numpy on
random words and the extreme distances: the carry-save-adder popcount of a
256-bit XOR (4 popcounts instead of 8)."""
import numpy as np


def _popc(v):
    v = v.astype(np.uint64)
    return np.array([bin(int(x)).count("1") for x in v], np.uint64)


def test_csa_popcount_equals_plain_popcount():
    rs = np.random.RandomState(0)
    a = rs.randint(0, 2**32, size=(4096, 8), dtype=np.uint64).astype(np.uint32)
    b = rs.randint(0, 2**32, size=(4096, 8), dtype=np.uint64).astype(np.uint32)
    b[:64] = a[:64]                  # distance 0
    b[64:128] = ~a[64:128]           # distance 256
    x = a ^ b
    x0, x1, x2, x3, x4, x5, x6, x7 = (x[:, i] for i in range(8))
    o1, t1 = x0 ^ x1 ^ x2, (x0 & x1) | (x2 & (x0 ^ x1))
    o2, t2 = o1 ^ x3 ^ x4, (o1 & x3) | (x4 & (o1 ^ x3))
    o3, t3 = o2 ^ x5 ^ x6, (o2 & x5) | (x6 & (o2 ^ x5))
    tw, f = t1 ^ t2 ^ t3, (t1 & t2) | (t3 & (t1 ^ t2))
    csa = _popc(o3) + _popc(x7) + 2 * _popc(tw) + 4 * _popc(f)
    plain = sum(_popc(x[:, i]) for i in range(8))
    assert np.array_equal(csa, plain)
    assert plain[:64].max() == 0 and plain[64:128].min() == 256
