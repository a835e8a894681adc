"""The arithmetic the tensor-core brute-force matcher (k_bf_mma, matcher 2)
relies on, checked on the CPU: the FP8 E4M3 codes of its operand values,
the accumulator value
    key = 64 dot + sum(ext_a * ext_b) = 32 (2 dot - popc(b) + 257) + s
staying an exact integer in [32, 16447] (so every partial sum is exact in
f32 whatever the order), the 16-bit key surviving "+ 2^23" in f32, and the
distance recovered from a key equal to popcount(a XOR b)."""
import numpy as np


def e4m3(code: int) -> float:
    """Value of an FP8 E4M3 (fn) code: 1 sign, 4 exponent (bias 7), 3 mantissa bits."""
    sign = -1.0 if code & 0x80 else 1.0
    e, m = (code >> 3) & 0xF, code & 7
    assert not (e == 15 and m == 7), "NaN"
    return sign * (2.0 ** (e - 7) * (1 + m / 8) if e else 2.0 ** -6 * (m / 8))


def small_int_code(v: int) -> int:
    """The device's e4m3_small_int: the code of an integer 0..16."""
    if v <= 0:
        return 0
    k = v.bit_length() - 1
    return ((k + 7) << 3) | (((v - (1 << k)) << 3) >> k)


# query-side extension (constant) and the train-side extension of a row with
# popcount pc and index s within its 32-row group (k_describe's PACK branch)
EXT_A = [0xE0] * 16 + [0x60, 0x38, 0x38, 0x60] + [0] * 12


def ext_b(pc: int, s: int):
    return ([small_int_code(min(16, max(0, pc - 16 * e))) for e in range(16)] +
            [0x78, small_int_code(min(s, 16)), small_int_code(max(s - 16, 0)), 0x38] + [0] * 12)


def test_codes():
    assert [e4m3(small_int_code(v)) for v in range(17)] == [float(v) for v in range(17)]
    assert (e4m3(0x50), e4m3(0x38), e4m3(0xE0), e4m3(0x60), e4m3(0x78)) == (8.0, 1.0, -32.0, 32.0, 256.0)


def test_extension_sum_and_key_range():
    va = np.array([e4m3(c) for c in EXT_A])
    for pc in range(257):
        for s in range(32):
            ext = float(np.dot(va, [e4m3(c) for c in ext_b(pc, s)]))
            assert ext == -32 * pc + 32 * 257 + s
    # extremes of 2 dot - popc(b): dot = 0 with popc(b) = 256, and dot = popc(b) = 256
    lo = 64 * 0 - 32 * 256 + 32 * 257 + 0
    hi = 64 * 256 - 32 * 256 + 32 * 257 + 31
    assert (lo, hi) == (32, 16447) and hi < 1 << 16


def _bits(words):
    return np.unpackbits(words.view(np.uint8), bitorder="little").astype(np.float32)


def test_key_to_distance_and_partial_sums_exact():
    rs = np.random.RandomState(1)
    a = rs.randint(0, 2**32, size=(512, 8), dtype=np.uint64).astype(np.uint32)
    b = rs.randint(0, 2**32, size=(512, 8), dtype=np.uint64).astype(np.uint32)
    b[:8] = a[:8]            # distance 0
    b[8:16] = ~a[8:16]       # distance 256
    a[16] = 0xFFFFFFFF
    b[16] = 0xFFFFFFFF       # dot = popc(b) = 256: the largest key
    a[17] = 0
    b[17] = 0xFFFFFFFF       # dot = 0, popc(b) = 256: the smallest key
    va = np.array([e4m3(c) for c in EXT_A], np.float32)
    for i in range(len(a)):
        s = i % 32
        pa, pb = _bits(a[i]) * 8.0, _bits(b[i]) * 8.0  # bits as 8.0 on both sides
        pc = int(_bits(b[i]).sum())
        terms = np.concatenate([pa * pb, va * np.array([e4m3(c) for c in ext_b(pc, s)], np.float32)])
        # summed in f32 in two different orders: integers below 2^24, so both exact
        fwd = np.float32(0)
        for t in terms:
            fwd = np.float32(fwd + t)
        rev = np.float32(0)
        for t in terms[::-1]:
            rev = np.float32(rev + t)
        key = int(fwd)
        assert fwd == rev and float(fwd) == key and 32 <= key <= 16447
        # the key in the low 16 bits of (value + 2^23) as f32 bits
        bits = np.array([np.float32(fwd) + np.float32(2**23)], np.float32).view(np.uint32)[0]
        assert bits & 0xFFFF == key and key & 31 == s
        popc_a = int(_bits(a[i]).sum())
        dist = popc_a + 257 - (key >> 5)
        assert dist == int(sum(bin(int(x)).count("1") for x in (a[i] ^ b[i])))
