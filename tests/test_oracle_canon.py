"""Accuracy of the canonical binary32 atan2 / sin / cos shared by the kernels
and the oracle (include/uslam_canon.h): a few ULP of the correctly rounded
value (WGSL itself allows 4096 ULP for atan2)."""
import math

import numpy as np

import oracle


def _ulps(got: float, ref: float) -> int:
    a = np.array([got], np.float32).view(np.int32)[0]
    b = np.array([ref], np.float32).view(np.int32)[0]
    if (a < 0) != (b < 0):
        return int(abs(int(a)) + abs(int(b)))
    return int(abs(int(a) - int(b)))


def test_atan2_accuracy():
    rs = np.random.RandomState(0)
    worst = 0
    for _ in range(20000):
        y, x = np.float32(rs.uniform(-50, 50)), np.float32(rs.uniform(-50, 50))
        worst = max(worst, _ulps(oracle.atan2f(float(y), float(x)), math.atan2(float(y), float(x))))
    assert worst <= 4


def test_atan2_special_values():
    assert oracle.atan2f(0.0, 0.0) == 0.0
    assert oracle.atan2f(0.0, -0.0) == np.float32(math.pi)
    assert oracle.atan2f(1.0, 0.0) == np.float32(math.pi / 2)
    assert oracle.atan2f(-1.0, 0.0) == -np.float32(math.pi / 2)
    assert oracle.atan2f(0.0, -1.0) == np.float32(math.pi)
    assert oracle.atan2f(-0.0, -1.0) == -np.float32(math.pi)


def test_sincos_accuracy():
    rs = np.random.RandomState(1)
    worst = 0
    for _ in range(20000):
        a = float(np.float32(rs.uniform(-math.pi, math.pi)))
        s, c = oracle.sincosf(a)
        worst = max(worst, _ulps(s, math.sin(a)), _ulps(c, math.cos(a)))
    assert worst <= 2
