"""GB300-native feature front-end of uni_slam (pyramid, FAST-style detect,
cull, rotated BRIEF, windowed mutual Hamming matching) behind a C ABI.

The compute path is ``libuslam.so`` (hand-written sm_103a kernels); these
Python modules are thin ctypes handles used by tests and the benchmark.
"""
from .frontend import Batch, Context, FeatureSet, Frontend, Server, level_dims  # noqa: F401
from .capi import FEATURE_DTYPE, MATCH_DTYPE, USlamError  # noqa: F401
