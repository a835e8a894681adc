"""Planted feature sets for the matcher's window edge (shared by the oracle
pin and the GPU test).

At 752x480 the window half-width is 0.1f * 752 = 75.2f.  A previous feature
at level 0, x = 58 (LOD-0 x 58) and a current feature at level 1, x = 111
(LOD-0 x fl(111 * 1.2f) = 133.2) are 75.2 apart: the current one lies inside
the window of the previous one (133.2 <= fl(58 + 75.2f)), while the previous
one lies outside the window of the current one (58 < fl(133.2 - 75.2f)).
match_features_cpu.cpp:106-115 tests the window of each query in f32, so the
two directions of FindMatches see different candidates here."""
import numpy as np

import oracle

W, H, L = 752, 480, 6


def window_edge_sets(case: int, seed: int = 5):
    """(prev features, prev kept, curr features, curr kept) for
    case 0: the edge pair (prev level 0 x 58, curr level 1 x 111), the curr
            feature in the prev feature's window only;
    case 1: the same positions with the frames' roles swapped, the prev
            feature in the curr feature's window only.
    Both features of the edge pair carry the same descriptor; a far feature
    in each set keeps every pool at two or more."""
    rs = np.random.RandomState(seed)
    D = rs.randint(0, 2**32, size=8, dtype=np.uint64).astype(np.uint32)
    far = rs.randint(0, 2**32, size=(2, 8), dtype=np.uint64).astype(np.uint32)

    def set_of(edge_level, edge_x, edge_y, far_desc):
        f = np.zeros(2, oracle.FEATURE_DTYPE)
        # level 0 first (kept order), then level 1
        lv = [edge_level, 0]
        recs = [(edge_x, edge_y, D), (600, 400, far_desc)]
        order = sorted(range(2), key=lambda i: lv[i])
        kept = np.zeros(L, np.int32)
        for k, i in enumerate(order):
            f[k]["x"], f[k]["y"], f[k]["strength"] = recs[i][0], recs[i][1], 12
            f[k]["descriptor"] = recs[i][2]
            kept[lv[i]] += 1
        return f, kept

    e0 = (0, 58, 100)  # level 0, LOD-0 (58, 100)
    e1 = (1, 111, 83)  # level 1, LOD-0 (133.2, 99.6)
    a = set_of(*(e0 if case == 0 else e1), far[0])
    b = set_of(*(e1 if case == 0 else e0), far[1])
    return a[0], a[1], b[0], b[1]
