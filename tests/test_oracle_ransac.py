"""The oracle's RANSAC scoring (Sampson distance of ransac_cpu.cpp:173-203 in
double, fixed evaluation order) against a numpy statement of the same
formula, on a synthetic two-view geometry (true F: every exact
correspondence is an inlier) with planted outliers and random matrices."""
import numpy as np

import oracle


def two_view(rs, n=400, outliers=100):
    K = np.array([[460.0, 0, 376.0], [0, 460.0, 240.0], [0, 0, 1.0]])
    X = np.c_[rs.uniform(-2, 2, n), rs.uniform(-1.5, 1.5, n), rs.uniform(4, 9, n)]
    ang = 0.05
    R = np.array([[np.cos(ang), 0, np.sin(ang)], [0, 1, 0], [-np.sin(ang), 0, np.cos(ang)]])
    t = np.array([0.3, 0.02, 0.05])
    x1 = (K @ X.T).T
    x2 = (K @ (R @ X.T + t[:, None])).T
    p = x1[:, :2] / x1[:, 2:]
    q = x2[:, :2] / x2[:, 2:]
    q[:outliers] += rs.uniform(-40, 40, (outliers, 2))
    tx = np.array([[0, -t[2], t[1]], [t[2], 0, -t[0]], [-t[1], t[0], 0]])
    Kinv = np.linalg.inv(K)
    F = Kinv.T @ tx @ R @ Kinv  # q^T F p = 0
    return F / np.linalg.norm(F), p, q


def numpy_counts(Fs, p, q, thr):
    out = []
    for F in Fs.reshape(-1, 3, 3):
        xp, yp, xc, yc = p[:, 0], p[:, 1], q[:, 0], q[:, 1]
        fx0 = (F[0, 0] * xp + F[0, 1] * yp) + F[0, 2]
        fx1 = (F[1, 0] * xp + F[1, 1] * yp) + F[1, 2]
        fx2 = (F[2, 0] * xp + F[2, 1] * yp) + F[2, 2]
        ft0 = (F[0, 0] * xc + F[1, 0] * yc) + F[2, 0]
        ft1 = (F[0, 1] * xc + F[1, 1] * yc) + F[2, 1]
        num = (xc * fx0 + yc * fx1) + fx2
        den = ((fx0 * fx0 + fx1 * fx1) + ft0 * ft0) + ft1 * ft1
        with np.errstate(divide="ignore", invalid="ignore"):
            d = np.where(den < 1e-12, np.inf, (num * num) / den)
        out.append(d < thr)
    return np.array(out)


def test_sampson_counts_match_numpy_and_geometry():
    rs = np.random.RandomState(3)
    F, p, q = two_view(rs)
    Fs = np.concatenate([F[None], rs.normal(size=(50, 3, 3)), np.zeros((1, 3, 3))])
    counts, masks = oracle.sampson_counts(Fs, p, q, 3.84)
    exp = numpy_counts(Fs, p, q, 3.84)
    assert np.array_equal(counts, exp.sum(1))
    bits = np.unpackbits(masks.view(np.uint8), axis=1, bitorder="little")[:, :len(p)].astype(bool)
    assert np.array_equal(bits, exp)
    # the true F keeps the 300 exact correspondences; the zero matrix keeps none
    assert exp[0, 100:].all() and counts[0] < 400 and counts[-1] == 0
