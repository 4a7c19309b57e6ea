"""Greedy k-means++ initialisation (KM_INIT_PLUSPLUS; the reference's
init_centroids_plus_plus, src/kmeans.cu:447-769).  The reference draws from
std::random_device, so no sequence of its own can be matched; the device's
seeded draws are restated in the oracle (orc_plusplus: the same RNG stream,
s = 2 + ceil(ln k) candidates, FP64 prefix sums, the lowest total cost) and
the picked rows must be identical.  Beside that, the properties the algorithm
guarantees: seeded determinism, centroids that are distinct data points, D^2
sampling that covers well-separated blobs, a lower starting cost than sample
picks."""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


def pp_centroids(km, X, k, seed):
    n, d = X.shape
    m = km.Lloyd(n, d, k, seed=seed, init="plusplus", maxiter=1).set_data(X)
    C = m.init_centroids()
    m.close()
    return C


def cost(X, C):
    X = X.astype(np.float64)
    C = C.astype(np.float64)
    d2 = (X * X).sum(1)[:, None] - 2 * X @ C.T + (C * C).sum(1)[None]
    return float(np.maximum(d2, 0).min(1).sum())


def test_plusplus_deterministic_and_distinct_points(km, gpu):
    X, _ = helpers.synth_blobs_np(20000, 16, 40, -10, 10, 1.0, 4)
    C1 = pp_centroids(km, X, 40, 7)
    C2 = pp_centroids(km, X, 40, 7)
    C3 = pp_centroids(km, X, 40, 8)
    np.testing.assert_array_equal(C1, C2)
    assert not np.array_equal(C1, C3)
    rows = {r.tobytes() for r in X}
    assert all(c.tobytes() in rows for c in C1)
    assert len({c.tobytes() for c in C1}) == 40


def test_plusplus_covers_separated_blobs(km, gpu):
    X, blob = helpers.synth_blobs_np(50000, 8, 64, -100, 100, 0.5, 6)
    C = pp_centroids(km, X, 64, 1)
    index = {r.tobytes(): i for i, r in enumerate(X)}
    hit = {int(blob[index[c.tobytes()]]) for c in C}
    assert len(hit) >= 60, len(hit)       # D^2 sampling: one pick per blob, bar a few
    # much better start than uniform sample picks
    m = km.Lloyd(50000, 8, 64, seed=1, init="sample", maxiter=1).set_data(X)
    Cs = m.init_centroids()
    m.close()
    assert cost(X, C) < 0.5 * cost(X, Cs)


def test_plusplus_with_duplicates_and_k_equal_distinct(km, gpu):
    base = np.arange(12, dtype=np.float32).reshape(6, 2)
    X = np.repeat(base, 50, axis=0)
    C = pp_centroids(km, X, 6, 3)
    assert {c.tobytes() for c in C} == {b.tobytes() for b in base}


def test_plusplus_fit_converges(km, gpu):
    X, _ = helpers.synth_blobs_np(30000, 32, 16, -5, 5, 0.5, 2)
    m = km.Lloyd(30000, 32, 16, seed=5, init="plusplus", maxiter=100, tol=1e-4).set_data(X)
    lab, C, r = m.fit()
    m.close()
    assert r.converged and r.iterations < 100
    assert lab.max() < 16


@pytest.mark.parametrize("n,d,k,seed", [(20000, 16, 40, 7), (7001, 37, 100, 3), (50000, 128, 256, 11),
                                        (3000, 3, 2, 0), (1000, 64, 1, 5)])
def test_plusplus_picks_match_oracle(km, gpu, n, d, k, seed):
    """The centroids are exactly the rows the oracle's restatement picks."""
    X, _ = helpers.synth_blobs_np(n, d, max(2, k // 2), -10, 10, 1.0, 100 + seed)
    C = pp_centroids(km, X, k, seed)
    picks = helpers.orc_plusplus(X, k, seed)
    np.testing.assert_array_equal(C.view(np.uint32), X[picks].view(np.uint32))

