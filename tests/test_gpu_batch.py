"""Batched Lloyd (km_batch_*): every restart of every problem, run in one
persistent launch, must equal the oracle's single run of that instance
(labels, centroids bitwise, returned iteration) — the reference CPU algorithm
with sample picks seeded seed + problem*restarts + restart."""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


def make_problems(rng, count, nmax=6000):
    shapes, Xs = [], []
    for p in range(count):
        n = int(np.exp(rng.uniform(np.log(300), np.log(nmax))))
        d = int(rng.choice([2, 8, 16, 32, 64, 128, 256]))
        k = int(rng.integers(2, 129))
        k = min(k, n - 1)
        X, _ = helpers.synth_blobs_np(n, d, k, -5, 5, 1.0, 100 + p)
        shapes.append((n, d, k))
        Xs.append(X)
    return shapes, Xs


def test_batch_matches_oracle_per_instance(km, gpu):
    rng = np.random.default_rng(2)
    shapes, Xs = make_problems(rng, 12)
    R, seed, tol, maxiter = 3, 7, 1e-4, 60
    b = km.Batch(shapes, restarts=R, seed=seed, tol=tol, maxiter=maxiter).set_data(Xs)
    best, results, ms = b.fit()
    for p, ((n, d, k), X) in enumerate(zip(shapes, Xs)):
        objs = []
        for r in range(R):
            it_o, lab_o, cen_o, ex_o = helpers.orc_lloyd(X, k, tol, seed + p * R + r, maxiter)
            lab, cen = b.instance(p, r)
            np.testing.assert_array_equal(lab, lab_o, err_msg=f"problem {p} restart {r} {shapes[p]}")
            np.testing.assert_array_equal(cen.view(np.uint32), cen_o.view(np.uint32))
            conv, iters, obj = results[p][r]
            assert conv == it_o and iters == ex_o
            objs.append(obj)
        rb = int(np.argmin(objs))
        np.testing.assert_array_equal(best[p][0], b.instance(p, rb)[0])
    b.close()


def test_batch_tune_and_variants_agree(km, gpu):
    rng = np.random.default_rng(9)
    shapes, Xs = make_problems(rng, 6, nmax=3000)
    b = km.Batch(shapes, restarts=2, seed=1, maxiter=20).set_data(Xs)
    v, ms = b.tune()
    assert 0 <= v < 6 and all(m > 0 for m in ms)
    best, _, _ = b.fit()
    for p, ((n, d, k), X) in enumerate(zip(shapes, Xs)):
        _, lab_o, _, _ = helpers.orc_lloyd(X, k, 1e-4, 1 + p * 2 + 0, 20)
        np.testing.assert_array_equal(b.instance(p, 0)[0], lab_o)
    b.close()


def test_batch_rejects_bad_shapes(km, gpu):
    with pytest.raises(km.KmError):
        km.Batch([(10, 4, 11)])               # k > n
    with pytest.raises(km.KmError) as e:
        km.Batch([(5000, 512, 128)])          # centroids beyond the shared-memory limit
    assert e.value.status == km.KM_ERR_UNSUPPORTED


def test_batch_full_workload_matches_oracle(km, gpu):
    """The full batched workload (512 problems, n up to 65,536, d up to 256,
    k up to 128, 8 restarts each, all 4096 instances in one launch): the eight
    largest problems (n*d*k) in all restarts and 24 others in two restarts
    each equal the oracle's single runs bit for bit (labels, centroids,
    returned iteration)."""
    shapes = helpers.batch_problems(512)
    Xs = helpers.batch_points(shapes)
    R, tol, maxiter = 8, 1e-4, 300
    b = km.Batch(shapes, restarts=R, seed=0, tol=tol, maxiter=maxiter).set_data(Xs)
    best, results, ms = b.fit()
    work = np.array([n * d * k for n, d, k in shapes])
    big = [int(p) for p in np.argsort(work)[::-1][:8]]
    rng = np.random.default_rng(5)
    rest = [int(p) for p in rng.permutation(512) if int(p) not in big][:24]
    checks = [(p, r) for p in big for r in range(R)] + [(p, r) for p in rest for r in (0, R - 1)]
    for p, r in checks:
        n, d, k = shapes[p]
        it_o, lab_o, cen_o, ex_o = helpers.orc_lloyd(Xs[p], k, tol, p * R + r, maxiter, threads=16)
        lab, cen = b.instance(p, r)
        np.testing.assert_array_equal(lab, lab_o, err_msg=f"problem {p} restart {r} {shapes[p]}")
        np.testing.assert_array_equal(cen.view(np.uint32), cen_o.view(np.uint32))
        conv, iters, _ = results[p][r]
        assert conv == it_o and iters == ex_o
    b.close()
