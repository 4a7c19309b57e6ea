"""The oracle is pinned before it is trusted: against the golden fixtures made by
the reference's own CPU k-means, against the reference itself where its tree
is present, against its known answers on its shipped datasets, and (kernel
k-means) against an independent numpy statement of the same math."""
import json
from pathlib import Path

import numpy as np
import pytest

import helpers

GOLD = Path(__file__).resolve().parent / "golden"
CASES = json.loads((GOLD / "lloyd_cases.json").read_text())
LABELS = np.load(GOLD / "lloyd_labels.npz")


def case_data(c):
    X, _ = helpers.synth_blobs_np(c["n"], c["d"], c["blobs"], c["lo"], c["hi"], c["sigma"],
                                  c["data_seed"], round_clip=c["round_clip"])
    return X


@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_golden(c):
    from golden.make_golden import x_hash
    X = case_data(c)
    assert x_hash(X) == c["x_sha256"], "generator drift: golden input no longer reproduced"
    it, lab, cen, ex = helpers.orc_lloyd(X, c["k"], c["tol"], c["seed"], c["maxiter"])
    assert it == c["ref_iter"]
    np.testing.assert_array_equal(lab, LABELS[c["name"]].astype(np.uint32))
    assert np.bincount(lab, minlength=c["k"]).tolist() == c["counts"]


def test_oracle_single_thread_equals_threaded():
    c = CASES[3]
    X = case_data(c)
    a = helpers.orc_lloyd(X, c["k"], c["tol"], c["seed"], c["maxiter"], threads=1)
    b = helpers.orc_lloyd(X, c["k"], c["tol"], c["seed"], c["maxiter"], threads=8)
    assert a[0] == b[0]
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(a[2].view(np.uint32), b[2].view(np.uint32))


needs_ref = pytest.mark.skipif(helpers.reference_lib() is None, reason="reference tree not present")


@needs_ref
@pytest.mark.parametrize("seed", [0, 1, 5])
@pytest.mark.parametrize("shape", [(3000, 5, 9), (2500, 33, 17), (700, 64, 70), (4000, 2, 3)])
def test_oracle_matches_reference_live(shape, seed):
    n, d, k = shape
    rng = np.random.default_rng(seed + 100 * d)
    X = (rng.standard_normal((n, d)) * 3 + rng.integers(0, 4, (n, 1))).astype(np.float32)
    it_r, lab_r = helpers.ref_lloyd(X, k, 1e-4, seed, 200)
    it_o, lab_o, _, _ = helpers.orc_lloyd(X, k, 1e-4, seed, 200)
    assert it_o == it_r
    np.testing.assert_array_equal(lab_o, lab_r)


@needs_ref
def test_oracle_value_duplicate_rejection_matches_reference():
    # many duplicate rows: the sample init must skip picks equal by value
    rng = np.random.default_rng(3)
    base = rng.integers(0, 3, (12, 4)).astype(np.float32)
    X = base[rng.integers(0, 12, 2000)]
    X[::7] *= -1.0  # -0.0 entries compare equal to +0.0
    k = int(len(np.unique(X, axis=0)))
    it_r, lab_r = helpers.ref_lloyd(X, k, 0.0, 9, 50)
    it_o, lab_o, _, _ = helpers.orc_lloyd(X, k, 0.0, 9, 50)
    assert it_o == it_r
    np.testing.assert_array_equal(lab_o, lab_r)


@needs_ref
@pytest.mark.parametrize("path,d,k,m,t,seed,iters,sizes", [
    ("datasets/N1797_D64_digits-sklearn.csv", 64, 10, 300, 1e-4, 0, 21, None),
    ("datasets/N1797_D64_digits-sklearn.csv", 64, 10, 300, 1e-4, 1, 14, None),
    ("datasets/N100K_D2.csv", 2, 4, 500, 1e-5, 0, 32, [27851, 19959, 32193, 19997]),
])
def test_oracle_known_answers_on_reference_datasets(path, d, k, m, t, seed, iters, sizes):
    X = helpers.read_reference_csv(helpers.REFERENCE / path, d)
    it_o, lab_o, _, _ = helpers.orc_lloyd(X, k, t, seed, m)
    it_r, lab_r = helpers.ref_lloyd(X, k, t, seed, m)
    assert it_o == it_r == iters
    np.testing.assert_array_equal(lab_o, lab_r)
    if sizes:
        assert np.bincount(lab_o, minlength=k).tolist() == sizes


def test_fp64_oracle_agrees_on_separated_blobs():
    X, _ = helpers.synth_blobs_np(4000, 16, 8, -20, 20, 0.5, 21)
    it32, lab32, _, _ = helpers.orc_lloyd(X, 8, 1e-4, 2, 100)
    it64, lab64, _, _ = helpers.orc_lloyd64(X, 8, 1e-4, 2, 100)
    assert (lab32 == lab64).mean() == 1.0


def test_update_oracle_semantics():
    # empty cluster -> zero vector; scale is float(1/(double)count)
    X = np.array([[1, 2], [3, 4], [5, 7]], np.float32)
    lab = np.array([0, 0, 2], np.uint32)
    Cc, cnt = helpers.orc_update(X, lab, 3)
    assert cnt.tolist() == [2, 0, 1]
    np.testing.assert_array_equal(Cc, np.array([[2, 3], [0, 0], [5, 7]], np.float32))


# ---- kernel k-means oracle vs an independent numpy statement -------------
# experiments/knKmeans.m:13-29 computes T = E K with a one-hot E (k x n),
# distances -2 T[c,i]/|c| + (1/|c|^2) sum_{a,b in c} K_ab; the reference GPU
# path (distances.cu:895-1002) is the same with ctilde == 0 -> +inf.

def numpy_kernel_kmeans(K, k, maxiter, tol, check):
    n = K.shape[0]
    lab = np.arange(n) % k
    last = None
    it = 0
    conv = maxiter
    score = 0.0
    while it < maxiter:
        it += 1
        V = np.zeros((k, n))
        V[lab, np.arange(n)] = 1.0
        cnt = V.sum(1)
        E = K @ V.T                                # n x k, E[i,c] = sum_{j in c} K_ij
        ct = np.where(cnt > 0, np.einsum("ic,ci->c", E, V) / np.maximum(cnt, 1) ** 2, 0.0)
        Dm = np.where(cnt > 0, -2.0 * E / np.maximum(cnt, 1), 0.0) + np.where(ct == 0, np.inf, ct)
        Dm = np.where(np.isfinite(Dm), Dm, np.inf)
        newlab = np.argmin(np.where(Dm < np.float32(np.finfo(np.float32).max), Dm, np.inf), axis=1)
        allinf = ~np.isfinite(Dm).any(1)
        newlab[allinf] = 0
        score = Dm[np.arange(n), newlab].sum()
        lab = newlab
        if it == maxiter:
            break
        if check and it > 1 and abs(score - last) < tol:
            conv = it
            break
        last = score
    return conv, lab, score


@pytest.mark.parametrize("kind,params", [(0, (1, 0, 1, 1)), (1, (1 / 8, 1, 2, 1)), (3, (1, 0, 1, 0.9)),
                                         (2, (0.05, 1, 1, 1))])
def test_kernel_kmeans_oracle_vs_numpy(kind, params):
    gamma, coef, degree, sigma = params
    X, _ = helpers.synth_blobs_np(300, 8, 4, -1, 1, 0.3, 5)
    n, d = X.shape
    K = np.empty((n, n))
    helpers.oracle().orc_kernel_matrix(X.ctypes.data, n, d, kind, gamma, coef, degree, sigma, 4, K.ctypes.data)
    Xd = X.astype(np.float64)
    G = Xd @ Xd.T
    sq = (Xd ** 2).sum(1)
    Kref = {0: G, 1: (gamma * G + coef) ** degree, 2: np.tanh(gamma * G + coef),
            3: np.exp(-np.maximum(sq[:, None] + sq[None] - 2 * G, 0) / (2 * sigma ** 2))}[kind]
    np.testing.assert_allclose(K, Kref, rtol=1e-12, atol=1e-12)
    lab = (np.arange(n) % 4).astype(np.uint32)
    import ctypes as C
    sc = C.c_double(0)
    ex = C.c_uint64(0)
    it = helpers.oracle().orc_kernel_kmeans(K.ctypes.data, n, 4, 30, 1e-9, 1, 4, lab.ctypes.data,
                                            C.byref(sc), C.byref(ex))
    it_np, lab_np, sc_np = numpy_kernel_kmeans(K, 4, 30, 1e-9, True)
    assert it == it_np
    np.testing.assert_array_equal(lab, lab_np)
    assert abs(sc.value - sc_np) <= 1e-9 * max(1.0, abs(sc_np))


@pytest.mark.parametrize("kind,params", [(1, (1 / 16, 1, 2, 1)), (3, (1, 0, 1, 0.7)), (0, (1, 0, 1, 1))])
def test_kkm_step_blocked_matches_oracle_iteration(kind, params):
    """oracle/kkm_step.py (K formed block by block, for n too large for an n x n
    FP64 matrix) gives the labels and score of one iteration of the oracle's
    orc_kernel_kmeans from the same labels, including an emptied cluster."""
    import ctypes as C
    import importlib.util
    spec = importlib.util.spec_from_file_location("kkm_step", helpers.ORACLE / "kkm_step.py")
    ks = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ks)
    gamma, coef, degree, sigma = params
    X, _ = helpers.synth_blobs_np(700, 16, 6, -1, 1, 0.3, 8)
    n, d = X.shape
    k = 7
    K = np.empty((n, n))
    helpers.oracle().orc_kernel_matrix(X.ctypes.data, n, d, kind, gamma, coef, degree, sigma, 4, K.ctypes.data)
    lab0 = np.random.default_rng(3).integers(0, k - 1, n).astype(np.uint32)     # cluster k-1 empty
    lab = lab0.copy()
    sc = C.c_double(0)
    ex = C.c_uint64(0)
    helpers.oracle().orc_kernel_kmeans(K.ctypes.data, n, k, 1, 0.0, 0, 4, lab.ctypes.data, C.byref(sc), C.byref(ex))
    new, score = ks.kkm_step_f64(X, lab0, k, kind, gamma, coef, degree, sigma, block=128, workers=3)
    np.testing.assert_array_equal(new, lab)
    assert abs(score - sc.value) <= 1e-9 * max(1.0, abs(sc.value))
    diag = ks.kernel_diag(X, kind, gamma, coef, degree, sigma)
    np.testing.assert_allclose(diag, np.diagonal(K), rtol=1e-12, atol=1e-12)


def test_plusplus_oracle_properties():
    """The oracle's seeded k-means++: deterministic per seed, k distinct rows on
    separated blobs, one pick per blob (D^2 sampling), and a cost well below
    uniform sample picks."""
    X, blob = helpers.synth_blobs_np(8000, 6, 24, -100, 100, 0.5, 3)
    a = helpers.orc_plusplus(X, 24, 9)
    b = helpers.orc_plusplus(X, 24, 9)
    c = helpers.orc_plusplus(X, 24, 10)
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
    assert len(set(a.tolist())) == 24
    assert len({int(blob[i]) for i in a}) >= 22
    d2 = lambda C: float(((X[:, None, :].astype(np.float64) - C[None].astype(np.float64)) ** 2).sum(2).min(1).sum())
    rc, sp = helpers.orc_sample_picks(X, 24, 9)
    assert d2(X[a]) < 0.5 * d2(X[sp])
