"""GPU parity of kernel k-means (the reference's popcorn GPU path) through the C
ABI: the kernel matrix K = f(X X^T) against an FP64 torch reference, and the
iteration against the FP64 oracle (orc_kernel_kmeans, itself checked against
an independent numpy statement in test_oracle.py)."""
import ctypes as C

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu

KERNELS = [("linear", dict()), ("polynomial", dict(gamma=1 / 16, coef=1.0, degree=2)),
           ("sigmoid", dict(gamma=0.01, coef=1.0)), ("gaussian", dict(sigma=3.0))]
# relative tolerance of K against FP64, as a fraction of the scale max|K| (or of
# |gamma| ||x|| ||y|| for the argument of f)
TOL = {"fp32": 2e-5, "bf16x3": 2e-4, "bf16": 3e-2}


def ref_kernel(X, kind, p):
    Xd = X.double()
    G = Xd @ Xd.T
    sq = (Xd * Xd).sum(1)
    if kind == "linear":
        return G
    if kind == "polynomial":
        return (p["gamma"] * G + p["coef"]) ** p["degree"]
    if kind == "sigmoid":
        return (p["gamma"] * G + p["coef"]).tanh()
    return (-(sq[:, None] + sq[None] - 2 * G).clamp_min(0) / (2 * p["sigma"] ** 2)).exp()


@pytest.mark.parametrize("out_bf16", [False, True])
@pytest.mark.parametrize("prec", ["fp32", "bf16", "bf16x3"])
@pytest.mark.parametrize("kind,params", KERNELS, ids=[k for k, _ in KERNELS])
@pytest.mark.parametrize("shape", [(1000, 37), (2048, 128)])
def test_kernel_matrix_vs_fp64(km, gpu, kind, params, prec, out_bf16, shape):
    import torch
    n, d = shape
    X = torch.from_numpy(helpers.synth_blobs_np(n, d, 5, -1, 1, 0.5, 3)[0]).to(gpu)
    K, dg = km.kernel_matrix(X, kernel=kind, precision=prec, out_bf16=out_bf16, want_diag=True, **params)
    ref = ref_kernel(X, kind, params)
    scale = float(ref.abs().max())
    tol = TOL[prec] + (2 ** -8 if out_bf16 else 0.0)
    err = float((K.double() - ref).abs().max())
    assert err <= tol * scale * 4, (err, scale)
    np.testing.assert_allclose(torch.diagonal(K).double().cpu().numpy(), dg.double().cpu().numpy(),
                               rtol=2 ** -8 if out_bf16 else 0, atol=0)


def oracle_kkm(X, kind, params, k, maxiter, tol, check):
    X = np.ascontiguousarray(X, np.float32)
    n, d = X.shape
    Kd = np.empty((n, n))
    kid = {"linear": 0, "polynomial": 1, "sigmoid": 2, "gaussian": 3}[kind]
    helpers.oracle().orc_kernel_matrix(X.ctypes.data, n, d, kid, params.get("gamma", 1.0), params.get("coef", 1.0),
                                       params.get("degree", 2), params.get("sigma", 1.0), 8, Kd.ctypes.data)
    lab = (np.arange(n) % k).astype(np.uint32)
    sc = C.c_double(0)
    ex = C.c_uint64(0)
    it = helpers.oracle().orc_kernel_kmeans(Kd.ctypes.data, n, k, maxiter, tol, int(check), 8, lab.ctypes.data,
                                            C.byref(sc), C.byref(ex))
    return it, lab, sc.value, ex.value


def test_kkm_linear_integer_data_exact(km, gpu):
    """Integer-valued points and the linear kernel: K, E and the distances are
    exact in every precision, so labels and iteration count equal the oracle's."""
    X, _ = helpers.synth_blobs_np(1500, 16, 7, 0, 8, 2.0, 5, round_clip=True)
    it_o, lab_o, sc_o, ex_o = oracle_kkm(X, "linear", {}, 7, 40, 1e-9, True)
    for prec, pr in (("fp32", 0), ("bf16", 0), ("bf16x3", 0), ("fp32", 512), ("bf16", "fused"),
                     ("bf16x3", "fused")):
        m = km.KernelKMeans(1500, 16, 7, kernel="linear", maxiter=40, tol=1e-9, precision=prec,
                            check_converged=True, panel_rows=pr).set_data(X)
        lab, r = m.fit()
        m.close()
        np.testing.assert_array_equal(lab, lab_o)
        assert r.converged_iter == it_o
        assert abs(r.score - sc_o) <= 1e-6 * max(1.0, abs(sc_o))


@pytest.mark.parametrize("kb16", [False, True])
@pytest.mark.parametrize("prec", ["fp32", "bf16x3", "bf16"])
@pytest.mark.parametrize("kind,params", [("polynomial", dict(gamma=1 / 32, coef=1.0, degree=2)),
                                         ("gaussian", dict(sigma=2.0))])
def test_kkm_vs_fp64_oracle(km, gpu, kind, params, prec, kb16):
    X, _ = helpers.synth_blobs_np(3000, 32, 6, -1, 1, 0.35, 9)
    maxiter = 8
    it_o, lab_o, sc_o, _ = oracle_kkm(X, kind, params, 6, maxiter, 0.0, False)
    m = km.KernelKMeans(3000, 32, 6, kernel=kind, maxiter=maxiter, precision=prec, k_bf16=kb16,
                        **params).set_data(X)
    lab, r = m.fit()
    m.close()
    agree = float((lab == lab_o).mean())
    reduced = prec == "bf16" or kb16
    # K stored in BF16 keeps 8 significant bits of every K_ij; with the
    # Gaussian kernel the cluster margins of E are thin and 8 iterations let a
    # few per cent of the labels drift from the FP64 trajectory.
    floor = 0.999 if not reduced else (0.98 if kind == "gaussian" else 0.99)
    assert agree >= floor, agree
    rel = abs(r.score - sc_o) / abs(sc_o)
    assert rel <= (1e-5 if prec == "fp32" and not kb16 else 1e-3 if not reduced else 2e-2), rel
    assert r.iterations == maxiter


def test_kkm_given_initial_labels_and_bad_labels(km, gpu):
    X, _ = helpers.synth_blobs_np(500, 8, 4, -2, 2, 0.5, 1)
    m = km.KernelKMeans(500, 8, 4, kernel="linear", maxiter=5).set_data(X)
    lab, r = m.fit(init_labels=np.zeros(500, np.uint32) + (np.arange(500) % 2))
    assert lab.max() < 4
    with pytest.raises(km.KmError) as e:
        m.fit(init_labels=np.full(500, 9, np.uint32))
    assert e.value.status == km.KM_ERR_ARG
    m.close()


def _fit(km, X, k, panel_rows, **kw):
    n, d = X.shape
    m = km.KernelKMeans(n, d, k, panel_rows=panel_rows, **kw).set_data(X)
    lab, r = m.fit()
    rows = m.panel_rows()
    m.close()
    return lab, r, rows


@pytest.mark.parametrize("kb16", [False, True])
@pytest.mark.parametrize("prec", ["fp32", "bf16x3", "bf16"])
@pytest.mark.parametrize("kind,params", [("polynomial", dict(gamma=1 / 32, coef=1.0, degree=2)),
                                         ("gaussian", dict(sigma=2.0))])
def test_kkm_panels_equal_resident(km, gpu, kind, params, prec, kb16):
    """K rebuilt every iteration in row panels (ragged last panel, panel rows
    not a multiple of the 128-row tile, one panel of all rows) gives the same
    K values in the same summation order as the resident matrix: labels,
    score and iteration count are identical, including a fit that stops
    early on the score rule with iterations still enqueued."""
    X, _ = helpers.synth_blobs_np(3000, 32, 6, -1, 1, 0.35, 9)
    kw = dict(kernel=kind, maxiter=12, tol=1e-3, precision=prec, k_bf16=kb16, check_converged=True, **params)
    lab0, r0, rows0 = _fit(km, X, 6, 0, **kw)
    assert rows0 == 0
    for pr in (1000, 128, 3000, 5000):
        lab, r, rows = _fit(km, X, 6, pr, **kw)
        assert rows == min(pr, 3000)
        np.testing.assert_array_equal(lab, lab0)
        assert r.score == r0.score and r.iterations == r0.iterations
        assert r.converged_iter == r0.converged_iter
        panels = -(-3000 // rows)
        # per enqueued iteration: 9 kernels resident; 8 + a build and a V.K per panel
        assert r.kernel_launches == r0.kernel_launches // 9 * (8 + 2 * panels)


def test_kkm_k256_global_labels_vs_oracle(km, gpu):
    """k = 256 leaves no room for the n byte labels beside the V.K bins in
    shared memory, so V.K reads them from a global byte copy (refreshed after
    every iteration): against the FP64 oracle, resident and panelled."""
    X, _ = helpers.synth_blobs_np(4096, 16, 256, -4, 4, 0.3, 21)
    params = dict(gamma=1 / 16, coef=1.0, degree=2)
    it_o, lab_o, sc_o, _ = oracle_kkm(X, "polynomial", params, 256, 6, 0.0, False)
    for pr in (0, 1024):
        lab, r, _ = _fit(km, X, 256, pr, kernel="polynomial", maxiter=6, precision="fp32", **params)
        assert float((lab == lab_o).mean()) >= 0.998
        assert abs(r.score - sc_o) <= 1e-4 * abs(sc_o)
        assert r.iterations == 6


def test_kkm_large_n_panels_equal_resident(km, gpu):
    """n = 170,000 points: the byte labels (166 KiB) no longer fit beside the
    bins of k = 64, which the resident path used to reject; BF16 K resident
    (58 GB) and in panels of 8192 rows (2.8 GB) give identical fits."""
    n, d, k = 170000, 32, 64
    X, _ = helpers.synth_blobs_np(n, d, k, -1, 1, 0.3, 33)
    kw = dict(kernel="gaussian", sigma=1.0, maxiter=3, precision="bf16", k_bf16=True)
    lab0, r0, _ = _fit(km, X, k, 0, **kw)
    lab1, r1, rows = _fit(km, X, k, 8192, **kw)
    assert rows == 8192
    np.testing.assert_array_equal(lab0, lab1)
    assert r0.score == r1.score and r0.iterations == r1.iterations == 3
    assert lab0.max() < k and np.isfinite(r0.score)


FUSED_CASES = [("linear", {}, "bf16x3"), ("polynomial", dict(gamma=1 / 32, coef=1.0, degree=2), "bf16x3"),
               ("sigmoid", dict(gamma=0.05, coef=1.0), "bf16x3"), ("gaussian", dict(sigma=2.0), "bf16x3"),
               ("polynomial", dict(gamma=1 / 32, coef=1.0, degree=2), "bf16"), ("gaussian", dict(sigma=2.0), "bf16")]


@pytest.mark.parametrize("kind,params,prec", FUSED_CASES, ids=[f"{k}-{p}" for k, _, p in FUSED_CASES])
def test_kkm_fused_vs_fp64_oracle(km, gpu, kind, params, prec):
    """No K in memory: each row's kernel values summed per cluster in the
    tensor-core epilogue over a label-sorted operand copy (n = 3000: a ragged
    last row block and column tile)."""
    X, _ = helpers.synth_blobs_np(3000, 32, 6, -1, 1, 0.35, 9)
    it_o, lab_o, sc_o, _ = oracle_kkm(X, kind, params, 6, 8, 0.0, False)
    lab, r, rows = _fit(km, X, 6, "fused", kernel=kind, maxiter=8, precision=prec, **params)
    assert rows == km.KKM_FUSED
    assert r.iterations == 8 and r.kernel_launches == 8 * 10
    agree = float((lab == lab_o).mean())
    # the floors of the resident path (test_kkm_vs_fp64_oracle): single BF16
    # operands move a few per cent of the Gaussian kernel's thin-margin labels
    floor = 0.999 if prec == "bf16x3" else (0.98 if kind == "gaussian" else 0.99)
    assert agree >= floor, agree
    assert abs(r.score - sc_o) <= (1e-3 if prec == "bf16x3" else 2e-2) * abs(sc_o)


def test_kkm_fused_empty_clusters_vs_oracle(km, gpu):
    """k = 256 over 4096 points: clusters empty out (their E entries are
    written as zero, D = +inf) and many cluster boundaries fall inside 64-column
    chunks; against the FP64 oracle and the resident matrix."""
    X, _ = helpers.synth_blobs_np(4096, 16, 256, -4, 4, 0.3, 21)
    params = dict(gamma=1 / 16, coef=1.0, degree=2)
    it_o, lab_o, sc_o, _ = oracle_kkm(X, "polynomial", params, 256, 6, 0.0, False)
    assert len(np.unique(lab_o)) < 256
    lab, r, _ = _fit(km, X, 256, "fused", kernel="polynomial", maxiter=6, precision="bf16x3", **params)
    lab0, r0, _ = _fit(km, X, 256, 0, kernel="polynomial", maxiter=6, precision="bf16x3", **params)
    assert float((lab == lab_o).mean()) >= 0.998
    assert float((lab == lab0).mean()) >= 0.998
    assert abs(r.score - sc_o) <= 1e-4 * abs(sc_o)


def test_kkm_fused_stops_on_score_rule(km, gpu):
    """The fused iteration under the score stop rule: the iterations enqueued
    after the stop do nothing, and the stop comes where the resident path's does."""
    X, _ = helpers.synth_blobs_np(2500, 24, 5, -1, 1, 0.3, 4)
    kw = dict(kernel="polynomial", gamma=1 / 24, coef=1.0, degree=2, maxiter=60, tol=1e-3, precision="bf16x3",
              check_converged=True)
    lab0, r0, _ = _fit(km, X, 5, 0, **kw)
    lab1, r1, _ = _fit(km, X, 5, "fused", **kw)
    assert r1.converged and r1.iterations < 60
    assert abs(int(r1.converged_iter) - int(r0.converged_iter)) <= 1
    assert float((lab0 == lab1).mean()) >= 0.999


def test_kkm_fused_large_n_vs_panels(km, gpu):
    """n = 170,000, k = 64: fused against K rebuilt in panels (FP32 K).
    Integer points and the linear kernel make every K entry and every partial
    sum exact (below 2^24), so the two summation orders must agree bit for
    bit; with the polynomial kernel on real-valued points they differ by
    rounding, which moves only near-tie labels of the random-mixture clusters
    of the first iterations."""
    n, k = 170000, 64
    Xi, _ = helpers.synth_blobs_np(n, 16, k, 0, 8, 2.0, 35, round_clip=True)
    kw = dict(kernel="linear", maxiter=3, precision="bf16x3")
    lab0, r0, _ = _fit(km, Xi, k, 8192, **kw)
    lab1, r1, _ = _fit(km, Xi, k, "fused", **kw)
    np.testing.assert_array_equal(lab0, lab1)
    assert r0.score == r1.score
    X, _ = helpers.synth_blobs_np(n, 32, k, -1, 1, 0.3, 33)
    kw = dict(kernel="polynomial", gamma=1 / 32, coef=1.0, degree=2, maxiter=3, precision="bf16x3")
    lab0, r0, _ = _fit(km, X, k, 8192, **kw)
    lab1, r1, _ = _fit(km, X, k, "fused", **kw)
    # measured: 0.9997 agreement, scores 6.6e-5 apart (each moved near-tie
    # point shifts the distances of two whole clusters); the resident path's
    # split-BF16x3 score bound against the oracle is 1e-3
    assert float((lab0 == lab1).mean()) >= 0.999
    assert abs(r1.score - r0.score) <= 1e-3 * abs(r0.score)
