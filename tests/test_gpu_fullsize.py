"""Parity at the workloads' full sizes, through the C ABI, against the oracle.

* n = 1,048,576, d = 128, k = 256 (256 blobs, centers U[-10,10]^128, sigma 1,
  the bench's own points): five iterations from the seeded sample picks in
  every precision give labels, centroids and the returned iteration bit for
  bit equal to the oracle's restatement of the reference CPU k-means
  (comparisons/CPU_Kmeans/src/kmeans.cpp:49-200), and, against the FP64
  oracle from the same start, >= 99.9 % label agreement and an objective
  within 1e-4 relative (the reduced-precision bar; measured: identical labels).
* n = 4,194,304, d = 256, k = 4096, BF16-stored points, Zipf(1.1) cluster
  sizes: one fit of two iterations; the centroids equal the oracle's update of
  the fit's labels over all n rows bit for bit, and the assignment of all n
  rows to the fit's centroids equals the oracle's on a sample of rows spread
  over the whole range (a whole-n oracle iteration at k = 4096 takes minutes
  on the host)."""
import os

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 8
AGREE_MIN, OBJ_RTOL = 0.999, 1e-4


@pytest.fixture(scope="module")
def lloyd_1m(km):
    n, d, k = 1_048_576, 128, 256
    X = km.synth_blobs(n, d, 256, -10.0, 10.0, 1.0, 1000, nthreads=THREADS)
    it32, lab32, cen32, ex32 = helpers.orc_lloyd(X, k, 1e-4, 0, 5, threads=THREADS)
    it64, lab64, _, _, obj64 = helpers.orc_lloyd64_obj(X, k, 1e-4, 0, 5, threads=THREADS)
    return X, (it32, lab32, cen32, ex32), (lab64, obj64)


@pytest.mark.parametrize("prec", ["fp32", "bf16", "bf16x3"])
def test_n1m_d128_k256_bitwise_vs_oracle(km, gpu, lloyd_1m, prec):
    import torch
    X, (it32, lab32, cen32, ex32), (lab64, obj64) = lloyd_1m
    n, d = X.shape
    Xd = torch.from_numpy(X).to(gpu)
    m = km.Lloyd(n, d, 256, tol=1e-4, seed=0, maxiter=5, precision=prec).set_data(Xd)
    lab, cen, r = m.fit()
    m.close()
    np.testing.assert_array_equal(lab, lab32)
    np.testing.assert_array_equal(cen.view(np.uint32), cen32.view(np.uint32))
    assert r.converged_iter == it32 and r.iterations == ex32
    assert (lab == lab64).mean() >= AGREE_MIN
    assert abs(r.objective - obj64) <= OBJ_RTOL * obj64


def to_bf16_bits(X):
    b = np.ascontiguousarray(X, np.float32).view(np.uint32).astype(np.uint64)
    return ((b + 0x7FFF + ((b >> 16) & 1)) >> 16).astype(np.uint16)


@pytest.fixture(scope="module")
def bigk_points(km):
    n, d, k = 4_194_304, 256, 4096
    X = km.synth_blobs(n, d, k, -20.0, 20.0, 1.0, 5000, sigma_range=(0.2, 2.0), zipf_s=1.1, nthreads=THREADS)
    bits = np.empty((n, d), np.uint16)
    for r0 in range(0, n, 262144):
        bits[r0:r0 + 262144] = to_bf16_bits(X[r0:r0 + 262144])
    del X
    return bits


@pytest.mark.parametrize("prec", ["bf16", "bf16x3"])
def test_n4m_d256_k4096_bf16_points_vs_oracle(km, gpu, bigk_points, prec):
    import torch
    bits = bigk_points
    n, d = bits.shape
    k = 4096
    tb = torch.from_numpy(bits.view(np.int16)).to(gpu)
    m = km.Lloyd(n, d, k, tol=1e-5, seed=1, maxiter=2, precision=prec, conv="none").set_data_bf16(tb)
    lab, cen, r = m.fit()
    m.close()
    assert r.iterations == 2
    Xf = tb.view(torch.bfloat16).float()                    # the points as FP32 (exact)
    del tb
    X = Xf.cpu().numpy()
    # (c) the update: the fit's centroids are the oracle's update of its labels
    cen_o, cnt_o = helpers.orc_update(X, lab, k, threads=THREADS)
    np.testing.assert_array_equal(cen.view(np.uint32), cen_o.view(np.uint32))
    assert int(np.bincount(lab, minlength=k).max()) == int(cnt_o.max())
    # (a)+(b) the assignment of all n rows against those centroids, checked on
    # 16384 rows spread over the whole range
    lab_all, _, _ = km.assign(Xf, torch.from_numpy(cen).to(gpu), precision=prec)
    lab_all = lab_all.cpu().numpy()
    rows = np.random.default_rng(11).choice(n, 16384, replace=False)
    rows.sort()
    lab_s, _ = helpers.orc_assign(X[rows], cen, threads=THREADS)
    np.testing.assert_array_equal(lab_all[rows].astype(np.uint32), lab_s)


# ---------------------------------------------------------------------------
# Kernel k-means, n = 65,536, d = 512, k = 64 (64 blobs, centers U[-1,1]^512,
# sigma 0.25), K resident (FP32 16 GiB or BF16 8 GiB).  One iteration against
# the FP64 oracle from the same labels (the fit's labels after four
# iterations from i % k): >= 99.9 % label agreement and the objective
# (score + trace K) within 1e-4 relative, the reduced-precision bar.  An FP64
# kernel matrix of this size (34 GB) is formed block by block by the oracle.
# ---------------------------------------------------------------------------
def _kkm_step_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("kkm_step", helpers.ORACLE / "kkm_step.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def kkm_points(km):
    return km.synth_blobs(65536, 512, 64, -1.0, 1.0, 0.25, 3000, nthreads=THREADS)


@pytest.mark.parametrize("kind,params,prec,kb16", [
    ("polynomial", dict(gamma=1 / 512, coef=1.0, degree=2), "bf16x3", False),
    ("polynomial", dict(gamma=1 / 512, coef=1.0, degree=2), "bf16", True),
    ("gaussian", dict(sigma=0.5), "bf16", True),
])
def test_kkm_n65536_d512_k64_one_step_vs_fp64(km, gpu, kkm_points, kind, params, prec, kb16):
    import torch
    ks = _kkm_step_module()
    X = kkm_points
    n, d = X.shape
    k = 64
    m = km.KernelKMeans(n, d, k, kernel=kind, maxiter=4, precision=prec, k_bf16=kb16,
                        **params).set_data(torch.from_numpy(X).to(gpu))
    lab_a, _ = m.fit()
    km.check(km.lib().km_kkm_configure(m.h, 1, m.p.tol, 0), "km_kkm_configure")
    lab_b, r = m.fit(init_labels=lab_a)
    m.close()
    torch.cuda.empty_cache()
    new, score = ks.kkm_step_f64(X, lab_a, k, kind, **params, workers=THREADS // 2)
    agree = float((lab_b == new).mean())
    trace = float(ks.kernel_diag(X, kind, **params).sum())
    rel = abs((r.score + trace) - (score + trace)) / abs(score + trace)
    assert agree >= AGREE_MIN, agree
    assert rel <= OBJ_RTOL, rel
