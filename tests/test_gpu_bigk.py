"""k > 256 (the chunked tensor-core distance kernel) and points stored as BF16:
labels, iteration counts and centroids identical to the oracle's restatement
of the reference CPU k-means in every precision, on uniform and Zipf-sized
clusters with per-cluster widths (the very-large-k workload, scaled down)."""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu
PRECISIONS = ["fp32", "bf16", "bf16x3"]


def to_bf16_bits(X):
    """Round-to-nearest-even FP32 -> BF16 bit patterns (finite inputs)."""
    b = np.ascontiguousarray(X, np.float32).view(np.uint32).astype(np.uint64)
    r = (b + 0x7FFF + ((b >> 16) & 1)) >> 16
    return r.astype(np.uint16)


def from_bf16_bits(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_lloyd_k600_matches_oracle(km, gpu, prec):
    X, _ = helpers.synth_blobs_np(20000, 48, 600, -10, 10, 1.0, 23)
    k, maxiter = 600, 8
    it_o, lab_o, cen_o, ex_o = helpers.orc_lloyd(X, k, 1e-4, 3, maxiter)
    m = km.Lloyd(20000, 48, k, tol=1e-4, seed=3, maxiter=maxiter, precision=prec).set_data(X)
    lab, cen, r = m.fit()
    m.close()
    np.testing.assert_array_equal(lab, lab_o)
    np.testing.assert_array_equal(cen.view(np.uint32), cen_o.view(np.uint32))
    assert r.converged_iter == it_o and r.iterations == ex_o


@pytest.mark.parametrize("prec", PRECISIONS)
def test_zipf_bf16_points_k1024(km, gpu, prec):
    """Zipf(1.1) cluster sizes, per-cluster sigma in [0.2, 2], centers in
    [-20, 20]^256, points stored as BF16."""
    n, d, k = 30000, 256, 1024
    X = km.synth_blobs(n, d, k, -20.0, 20.0, 1.0, 77, sigma_range=(0.2, 2.0), zipf_s=1.1)
    bits = to_bf16_bits(X)
    Xd = from_bf16_bits(bits)
    maxiter = 4
    it_o, lab_o, cen_o, ex_o = helpers.orc_lloyd(Xd, k, 1e-5, 9, maxiter)
    m = km.Lloyd(n, d, k, tol=1e-5, seed=9, maxiter=maxiter, precision=prec).set_data_bf16(bits)
    lab, cen, r = m.fit()
    m.close()
    np.testing.assert_array_equal(lab, lab_o)
    np.testing.assert_array_equal(cen.view(np.uint32), cen_o.view(np.uint32))
    assert r.iterations == ex_o
    sizes = np.bincount(lab, minlength=k)
    assert sizes.max() > 20 * max(1, int(np.median(sizes)))     # the Zipf head is there


def test_bf16_points_device_input(km, gpu):
    import torch
    n, d, k = 5000, 64, 300
    X = km.synth_blobs(n, d, k, -5.0, 5.0, 0.5, 5)
    bits = to_bf16_bits(X)
    Xd = from_bf16_bits(bits)
    t = torch.from_numpy(bits.view(np.int16)).to(gpu)
    m1 = km.Lloyd(n, d, k, seed=1, maxiter=5, precision="bf16").set_data_bf16(t)
    m2 = km.Lloyd(n, d, k, seed=1, maxiter=5, precision="bf16").set_data(Xd)
    l1, c1, _ = m1.fit()
    l2, c2, _ = m2.fit()
    m1.close(); m2.close()
    np.testing.assert_array_equal(l1, l2)
    np.testing.assert_array_equal(c1, c2)
