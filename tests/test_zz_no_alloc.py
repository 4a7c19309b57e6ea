"""km_update_noalloc: the centroid update for callers that cannot allocate
device memory (hosts that own all device memory through their own pool and
forbid cudaMalloc/cudaFree after start-up, or latency-critical loops).

It is called through the C ABI and must give exactly what km_update gives
(bit-identical centroids, identical counts: the same tolerance as the other
update tests) on two calls in a row with different inputs, because every call
reuses the same static scratch array.  A warmed-up call must leave the
device's free memory unchanged, and an error (labels >= k) must be reported
and must not leak into the next call.  This file is collected last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(km, X, lab, k):
    import torch
    n, d = X.shape
    Cc = torch.full((k, d), float("nan"), device=X.device)
    cnt = torch.full((k,), -1, dtype=torch.int32, device=X.device)
    st = km.lib().km_update_noalloc(X.data_ptr(), lab.data_ptr(), n, d, k, Cc.data_ptr(), cnt.data_ptr(),
                                    torch.cuda.current_stream().cuda_stream)
    km.check(st, "km_update_noalloc")
    torch.cuda.synchronize()
    return Cc, cnt


@pytest.mark.parametrize("shape", [[(200000, 37, 300), (70001, 128, 1024)], [(1000, 5, 7), (1048576, 16, 64)]])
def test_noalloc_update_matches_km_update_twice(km, gpu, shape):
    import torch
    rng = np.random.default_rng(17)
    for (n, d, k) in shape:
        X = torch.from_numpy((rng.standard_normal((n, d)) * 10).astype(np.float32)).to(gpu)
        lab = torch.from_numpy(rng.integers(0, k - 3, n).astype(np.int32)).to(gpu)   # some clusters empty
        C_ref, cnt_ref, _, _ = km.update(X, lab, k)
        C_na, cnt_na = _noalloc(km, X, lab, k)
        np.testing.assert_array_equal(C_na.cpu().numpy().view(np.uint32), C_ref.cpu().numpy().view(np.uint32))
        np.testing.assert_array_equal(cnt_na.cpu().numpy(), cnt_ref.cpu().numpy())


def test_noalloc_rejects_sizes_beyond_its_scratch(km, gpu):
    import torch
    lib = km.lib()
    X = torch.zeros((4, 4), device=gpu)
    lab = torch.zeros(4, dtype=torch.int32, device=gpu)
    Cc = torch.zeros((2048, 4), device=gpu)
    s = torch.cuda.current_stream().cuda_stream
    too_many_rows = 1048577
    assert lib.km_update_noalloc(X.data_ptr(), lab.data_ptr(), too_many_rows, 4, 2, Cc.data_ptr(), None, s) \
        == km.KM_ERR_UNSUPPORTED
    assert lib.km_update_noalloc(X.data_ptr(), lab.data_ptr(), 2000, 4, 1025, Cc.data_ptr(), None, s) \
        == km.KM_ERR_UNSUPPORTED
    bad = torch.full((4,), 9, dtype=torch.int32, device=gpu)
    assert lib.km_update_noalloc(X.data_ptr(), bad.data_ptr(), 4, 4, 2, Cc.data_ptr(), None, s) == km.KM_ERR_ARG


def test_noalloc_allocates_nothing(km, gpu):
    """After the first call on the device (which looks up the array), further
    calls change neither the device's free memory nor torch's allocator.  The
    outputs are allocated once, before the measurement."""
    import torch
    rng = np.random.default_rng(5)
    n, d, k = 300000, 64, 200
    X = torch.from_numpy(rng.standard_normal((n, d)).astype(np.float32)).to(gpu)
    lab = torch.from_numpy(rng.integers(0, k, n).astype(np.int32)).to(gpu)
    Cc = torch.empty((k, d), device=gpu)
    cnt = torch.empty((k,), dtype=torch.int32, device=gpu)
    s = torch.cuda.current_stream().cuda_stream
    lib = km.lib()

    def call():
        km.check(lib.km_update_noalloc(X.data_ptr(), lab.data_ptr(), n, d, k, Cc.data_ptr(), cnt.data_ptr(), s),
                 "km_update_noalloc")

    call()                                               # first call: set-up on this device
    torch.cuda.synchronize()
    first = Cc.cpu().numpy().copy()
    free0, _ = torch.cuda.mem_get_info()
    reserved0 = torch.cuda.memory_reserved()
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_reserved() == reserved0
    np.testing.assert_array_equal(Cc.cpu().numpy().view(np.uint32), first.view(np.uint32))


def test_noalloc_error_does_not_leak_into_the_next_call(km, gpu):
    """A label >= k returns KM_ERR_ARG; the next call with valid labels
    succeeds and matches km_update (the error bits start at zero each call)."""
    import torch
    rng = np.random.default_rng(9)
    n, d, k = 50000, 32, 40
    X = torch.from_numpy(rng.standard_normal((n, d)).astype(np.float32)).to(gpu)
    good = rng.integers(0, k, n).astype(np.int32)
    bad = good.copy()
    bad[12345] = k + 3
    Cc = torch.empty((k, d), device=gpu)
    s = torch.cuda.current_stream().cuda_stream
    lb = torch.from_numpy(bad).to(gpu)
    assert km.lib().km_update_noalloc(X.data_ptr(), lb.data_ptr(), n, d, k, Cc.data_ptr(), None, s) \
        == km.KM_ERR_ARG
    lg = torch.from_numpy(good).to(gpu)
    C_na, cnt_na = _noalloc(km, X, lg, k)
    C_ref, cnt_ref, _, _ = km.update(X, lg, k)
    np.testing.assert_array_equal(C_na.cpu().numpy().view(np.uint32), C_ref.cpu().numpy().view(np.uint32))
    np.testing.assert_array_equal(cnt_na.cpu().numpy(), cnt_ref.cpu().numpy())
