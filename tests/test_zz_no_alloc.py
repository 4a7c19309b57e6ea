"""km_update_noalloc: the centroid update for callers that cannot allocate
device memory (hosts that own all device memory through their own pool and
forbid cudaMalloc/cudaFree after start-up, or latency-critical loops).

It is called through the C ABI and must give exactly what km_update gives
(bit-identical centroids, identical counts: the same tolerance as the other
update tests) on two calls in a row with different inputs, because every call
reuses the same static scratch array.  This file is collected last."""
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
