"""ctypes binding of libkm_sm103 (include/km.h) for tests and benchmarks.

The library is the product; this module only marshals arguments.  It raises
if the shared library has not been built: there is no Python or CPU fallback.
Device buffers are passed as torch CUDA tensors (data_ptr()).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libkm_sm103.so"

KM_OK, KM_ERR_ARG, KM_ERR_ALLOC, KM_ERR_CUDA, KM_ERR_TIMEOUT, KM_ERR_UNSUPPORTED, KM_ERR_NO_DEVICE, KM_ERR_STATE = range(8)
INIT_SAMPLE, INIT_ROUND_ROBIN, INIT_GIVEN = 0, 1, 2
PREC = {"fp32": 0, "bf16": 1, "bf16x3": 2}
CONV = {"shift": 0, "score": 1, "none": 2}
KERNEL = {"linear": 0, "polynomial": 1, "sigmoid": 2, "gaussian": 3}


class KmError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: {_lib().km_status_str(status).decode()} (status {status})")
        self.status = status


class LloydParams(C.Structure):
    _fields_ = [("n", C.c_uint64), ("d", C.c_uint32), ("k", C.c_uint32), ("tol", C.c_float),
                ("seed", C.c_int32), ("maxiter", C.c_uint64), ("init", C.c_int32),
                ("precision", C.c_int32), ("conv", C.c_int32), ("device", C.c_int32),
                ("stream", C.c_void_p), ("empty", C.c_int32)]


class Result(C.Structure):
    _fields_ = [("converged_iter", C.c_uint64), ("iterations", C.c_uint64), ("converged", C.c_int32),
                ("reserved0", C.c_int32), ("objective", C.c_double), ("score", C.c_double),
                ("max_shift", C.c_double), ("refined_rows", C.c_uint64),
                ("full_rescore_rows", C.c_uint64), ("fit_ms", C.c_double),
                ("kernel_launches", C.c_uint64)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved0"}


class KkmParams(C.Structure):
    _fields_ = [("n", C.c_uint64), ("d", C.c_uint32), ("k", C.c_uint32), ("tol", C.c_float),
                ("maxiter", C.c_uint64), ("kernel_fn", C.c_int32), ("gamma", C.c_float),
                ("coef", C.c_float), ("sigma", C.c_float), ("degree", C.c_int32),
                ("precision", C.c_int32), ("k_bf16", C.c_int32), ("check_converged", C.c_int32),
                ("device", C.c_int32), ("stream", C.c_void_p), ("panel_rows", C.c_uint64)]


KKM_PANEL_AUTO = (1 << 64) - 1
KKM_FUSED = (1 << 64) - 2
_LIB = None

# Exported symbols with their ctypes signatures (restype, argtypes).
class BatchProblem(C.Structure):
    _fields_ = [("n", C.c_uint64), ("d", C.c_uint32), ("k", C.c_uint32)]


class BatchParams(C.Structure):
    _fields_ = [("problems", C.c_uint32), ("restarts", C.c_uint32), ("seed", C.c_int32), ("tol", C.c_float),
                ("maxiter", C.c_uint64), ("device", C.c_int32), ("stream", C.c_void_p)]


class BatchResult(C.Structure):
    _fields_ = [("converged_iter", C.c_uint64), ("iterations", C.c_uint64), ("objective", C.c_double)]


SIGNATURES = {
    "km_status_str": (C.c_char_p, [C.c_int]),
    "km_version": (C.c_char_p, []),
    "km_device_count": (C.c_int, []),
    "km_mem_info": (C.c_int, [C.c_int32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "km_lloyd_configure": (C.c_int, [C.c_void_p, C.c_uint64, C.c_float, C.c_int32]),
    "km_lloyd_init": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "km_lloyd_set_data_bf16": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "km_kkm_configure": (C.c_int, [C.c_void_p, C.c_uint64, C.c_float, C.c_int32]),
    "km_kkm_build_ms": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "km_kkm_panel_rows": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "km_lloyd_create": (C.c_int, [C.POINTER(LloydParams), C.POINTER(C.c_void_p)]),
    "km_lloyd_set_data": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "km_lloyd_fit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(Result)]),
    "km_lloyd_device_results": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "km_lloyd_profile": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_double)]),
    "km_lloyd_destroy": (None, [C.c_void_p]),
    "km_assign": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int32,
                            C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64), C.c_void_p]),
    "km_distances": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int32,
                               C.c_void_p, C.c_void_p]),
    "km_update": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p,
                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "km_update_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32,
                                    C.c_void_p, C.c_void_p, C.c_void_p]),
    "km_kernel_matrix": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint32, C.c_int32, C.c_float, C.c_float,
                                   C.c_int32, C.c_float, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                   C.c_void_p]),
    "km_kkm_create": (C.c_int, [C.POINTER(KkmParams), C.POINTER(C.c_void_p)]),
    "km_kkm_set_data": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "km_kkm_fit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(Result)]),
    "km_kkm_destroy": (None, [C.c_void_p]),
    "km_batch_create": (C.c_int, [C.POINTER(BatchParams), C.POINTER(BatchProblem), C.POINTER(C.c_void_p)]),
    "km_batch_set_data": (C.c_int, [C.c_void_p, C.c_void_p]),
    "km_batch_tune": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "km_batch_fit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "km_batch_instance_labels": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]),
    "km_batch_destroy": (None, [C.c_void_p]),
    "km_synth_blobs": (C.c_int, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_double, C.c_double, C.c_int32, C.c_uint64, C.c_int32,
                                 C.c_void_p, C.c_void_p]),
}


def _lib():
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is not built (run __graft_entry__.build())")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    return _LIB


def lib():
    return _lib()


def check(status: int, what: str):
    if status != KM_OK:
        raise KmError(status, what)


def device_count() -> int:
    return _lib().km_device_count()


def _ptr(t) -> int:
    return 0 if t is None else int(t.data_ptr())


def synth_blobs(n, d, blobs, lo, hi, sigma, seed, round_clip=False, sigma_range=None, zipf_s=0.0,
                nthreads=8, with_blob=False):
    X = np.empty((n, d), np.float32)
    b = np.empty(n, np.uint32) if with_blob else None
    slo, shi = sigma_range if sigma_range else (0.0, 0.0)
    check(_lib().km_synth_blobs(n, d, blobs, lo, hi, sigma, slo, shi, zipf_s, int(round_clip), seed,
                                nthreads, X.ctypes.data, b.ctypes.data if b is not None else None),
          "km_synth_blobs")
    return (X, b) if with_blob else X


class Lloyd:
    """Handle over km_lloyd_*: the Kmeans(...) / run() / get_score() surface."""

    def __init__(self, n, d, k, tol=1e-4, seed=0, maxiter=300, init="sample", precision="fp32",
                 conv="shift", device=0, stream=0, empty="zero"):
        self.p = LloydParams(n, d, k, tol, seed, maxiter,
                             {"sample": INIT_SAMPLE, "round_robin": INIT_ROUND_ROBIN, "given": INIT_GIVEN,
                              "plusplus": 3}[init],
                             PREC[precision], CONV[conv], device, stream or None,
                             {"zero": 0, "exclude": 1}[empty])
        h = C.c_void_p()
        check(_lib().km_lloyd_create(C.byref(self.p), C.byref(h)), "km_lloyd_create")
        self.h = h

    def set_data(self, X):
        if isinstance(X, np.ndarray):
            X = np.ascontiguousarray(X, dtype=np.float32)
            check(_lib().km_lloyd_set_data(self.h, X.ctypes.data, 0), "km_lloyd_set_data")
        else:
            check(_lib().km_lloyd_set_data(self.h, X.data_ptr(), 1), "km_lloyd_set_data")
        return self

    def set_data_bf16(self, Xbits):
        """Points stored as BF16: a uint16 numpy array of the bit patterns, or a
        torch.bfloat16 / int16 device tensor."""
        if isinstance(Xbits, np.ndarray):
            Xbits = np.ascontiguousarray(Xbits, dtype=np.uint16)
            check(_lib().km_lloyd_set_data_bf16(self.h, Xbits.ctypes.data, 0), "km_lloyd_set_data_bf16")
        else:
            check(_lib().km_lloyd_set_data_bf16(self.h, Xbits.data_ptr(), 1), "km_lloyd_set_data_bf16")
        return self

    def fit(self, C0=None, want_centroids=True):
        n, k, d = self.p.n, self.p.k, self.p.d
        labels = np.empty(n, np.uint32)
        cents = np.empty((k, d), np.float32) if want_centroids else None
        c0 = None
        if C0 is not None:
            c0 = np.ascontiguousarray(C0, dtype=np.float32)
        r = Result()
        check(_lib().km_lloyd_fit(self.h, c0.ctypes.data if c0 is not None else None, labels.ctypes.data,
                                  cents.ctypes.data if cents is not None else None, C.byref(r)),
              "km_lloyd_fit")
        return labels, cents, r

    def init_centroids(self, C0=None):
        """The configured initialisation alone (km_lloyd_init)."""
        out = np.empty((self.p.k, self.p.d), np.float32)
        c0 = None if C0 is None else np.ascontiguousarray(C0, dtype=np.float32)
        check(_lib().km_lloyd_init(self.h, None if c0 is None else c0.ctypes.data, out.ctypes.data),
              "km_lloyd_init")
        return out

    def profile(self, iters):
        """Mean ms per iteration of the five stages (see km_lloyd_profile)."""
        out = (C.c_double * 5)()
        check(_lib().km_lloyd_profile(self.h, iters, out), "km_lloyd_profile")
        return list(out)

    def close(self):
        if self.h:
            _lib().km_lloyd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def kernel_matrix(X, kernel="linear", gamma=1.0, coef=1.0, degree=2, sigma=1.0, precision="fp32",
                  out_bf16=False, want_diag=False):
    """K = f(X X^T) for a torch CUDA tensor X (n, d)."""
    import torch
    n, d = X.shape
    K = torch.empty((n, n), dtype=torch.bfloat16 if out_bf16 else torch.float32, device=X.device)
    dg = torch.empty(n, dtype=torch.float32, device=X.device) if want_diag else None
    check(_lib().km_kernel_matrix(_ptr(X), n, d, KERNEL[kernel], gamma, coef, degree, sigma, PREC[precision],
                                  int(out_bf16), _ptr(K), _ptr(dg), torch.cuda.current_stream().cuda_stream),
          "km_kernel_matrix")
    return (K, dg) if want_diag else K


class KernelKMeans:
    """Handle over km_kkm_*: kernel k-means with the reference GPU path's semantics."""

    def __init__(self, n, d, k, kernel="linear", gamma=1.0, coef=1.0, degree=2, sigma=1.0, tol=1e-4,
                 maxiter=30, precision="fp32", k_bf16=False, check_converged=False, device=0, stream=0,
                 panel_rows=0):
        """panel_rows: 0 keeps K resident (n*n); r > 0 rebuilds K every
        iteration in panels of r rows; "fused" (KKM_FUSED) keeps no K and sums
        the kernel values per cluster inside the tensor-core kernel; "auto"
        (KKM_PANEL_AUTO) leaves K resident when n*n fits the free device
        memory, else fused (tensor-core precisions) or panels (FP32)."""
        pr = {"auto": KKM_PANEL_AUTO, "fused": KKM_FUSED}.get(panel_rows, panel_rows)
        pr = int(pr)
        self.p = KkmParams(n, d, k, tol, maxiter, KERNEL[kernel], gamma, coef, sigma, degree, PREC[precision],
                           int(k_bf16), int(check_converged), device, stream or None, pr)
        h = C.c_void_p()
        check(_lib().km_kkm_create(C.byref(self.p), C.byref(h)), "km_kkm_create")
        self.h = h

    def set_data(self, X):
        if isinstance(X, np.ndarray):
            X = np.ascontiguousarray(X, dtype=np.float32)
            check(_lib().km_kkm_set_data(self.h, X.ctypes.data, 0), "km_kkm_set_data")
        else:
            check(_lib().km_kkm_set_data(self.h, X.data_ptr(), 1), "km_kkm_set_data")
        return self

    def build_ms(self):
        """Device time of the kernel-matrix build of the last set_data."""
        ms = C.c_double(0)
        check(_lib().km_kkm_build_ms(self.h, C.byref(ms)), "km_kkm_build_ms")
        return ms.value

    def panel_rows(self):
        """Rows of K per panel (0: K resident, KKM_FUSED: no K)."""
        r = C.c_uint64(0)
        check(_lib().km_kkm_panel_rows(self.h, C.byref(r)), "km_kkm_panel_rows")
        return r.value

    def fit(self, init_labels=None):
        lab = np.empty(self.p.n, np.uint32)
        il = None if init_labels is None else np.ascontiguousarray(init_labels, np.uint32)
        r = Result()
        check(_lib().km_kkm_fit(self.h, None if il is None else il.ctypes.data, lab.ctypes.data, C.byref(r)),
              "km_kkm_fit")
        return lab, r

    def close(self):
        if self.h:
            _lib().km_kkm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def assign(X, Cc, precision="fp32", want_mindist=False):
    """labels (and fast-path min distance) of torch CUDA tensors X (n,d), C (k,d)."""
    import torch
    n, d = X.shape
    k = Cc.shape[0]
    lab = torch.empty(n, dtype=torch.int32, device=X.device)
    md = torch.empty(n, dtype=torch.float32, device=X.device) if want_mindist else None
    ref = C.c_uint64(0)
    check(_lib().km_assign(_ptr(X), _ptr(Cc), n, d, k, PREC[precision], _ptr(lab), _ptr(md), C.byref(ref),
                           torch.cuda.current_stream().cuda_stream), "km_assign")
    return lab, md, ref.value


def distances(X, Cc, precision="fp32"):
    import torch
    n, d = X.shape
    k = Cc.shape[0]
    D = torch.empty((n, k), dtype=torch.float32, device=X.device)
    check(_lib().km_distances(_ptr(X), _ptr(Cc), n, d, k, PREC[precision], _ptr(D),
                              torch.cuda.current_stream().cuda_stream), "km_distances")
    return D


def update(X, labels, k):
    import torch
    n, d = X.shape
    Cc = torch.empty((k, d), dtype=torch.float32, device=X.device)
    cnt = torch.empty(k, dtype=torch.int32, device=X.device)
    perm = torch.empty(n, dtype=torch.int32, device=X.device)
    off = torch.empty(k + 1, dtype=torch.int32, device=X.device)
    check(_lib().km_update(_ptr(X), _ptr(labels), n, d, k, _ptr(Cc), _ptr(cnt), _ptr(perm), _ptr(off),
                           torch.cuda.current_stream().cuda_stream), "km_update")
    return Cc, cnt, perm, off


class Batch:
    """Handle over km_batch_*: many independent Lloyd problems (list of (n, d, k)),
    `restarts` seeded restarts each, in one persistent launch."""

    def __init__(self, shapes, restarts=8, seed=0, tol=1e-4, maxiter=300, device=0, stream=0):
        self.shapes = [(int(n), int(d), int(k)) for n, d, k in shapes]
        self.restarts = restarts
        arr = (BatchProblem * len(self.shapes))(*[BatchProblem(n, d, k) for n, d, k in self.shapes])
        self.p = BatchParams(len(self.shapes), restarts, seed, tol, maxiter, device, stream or None)
        h = C.c_void_p()
        check(_lib().km_batch_create(C.byref(self.p), arr, C.byref(h)), "km_batch_create")
        self.h = h

    def set_data(self, Xs):
        """Xs: list of (n, d) float32 arrays, one per problem."""
        packed = np.concatenate([np.ascontiguousarray(x, np.float32).ravel() for x in Xs])
        check(_lib().km_batch_set_data(self.h, packed.ctypes.data), "km_batch_set_data")
        return self

    def tune(self):
        v = C.c_int32(-1)
        ms = (C.c_double * 6)()
        check(_lib().km_batch_tune(self.h, C.byref(v), ms), "km_batch_tune")
        return v.value, list(ms)

    def fit(self):
        P, R = len(self.shapes), self.restarts
        res = (BatchResult * (P * R))()
        lab = np.empty(sum(n for n, _, _ in self.shapes), np.uint32)
        cen = np.empty(sum(k * d for _, d, k in self.shapes), np.float32)
        ms = C.c_double(0)
        check(_lib().km_batch_fit(self.h, res, lab.ctypes.data, cen.ctypes.data, C.byref(ms)), "km_batch_fit")
        out, lo, co = [], 0, 0
        for (n, d, k) in self.shapes:
            out.append((lab[lo:lo + n], cen[co:co + k * d].reshape(k, d)))
            lo += n
            co += k * d
        results = [[(res[p * R + r].converged_iter, res[p * R + r].iterations, res[p * R + r].objective)
                    for r in range(R)] for p in range(P)]
        return out, results, ms.value

    def instance(self, problem, restart):
        n, d, k = self.shapes[problem]
        lab = np.empty(n, np.uint32)
        cen = np.empty((k, d), np.float32)
        check(_lib().km_batch_instance_labels(self.h, problem, restart, lab.ctypes.data, cen.ctypes.data),
              "km_batch_instance_labels")
        return lab, cen

    def close(self):
        if self.h:
            _lib().km_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

