"""Shared test helpers: loaders for the product library (km.py), the oracle
(oracle/liboracle.so) and the reference build (oracle/_ref), plus a numpy twin
of the synthetic-data generator."""
from __future__ import annotations

import ctypes as C
import importlib.util
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "matrix-centric-k-means_gb300"
ORACLE = ROOT / "oracle"


def _reference_root() -> Path:
    """The reference tree's root as oracle/build_ref.sh resolves it (its
    argument, $KM_REFERENCE_ROOT, or its default); it may not exist (the GPU
    box has no reference tree)."""
    try:
        out = subprocess.run([str(ORACLE / "build_ref.sh"), "--print-root"], capture_output=True,
                             text=True, check=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return Path("/nonexistent-reference-root")
    return Path(out)


REFERENCE = _reference_root()

_km = None


def km():
    """The product's ctypes binding (matrix-centric-k-means_gb300/km.py)."""
    global _km
    if _km is None:
        spec = importlib.util.spec_from_file_location("km_gb300", PKG / "km.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        _km = mod
    return _km


# ---------------------------------------------------------------------------
# Oracle (test infrastructure)
# ---------------------------------------------------------------------------
_orc = None


def oracle():
    global _orc
    if _orc is None:
        so = ORACLE / "liboracle.so"
        src = ORACLE / "km_oracle.cpp"
        if not so.exists() or so.stat().st_mtime < src.stat().st_mtime:
            subprocess.run(["make", "-C", str(ORACLE), "-s"], check=True)
        lib = C.CDLL(str(so))
        u64, u32, f32, i32, vp = C.c_uint64, C.c_uint32, C.c_float, C.c_int, C.c_void_p
        lib.orc_sample_picks.restype = i32
        lib.orc_sample_picks.argtypes = [vp, u64, u32, u32, i32, vp]
        lib.orc_assign_f32.restype = None
        lib.orc_assign_f32.argtypes = [vp, vp, u64, u32, u32, i32, vp, vp]
        lib.orc_update_f32.restype = None
        lib.orc_update_f32.argtypes = [vp, vp, u64, u32, u32, i32, vp, vp]
        lib.orc_lloyd_f32.restype = u64
        lib.orc_lloyd_f32.argtypes = [vp, u64, u32, u32, f32, i32, u64, vp, i32, vp, vp, C.POINTER(u64)]
        lib.orc_lloyd_f64.restype = u64
        lib.orc_lloyd_f64.argtypes = [vp, u64, u32, u32, C.c_double, i32, u64, vp, i32, vp, vp, C.POINTER(u64)]
        lib.orc_lloyd_f64_obj.restype = u64
        lib.orc_lloyd_f64_obj.argtypes = [vp, u64, u32, u32, C.c_double, i32, u64, vp, i32, vp, vp,
                                          C.POINTER(u64), C.POINTER(C.c_double)]
        lib.orc_plusplus.restype = i32
        lib.orc_plusplus.argtypes = [vp, u64, u32, u32, i32, i32, vp]
        lib.orc_inertia.restype = C.c_double
        lib.orc_inertia.argtypes = [vp, vp, vp, u64, u32, u32, i32]
        lib.orc_kernel_matrix.restype = None
        lib.orc_kernel_matrix.argtypes = [vp, u64, u32, i32, C.c_double, C.c_double, i32, C.c_double, i32, vp]
        lib.orc_kernel_kmeans.restype = u64
        lib.orc_kernel_kmeans.argtypes = [vp, u64, u32, u64, C.c_double, i32, i32, vp, vp, C.POINTER(u64)]
        _orc = lib
    return _orc


def orc_lloyd(X, k, tol, seed, maxiter, C0=None, threads=8):
    X = np.ascontiguousarray(X, np.float32)
    n, d = X.shape
    lab = np.empty(n, np.uint32)
    cen = np.empty((k, d), np.float32)
    ex = C.c_uint64(0)
    c0 = None if C0 is None else np.ascontiguousarray(C0, np.float32)
    it = oracle().orc_lloyd_f32(X.ctypes.data, n, d, k, tol, seed, maxiter,
                                None if c0 is None else c0.ctypes.data, threads, lab.ctypes.data,
                                cen.ctypes.data, C.byref(ex))
    return int(it), lab, cen, int(ex.value)


def orc_lloyd64(X, k, tol, seed, maxiter, C0=None, threads=8):
    X = np.ascontiguousarray(X, np.float32)
    n, d = X.shape
    lab = np.empty(n, np.uint32)
    cen = np.empty((k, d), np.float64)
    ex = C.c_uint64(0)
    c0 = None if C0 is None else np.ascontiguousarray(C0, np.float32)
    it = oracle().orc_lloyd_f64(X.ctypes.data, n, d, k, tol, seed, maxiter,
                                None if c0 is None else c0.ctypes.data, threads, lab.ctypes.data,
                                cen.ctypes.data, C.byref(ex))
    return int(it), lab, cen, int(ex.value)


def orc_lloyd64_obj(X, k, tol, seed, maxiter, C0=None, threads=8):
    """FP64 oracle Lloyd; also returns the FP64 objective of its last
    assignment step (iters, labels, centroids, executed, objective)."""
    X = np.ascontiguousarray(X, np.float32)
    n, d = X.shape
    lab = np.empty(n, np.uint32)
    cen = np.empty((k, d), np.float64)
    ex = C.c_uint64(0)
    obj = C.c_double(0.0)
    c0 = None if C0 is None else np.ascontiguousarray(C0, np.float32)
    it = oracle().orc_lloyd_f64_obj(X.ctypes.data, n, d, k, tol, seed, maxiter,
                                    None if c0 is None else c0.ctypes.data, threads, lab.ctypes.data,
                                    cen.ctypes.data, C.byref(ex), C.byref(obj))
    return int(it), lab, cen, int(ex.value), float(obj.value)


def orc_plusplus(X, k, seed, threads=8):
    """The oracle's seeded greedy k-means++: the k picked row indices."""
    X = np.ascontiguousarray(X, np.float32)
    picks = np.empty(k, np.int64)
    rc = oracle().orc_plusplus(X.ctypes.data, X.shape[0], X.shape[1], k, seed, threads, picks.ctypes.data)
    if rc != 0:
        raise ValueError("orc_plusplus: unsupported k")
    return picks


def orc_assign(X, Cc, threads=8):
    X = np.ascontiguousarray(X, np.float32)
    Cc = np.ascontiguousarray(Cc, np.float32)
    n, d = X.shape
    k = Cc.shape[0]
    lab = np.empty(n, np.uint32)
    md = np.empty(n, np.float32)
    oracle().orc_assign_f32(X.ctypes.data, Cc.ctypes.data, n, d, k, threads, lab.ctypes.data, md.ctypes.data)
    return lab, md


def orc_update(X, labels, k, threads=8):
    X = np.ascontiguousarray(X, np.float32)
    labels = np.ascontiguousarray(labels, np.uint32)
    n, d = X.shape
    Cc = np.empty((k, d), np.float32)
    cnt = np.empty(k, np.uint32)
    oracle().orc_update_f32(X.ctypes.data, labels.ctypes.data, n, d, k, threads, Cc.ctypes.data, cnt.ctypes.data)
    return Cc, cnt


def orc_inertia(X, labels, Cc, threads=8):
    X = np.ascontiguousarray(X, np.float32)
    n, d = X.shape
    return oracle().orc_inertia(X.ctypes.data, np.ascontiguousarray(labels, np.uint32).ctypes.data,
                                np.ascontiguousarray(Cc, np.float32).ctypes.data, n, d, Cc.shape[0], threads)


def orc_sample_picks(X, k, seed):
    X = np.ascontiguousarray(X, np.float32)
    picks = np.empty(k, np.int32)
    rc = oracle().orc_sample_picks(X.ctypes.data, X.shape[0], X.shape[1], k, seed, picks.ctypes.data)
    return rc, picks


# ---------------------------------------------------------------------------
# The reference's own CPU k-means, built from its sources (oracle/_ref)
# ---------------------------------------------------------------------------
_ref = None


def reference_lib():
    """Loads oracle/_ref/libref_kmeans.so, building it when the reference tree
    is present.  Returns None where neither exists (e.g. on the GPU machine)."""
    global _ref
    if _ref is None:
        so = ORACLE / "_ref" / "libref_kmeans.so"
        if not so.exists() and REFERENCE.exists():
            subprocess.run([str(ORACLE / "build_ref.sh")], check=True, capture_output=True)
        if not so.exists():
            return None
        try:
            lib = C.CDLL(str(so))
        except OSError:
            return None
        lib.ref_cpu_kmeans.restype = C.c_uint64
        lib.ref_cpu_kmeans.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_float,
                                       C.c_int, C.c_uint64, C.c_void_p]
        _ref = lib
    return _ref


def ref_lloyd(X, k, tol, seed, maxiter):
    X = np.ascontiguousarray(X, np.float32)
    lab = np.empty(X.shape[0], np.uint32)
    it = reference_lib().ref_cpu_kmeans(X.ctypes.data, X.shape[0], X.shape[1], k, tol, seed, maxiter,
                                        lab.ctypes.data)
    return int(it), lab


_ref_io = None


def reference_io_lib():
    """oracle/_ref/libref_io.so: the reference's own dataset reader/writer
    (src/include/input_parser.hpp) behind C entry points; None where the
    reference tree is absent."""
    global _ref_io
    if _ref_io is None:
        so = ORACLE / "_ref" / "libref_io.so"
        if not so.exists() and REFERENCE.exists():
            subprocess.run([str(ORACLE / "build_ref.sh")], check=True, capture_output=True)
        if not so.exists():
            return None
        lib = C.CDLL(str(so))
        vp, u64 = C.c_void_p, C.c_uint64
        lib.ref_io_read.restype = None
        lib.ref_io_read.argtypes = [C.c_char_p, u64, C.c_int, C.c_int, u64, vp]
        lib.ref_io_random.restype = None
        lib.ref_io_random.argtypes = [C.c_int, C.c_int, u64, vp]
        lib.ref_io_to_csv.restype = u64
        lib.ref_io_to_csv.argtypes = [vp, vp, C.c_int, u64, vp, u64]
        _ref_io = lib
    return _ref_io


_host = None


def host_lib():
    """The product's host library (lib/libkmeans_host.so, km_host.h)."""
    global _host
    if _host is None:
        so = PKG / "lib" / "libkmeans_host.so"
        if not so.exists():
            km().lib()   # raises with the build hint when nothing is built
        lib = C.CDLL(str(so))
        vp, u64, u32, i32 = C.c_void_p, C.c_uint64, C.c_uint32, C.c_int32
        lib.kmh_read_points.restype = C.c_int
        lib.kmh_read_points.argtypes = [C.c_char_p, u32, u64, i32, vp, C.POINTER(u64)]
        lib.kmh_parse_points.restype = C.c_int
        lib.kmh_parse_points.argtypes = [C.c_char_p, u64, i32, u32, u64, i32, vp, C.POINTER(u64)]
        lib.kmh_random_points.restype = C.c_int
        lib.kmh_random_points.argtypes = [i32, u32, u64, vp]
        lib.kmh_write_csv.restype = C.c_int
        lib.kmh_write_csv.argtypes = [C.c_char_p, vp, vp, u32, u64]
        _host = lib
    return _host


def gpukmeans_bin():
    return PKG / "lib" / "gpukmeans"


def read_reference_csv(path, d):
    """The reference's CSV reader semantics (src/include/input_parser.hpp:103-131):
    header skipped, column 0 dropped, the next d columns read, missing -> 0."""
    rows = Path(path).read_text().strip().split("\n")[1:]
    X = np.zeros((len(rows), d), np.float32)
    for i, r in enumerate(rows):
        toks = r.split(",")[1:1 + d]
        X[i, :len(toks)] = [float(t) for t in toks]
    return X


# ---------------------------------------------------------------------------
# numpy twin of km_synth_blobs (matrix-centric-k-means_gb300/csrc/km_synth.cpp)
# ---------------------------------------------------------------------------
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_G = np.uint64(0x9E3779B97F4A7C15)
_MASK = (1 << 64) - 1


def _mix64(z):
    with np.errstate(over="ignore"):
        z = z ^ (z >> np.uint64(30))
        z = z * _M1
        z = z ^ (z >> np.uint64(27))
        z = z * _M2
        return z ^ (z >> np.uint64(31))


def _stream_key(seed, stream):
    v = (seed * 0x9E3779B97F4A7C15 + stream * 0xD1B54A32D192ED03 + 0x632BE59BD9B4E019) & _MASK
    return _mix64(np.array([v], np.uint64))[0]


def _uniform(key, idx):
    with np.errstate(over="ignore"):
        z = _mix64(key + (idx.astype(np.uint64) + np.uint64(1)) * _G)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def synth_blobs_np(n, d, blobs, lo, hi, sigma, seed, round_clip=False):
    k0, k1, k2 = (_stream_key(seed, s) for s in range(3))
    center = lo + (hi - lo) * _uniform(k0, np.arange(blobs * d, dtype=np.uint64))
    center = center.reshape(blobs, d)
    b = (_uniform(k1, np.arange(n, dtype=np.uint64)) * blobs).astype(np.int64)
    b = np.minimum(b, blobs - 1)
    idx = np.arange(n * d, dtype=np.uint64) * np.uint64(4)
    s = _uniform(k2, idx)
    s = s + _uniform(k2, idx + np.uint64(1))
    s = s + _uniform(k2, idx + np.uint64(2))
    s = s + _uniform(k2, idx + np.uint64(3))
    z = ((s - 2.0) * np.sqrt(3.0)).reshape(n, d)
    v = center[b] + sigma * z
    if round_clip:
        v = np.minimum(hi, np.maximum(lo, np.rint(v))) + 0.0  # -0 -> +0
    return v.astype(np.float32), b.astype(np.uint32)


def synth_blobs_np_chunked(n, d, blobs, lo, hi, sigma, seed, rows_per_chunk=65536):
    """synth_blobs_np for large n, generated in row chunks (same values: every
    draw is indexed by its global row and column)."""
    k0, k1, k2 = (_stream_key(seed, s) for s in range(3))
    center = (lo + (hi - lo) * _uniform(k0, np.arange(blobs * d, dtype=np.uint64))).reshape(blobs, d)
    out = np.empty((n, d), np.float32)
    lab = np.empty(n, np.uint32)
    for r0 in range(0, n, rows_per_chunk):
        r1 = min(n, r0 + rows_per_chunk)
        b = (_uniform(k1, np.arange(r0, r1, dtype=np.uint64)) * blobs).astype(np.int64)
        b = np.minimum(b, blobs - 1)
        idx = np.arange(r0 * d, r1 * d, dtype=np.uint64) * np.uint64(4)
        s = _uniform(k2, idx)
        s = s + _uniform(k2, idx + np.uint64(1))
        s = s + _uniform(k2, idx + np.uint64(2))
        s = s + _uniform(k2, idx + np.uint64(3))
        z = ((s - 2.0) * np.sqrt(3.0)).reshape(r1 - r0, d)
        out[r0:r1] = (center[b] + sigma * z).astype(np.float32)
        lab[r0:r1] = b
    return out, lab


def batch_problems(count=512, seed=4000):
    """Shapes of the batched workload: n log-uniform in [1024, 65536], d in
    {2, 8, 16, 32, 64, 128, 256}, k uniform in [2, 128] (k < n)."""
    rng = np.random.default_rng(seed)
    shapes = []
    for _ in range(count):
        n = int(np.exp(rng.uniform(np.log(1024), np.log(65536))))
        d = int(rng.choice([2, 8, 16, 32, 64, 128, 256]))
        k = min(int(rng.integers(2, 129)), n - 1)
        shapes.append((n, d, k))
    return shapes


def batch_points(shapes, seed=4000, nthreads=8):
    """Points of the batched workload: problem p is one seeded Gaussian blob
    per cluster (sigma 1, centers U[-5,5]^d), seed + p."""
    return [km().synth_blobs(n, d, k, -5.0, 5.0, 1.0, seed + p, nthreads=nthreads)
            for p, (n, d, k) in enumerate(shapes)]


def config1_data(seed=0):
    """Plain Lloyd workload: n=1797, d=64, k=10 blobs, centers U[0,16]^64,
    sigma=3, rounded and clipped to [0,16] (integer-valued floats)."""
    X, _ = synth_blobs_np(1797, 64, 10, 0.0, 16.0, 3.0, seed, round_clip=True)
    return X
