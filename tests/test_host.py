"""Host-side checks that need no GPU: the library loads and exports every
symbol include/km.h declares, argument validation and status strings, and the
synthetic generator equals its numpy twin bit for bit."""
import re
from pathlib import Path

import numpy as np
import pytest

import helpers

HEADER = helpers.ROOT / "include" / "km.h"


def declared_functions():
    src = HEADER.read_text()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(km_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(km):
    lib = km.lib()
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(km.SIGNATURES), "km.py signatures out of sync with km.h"


C_TYPES = {"uint64_t": "c_ulong", "uint32_t": "c_uint", "int32_t": "c_int", "float": "c_float",
           "double": "c_double", "void*": "c_void_p"}


def declared_structs():
    """{name: [(field, c type), ...]} of the plain structs km.h defines."""
    src = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    out = {}
    for name, body in re.findall(r"typedef struct (km_\w+) \{(.*?)\} \1;", src, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            m = re.match(r"(\w+\s*\*?)\s*(.+)", decl)
            ctype = m.group(1).replace(" ", "")
            for f in m.group(2).split(","):
                f = f.strip()
                if f.startswith("*"):
                    ctype, f = ctype + "*", f[1:].strip()
                fields.append((f, ctype))
        out[name] = fields
    return out


def test_ctypes_structures_match_the_header(km):
    """Every structure km.py passes through the ABI has the header's fields,
    in the header's order, with the same C types (a drift would shift fields
    silently), and the kernel k-means mode constants agree."""
    import ctypes as C
    pairs = {"km_lloyd_params": km.LloydParams, "km_result": km.Result, "km_kkm_params": km.KkmParams,
             "km_batch_problem": km.BatchProblem, "km_batch_params": km.BatchParams,
             "km_batch_result": km.BatchResult}
    structs = declared_structs()
    assert set(pairs) <= set(structs), set(pairs) - set(structs)
    for cname, py in pairs.items():
        want = structs[cname]
        got = [(f, t.__name__) for f, t in py._fields_]
        assert [f for f, _ in got] == [f for f, _ in want], cname
        for (f, t), (_, ct) in zip(got, want):
            exp = getattr(C, C_TYPES[ct]).__name__
            assert t == exp, (cname, f, t, ct)
    src = HEADER.read_text()
    assert "#define KM_KKM_PANEL_AUTO UINT64_MAX" in src and km.KKM_PANEL_AUTO == 2 ** 64 - 1
    assert "#define KM_KKM_FUSED (UINT64_MAX - 1)" in src and km.KKM_FUSED == 2 ** 64 - 2


def test_status_strings(km):
    lib = km.lib()
    for s in range(8):
        assert lib.km_status_str(s)
    assert b"sm_103a" in lib.km_version()


def test_argument_validation_without_device(km):
    import ctypes as C
    lib = km.lib()
    h = C.c_void_p()
    bad = [dict(n=10, d=2, k=11), dict(n=10, d=0, k=2), dict(n=0, d=2, k=1), dict(n=10, d=2, k=0)]
    for b in bad:
        p = km.LloydParams(b["n"], b["d"], b["k"], 1e-4, 0, 10, 0, 0, 0, 0, None)
        assert lib.km_lloyd_create(C.byref(p), C.byref(h)) == km.KM_ERR_ARG
    p = km.LloydParams(100, 2, 3, 1e-4, 0, 0, 0, 0, 0, 0, None)   # maxiter 0
    assert lib.km_lloyd_create(C.byref(p), C.byref(h)) == km.KM_ERR_ARG
    p = km.LloydParams(100, 2, 3, float("nan"), 0, 10, 0, 0, 0, 0, None)
    assert lib.km_lloyd_create(C.byref(p), C.byref(h)) == km.KM_ERR_ARG
    assert lib.km_lloyd_fit(None, None, None, None, None) == km.KM_ERR_ARG
    # kernel k-means, resident K and panels alike
    for pr in (0, 512, km.KKM_PANEL_AUTO):
        for n, d, k in ((10, 2, 11), (10, 0, 2), (0, 2, 1), (10, 2, 0)):
            kp = km.KkmParams(n, d, k, 1e-4, 10, 1, 1.0, 1.0, 1.0, 2, 0, 0, 0, 0, None, pr)
            assert lib.km_kkm_create(C.byref(kp), C.byref(h)) == km.KM_ERR_ARG
        kp = km.KkmParams(1000, 4, 300, 1e-4, 10, 1, 1.0, 1.0, 1.0, 2, 0, 0, 0, 0, None, pr)   # k > 256
        assert lib.km_kkm_create(C.byref(kp), C.byref(h)) == km.KM_ERR_UNSUPPORTED
    r = C.c_uint64(0)
    assert lib.km_kkm_panel_rows(None, C.byref(r)) == km.KM_ERR_ARG


def test_no_device_is_reported_not_faked(km):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import ctypes as C
    h = C.c_void_p()
    p = km.LloydParams(100, 2, 3, 1e-4, 0, 10, 0, 0, 0, 0, None)
    assert km.lib().km_lloyd_create(C.byref(p), C.byref(h)) == km.KM_ERR_NO_DEVICE
    assert km.device_count() == 0


@pytest.mark.parametrize("args", [
    (1797, 64, 10, 0.0, 16.0, 3.0, 0, True),
    (5000, 16, 7, -10.0, 10.0, 1.5, 3, False),
    (777, 3, 40, -5.0, 5.0, 1.0, 7, False),
])
def test_generator_matches_numpy_twin(km, args):
    n, d, blobs, lo, hi, sigma, seed, rc = args
    X_c, b_c = km.synth_blobs(n, d, blobs, lo, hi, sigma, seed, round_clip=rc, with_blob=True)
    X_n, b_n = helpers.synth_blobs_np(n, d, blobs, lo, hi, sigma, seed, round_clip=rc)
    np.testing.assert_array_equal(b_c, b_n)
    np.testing.assert_array_equal(X_c.view(np.uint32), X_n.view(np.uint32))


def test_generator_threads_do_not_change_bits(km):
    a = km.synth_blobs(50000, 8, 5, -1, 1, 0.5, 9, nthreads=1)
    b = km.synth_blobs(50000, 8, 5, -1, 1, 0.5, 9, nthreads=8)
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
