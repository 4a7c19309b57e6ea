"""The gpukmeans reader, writer and seeded random data (include/input_parser.hpp
through km_host.h) against the reference's own InputParser
(src/include/input_parser.hpp, built from the reference tree into oracle/_ref),
and the CLI's argument handling and exit codes.  No GPU needed."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import helpers


def ours_parse(text: bytes, svm: bool, d: int, n: int, plain=False):
    out = np.full((n, d), np.nan, np.float32)
    rows = C.c_uint64(0)
    rc = helpers.host_lib().kmh_parse_points(text, len(text), int(svm), d, n, int(plain), out.ctypes.data,
                                             C.byref(rows))
    assert rc == 0
    return out, rows.value


def ref_parse(text: bytes, svm: bool, d: int, n: int):
    lib = helpers.reference_io_lib()
    if lib is None:
        pytest.skip("reference tree absent")
    out = np.full((n, d), np.nan, np.float32)
    lib.ref_io_read(text, len(text), int(svm), d, n, out.ctypes.data)
    return out


def csv_text(rows, header="id,a,b,c"):
    return (header + "\n" + "\n".join(rows) + "\n").encode()


CSV_CASES = {
    "plain": (["0,1.5,2,3", "1,-4,5e-3,6", "2,7,8,9.25"], 3),
    "label_last": (["5,1,2,0", "6,3,4,1"], 3),
    "short_rows": (["0,1", "1,2,3", "2,,4,5"], 3),
    "empty_line": (["0,1,2,3", "", "2,4,5,6"], 3),
    "crlf": (["0,1,2,3\r", "1,4,5,6\r"], 3),
    "spaces_exponents": (["0, 1.0e+1 ,  -2.5E-2,3", "1,0.1,0.2,0.30000001"], 3),
    "rounding": (["0,0.1,16777217,3.4028235e38", "1,1e-45,-0,1.00000005960464477539"], 3),
    "hex_inf_words": (["0,0x1A,abc,12abc", "1,+5,.5,5."], 3),
}


@pytest.mark.parametrize("case", sorted(CSV_CASES))
def test_csv_reader_matches_reference(case):
    rows, d = CSV_CASES[case]
    text = csv_text(rows)
    n = len(rows)
    ref = ref_parse(text, False, d, n)
    ours, got = ours_parse(text, False, d, n)
    assert got == n
    np.testing.assert_array_equal(ours.view(np.uint32), ref.view(np.uint32))


def test_csv_reader_on_reference_dataset():
    path = helpers.REFERENCE / "datasets" / "N1797_D64_digits-sklearn.csv"
    if not path.exists():
        pytest.skip("reference tree absent")
    text = path.read_bytes()
    ref = ref_parse(text, False, 64, 1797)
    ours, got = ours_parse(text, False, 64, 1797)
    assert got == 1797
    np.testing.assert_array_equal(ours.view(np.uint32), ref.view(np.uint32))
    # through the file entry point as well
    out = np.empty((1797, 64), np.float32)
    rows = C.c_uint64(0)
    assert helpers.host_lib().kmh_read_points(str(path).encode(), 64, 1797, 0, out.ctypes.data, C.byref(rows)) == 0
    np.testing.assert_array_equal(out, ours)


def test_csv_reader_bounds_and_plain_mode():
    text = csv_text(["0,1,2,3,4,5", "1,6,7,8,9,10", "2,1,1,1,1,1"])
    ours, got = ours_parse(text, False, 3, 2)            # more rows and columns than asked
    assert got == 2
    np.testing.assert_array_equal(ours, [[1, 2, 3], [6, 7, 8]])
    plain, _ = ours_parse(text, False, 3, 2, plain=True)
    np.testing.assert_array_equal(plain, [[0, 1, 2], [1, 6, 7]])
    few, got = ours_parse(csv_text(["0,1,2,3"]), False, 3, 4)
    assert got == 1                                       # the CLI reports this as exit 4


def test_svm_reader_matches_reference():
    lines = ["1 1:0.5 3:2", "0 2:-1.25 4:7e2", "1", "3 1:1 2:2 3:3 4:4"]
    text = ("\n".join(lines) + "\n").encode()
    ref = ref_parse(text, True, 4, 4)
    ours, got = ours_parse(text, True, 4, 4)
    assert got == 4
    np.testing.assert_array_equal(ours.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("seed,d,n", [(0, 3, 10), (7, 64, 1000), (-5, 1, 17)])
def test_random_points_match_reference(seed, d, n):
    lib = helpers.reference_io_lib()
    if lib is None:
        pytest.skip("reference tree absent")
    ref = np.empty((n, d), np.float32)
    lib.ref_io_random(seed, d, n, ref.ctypes.data)
    ours = np.empty((n, d), np.float32)
    assert helpers.host_lib().kmh_random_points(seed, d, n, ours.ctypes.data) == 0
    np.testing.assert_array_equal(ours.view(np.uint32), ref.view(np.uint32))


def test_csv_writer_matches_reference(tmp_path):
    lib = helpers.reference_io_lib()
    if lib is None:
        pytest.skip("reference tree absent")
    rng = np.random.default_rng(3)
    n, d = 40000, 5         # more than one parallel block of rows
    X = (rng.standard_normal((n, d)) * np.array([1e-7, 1, 1e3, 1e7, 1e30])).astype(np.float32)
    X[0] = [0.1, -0.0, 16777217, 1 / 3, 123456789]
    X[1] = np.arange(5)
    lab = rng.integers(0, 1000, n).astype(np.uint32)
    cap = 64 * n * (d + 1) + 1000
    buf = C.create_string_buffer(cap)
    m = lib.ref_io_to_csv(X.ctypes.data, lab.ctypes.data, d, n, buf, cap)
    ref = buf.raw[:m]
    path = tmp_path / "out.csv"
    assert helpers.host_lib().kmh_write_csv(str(path).encode(), X.ctypes.data, lab.ctypes.data, d, n) == 0
    assert path.read_bytes() == ref


# ---------------------------------------------------------------------------
# CLI argument handling (no GPU needed up to the device check)
# ---------------------------------------------------------------------------
def run_cli(*args, cwd=None):
    exe = helpers.gpukmeans_bin()
    if not exe.exists():
        helpers.km().lib()
        pytest.skip("gpukmeans not built")
    return subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, cwd=cwd, timeout=120)


BASE = ["-n", "100", "-d", "3", "-k", "4", "-m", "10", "-b", "random", "-f", "linear", "-l", "3"]


def test_cli_help():
    r = run_cli("-h")
    assert r.returncode == 0 and "--n-samples" in r.stdout


@pytest.mark.parametrize("drop", ["-n", "-d", "-k", "-m", "-b", "-f", "-l"])
def test_cli_missing_required_argument(drop):
    args = list(BASE)
    i = args.index(drop)
    del args[i:i + 2]
    r = run_cli(*args)
    assert r.returncode == 1
    assert "Invalid or missing argument" in r.stderr


def test_cli_bad_values_and_unknown_option():
    assert run_cli(*BASE, "--bogus", "1").returncode == 1
    args = list(BASE)
    args[args.index("-n") + 1] = "abc"
    assert run_cli(*args).returncode == 1
    args = list(BASE)
    args[args.index("-k") + 1] = "0"
    assert run_cli(*args).returncode == 1


def test_cli_precision_values():
    """-p takes auto (the default), fp32, bf16 or bf16x3; anything else is an
    argument error (exit 1) before the device is touched."""
    r = run_cli(*BASE, "-p", "fp16")
    assert r.returncode == 1 and "Invalid or missing argument" in r.stderr
    if helpers.km().device_count() == 0:
        for prec in ("auto", "fp32", "bf16", "bf16x3"):
            assert run_cli(*BASE, "-p", prec).returncode == 2        # parsed; no device here


def test_cli_invalid_input_file(tmp_path):
    r = run_cli(*BASE, "-i", tmp_path / "missing.csv")
    assert r.returncode == 4 and "Invalid input file" in r.stderr
    (tmp_path / "x.txt").write_text("a,b\n1,2\n")
    assert run_cli(*BASE, "-i", tmp_path / "x.txt").returncode == 4
    (tmp_path / "short.csv").write_text("h,a,b,c\n0,1,2,3\n")     # 1 row for -n 100
    assert run_cli(*BASE, "-i", tmp_path / "short.csv").returncode == 4


def test_cli_long_and_attached_forms_reach_device_check():
    if helpers.km().device_count() > 0:
        pytest.skip("a GPU is present: the run itself is covered by the GPU tests")
    r = run_cli("--n-samples=100", "-d3", "--n-clusters", "4", "-m", "10", "--init=random", "-f", "linear",
                "-l", "3", "-s", "1")
    assert r.returncode == 2
    assert "no available device" in r.stderr
