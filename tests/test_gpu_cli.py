"""gpukmeans end to end on the GPU: the reference's flags, CSV in and out,
stdout lines, and the Kmeans class semantics of the reference GPU path
(labels i % k, |score - last| < tol from the second iteration with -c 1,
score without sum ||x||^2, empty clusters never chosen again), checked
against the FP64 oracle of that algorithm (orc_kernel_kmeans on K = f(X X^T),
the popcorn distance of src/kernels/distances.cu:895-1002)."""
import ctypes as C
import re
import subprocess

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


def write_csv(path, X):
    """CSV as the reference reads it: a header, then an id column that the
    reader drops, then the d coordinates."""
    n, d = X.shape
    with open(path, "w") as f:
        f.write("id," + ",".join(f"f{j}" for j in range(d)) + "\n")
        for i in range(n):
            f.write(str(i) + "," + ",".join(repr(float(v)) for v in X[i]) + "\n")


def run_cli(*args):
    exe = helpers.gpukmeans_bin()
    assert exe.exists(), "gpukmeans not built"
    r = subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def parse_stdout(out, runs):
    conv = []
    for line in out.splitlines():
        m = re.search(r"converged at iteration (\d+) -", line)
        if m:
            conv.append(int(m.group(1)))
        elif "did NOT converge" in line:
            conv.append(None)
    assert len(conv) == runs, out
    score = float(re.search(r"Score: (-?\d+\.\d+)", out).group(1))
    assert re.search(r"GPU_Kmeans: \S+s \(%d runs\)" % runs, out)
    assert re.search(r"MEMORY FOOTPRINT: \d+ MB", out)
    return conv, score


def read_out_csv(path, d):
    lines = open(path).read().splitlines()
    assert lines[0] == "cluster," + ",".join(f"d{j}" for j in range(d))
    rows = [l.split(",") for l in lines[1:]]
    lab = np.array([int(r[0]) for r in rows], np.uint32)
    X = np.array([[float(v) for v in r[1:]] for r in rows], np.float32)
    return lab, X


def oracle_popcorn(X, kind, k, maxiter, tol, check):
    X = np.ascontiguousarray(X, np.float32)
    n, d = X.shape
    K = np.empty((n, n))
    kid = {"linear": 0, "polynomial": 1, "sigmoid": 2}[kind]
    helpers.oracle().orc_kernel_matrix(X.ctypes.data, n, d, kid, 1.0, 1.0, 2, 1.0, 8, K.ctypes.data)
    lab = (np.arange(n) % k).astype(np.uint32)
    sc, ex = C.c_double(0), C.c_uint64(0)
    it = helpers.oracle().orc_kernel_kmeans(K.ctypes.data, n, k, maxiter, tol, int(check), 8, lab.ctypes.data,
                                            C.byref(sc), C.byref(ex))
    return int(it), lab, sc.value


@pytest.mark.parametrize("prec", ["fp32", "bf16", "bf16x3", "auto"])
def test_cli_linear_matches_reference_gpu_semantics(tmp_path, gpu, prec):
    X = helpers.config1_data()
    n, d = X.shape
    k, maxiter, tol = 10, 300, 1e-4
    write_csv(tmp_path / "in.csv", X)
    out = run_cli("-n", n, "-d", d, "-k", k, "-m", maxiter, "-t", tol, "-c", 1, "-b", "random", "-f", "linear",
                  "-l", 3, "-r", 2, "-s", 0, "-p", prec, "-i", tmp_path / "in.csv", "-o", tmp_path / "out.csv")
    conv, score = parse_stdout(out, 2)
    it_o, lab_o, sc_o = oracle_popcorn(X, "linear", k, maxiter, tol, True)
    lab, Xo = read_out_csv(tmp_path / "out.csv", d)
    np.testing.assert_array_equal(Xo, X)
    np.testing.assert_array_equal(lab, lab_o)
    assert conv[0] == conv[1] == (it_o if it_o < maxiter else None)
    assert abs(score - sc_o) <= 1e-6 * abs(sc_o) + 1e-3


def test_cli_linear_without_check_runs_maxiter(tmp_path, gpu):
    X = helpers.config1_data()
    n, d = X.shape
    write_csv(tmp_path / "in.csv", X)
    out = run_cli("-n", n, "-d", d, "-k", 10, "-m", 7, "-b", "random", "-f", "linear", "-l", 0, "-r", 2,
                  "-i", tmp_path / "in.csv", "-o", tmp_path / "out.csv")
    conv, _ = parse_stdout(out, 2)
    assert conv == [None, None]
    it_o, lab_o, _ = oracle_popcorn(X, "linear", 10, 7, 1e-4, False)
    lab, _ = read_out_csv(tmp_path / "out.csv", d)
    np.testing.assert_array_equal(lab, lab_o)


def test_cli_empty_clusters_stay_empty(tmp_path, gpu):
    """k close to the number of distinct points: clusters empty out, and the
    reference GPU rule keeps them out (+inf distance) where the CPU rule would
    park a zero centroid that can win points back."""
    rng = np.random.default_rng(5)
    X = np.repeat(rng.integers(-3, 4, (12, 4)).astype(np.float32), 40, axis=0)
    X = X[rng.permutation(len(X))]
    n, d = X.shape
    k = 24
    write_csv(tmp_path / "in.csv", X)
    out = run_cli("-n", n, "-d", d, "-k", k, "-m", 30, "-t", 1e-4, "-c", 1, "-b", "random", "-f", "linear",
                  "-l", 3, "-r", 2, "-i", tmp_path / "in.csv", "-o", tmp_path / "out.csv")
    conv, score = parse_stdout(out, 2)
    it_o, lab_o, sc_o = oracle_popcorn(X, "linear", k, 30, 1e-4, True)
    lab, _ = read_out_csv(tmp_path / "out.csv", d)
    assert len(np.unique(lab_o)) < k           # the case does empty clusters
    np.testing.assert_array_equal(lab, lab_o)
    assert abs(score - sc_o) <= 1e-6 * abs(sc_o) + 1e-3


@pytest.mark.parametrize("kind", ["polynomial", "sigmoid"])
def test_cli_kernel_kmeans(tmp_path, gpu, kind):
    X, _ = helpers.synth_blobs_np(1200, 8, 5, -1, 1, 0.2, 11)
    X = X.astype(np.float32)
    n, d = X.shape
    k, maxiter = 5, 20
    write_csv(tmp_path / "in.csv", X)
    out = run_cli("-n", n, "-d", d, "-k", k, "-m", maxiter, "-t", 1e-4, "-c", 1, "-b", "random", "-f", kind,
                  "-l", 3, "-r", 2, "-i", tmp_path / "in.csv", "-o", tmp_path / "out.csv")
    conv, score = parse_stdout(out, 2)
    it_o, lab_o, sc_o = oracle_popcorn(X, kind, k, maxiter, 1e-4, True)
    lab, _ = read_out_csv(tmp_path / "out.csv", d)
    assert float((lab == lab_o).mean()) >= 0.999
    assert abs(score - sc_o) <= 1e-4 * abs(sc_o)


def test_cli_random_data_and_plusplus(gpu):
    out = run_cli("-n", 5000, "-d", 16, "-k", 8, "-m", 5, "-b", "random", "-f", "linear", "-l", 3, "-s", 3,
                  "-r", 2)
    parse_stdout(out, 2)
    out = run_cli("-n", 5000, "-d", 16, "-k", 8, "-m", 50, "-t", 1e-3, "-c", 1, "-b", "plusplus", "-f", "linear",
                  "-l", 3, "-s", 3, "-r", 2)
    conv, _ = parse_stdout(out, 2)
    assert conv[0] == conv[1]          # seeded: both runs identical
    exe = helpers.gpukmeans_bin()
    r = subprocess.run([str(exe), "-n", "100", "-d", "2", "-k", "3", "-m", "5", "-b", "plusplus", "-f",
                        "polynomial", "-l", "3"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 1 and "plus_plus" in r.stderr
