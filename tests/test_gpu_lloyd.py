"""GPU parity of the Lloyd path (through the C ABI of libkm_sm103) against the
golden fixtures made by the reference's own CPU k-means and against the
oracle.  Labels and iteration counts must be identical in every precision:
rows whose fast-path margin is inside the error bound are re-scored with the
reference formula.  Objective: within 1e-5 relative of the FP64 oracle's
objective for the same assignment."""
import json
from pathlib import Path

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
CASES = json.loads((GOLD / "lloyd_cases.json").read_text())
LABELS = np.load(GOLD / "lloyd_labels.npz")
PRECISIONS = ["fp32", "bf16", "bf16x3"]
OBJ_RTOL = 1e-5


def case_data(c):
    from golden.make_golden import x_hash
    X, _ = helpers.synth_blobs_np(c["n"], c["d"], c["blobs"], c["lo"], c["hi"], c["sigma"],
                                  c["data_seed"], round_clip=c["round_clip"])
    assert x_hash(X) == c["x_sha256"], "generator drift"
    return X


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_lloyd_matches_reference_golden(km, gpu, c, prec):
    X = case_data(c)
    m = km.Lloyd(c["n"], c["d"], c["k"], tol=c["tol"], seed=c["seed"], maxiter=c["maxiter"],
                 precision=prec).set_data(X)
    lab, cen, r = m.fit()
    m.close()
    np.testing.assert_array_equal(lab, LABELS[c["name"]].astype(np.uint32))
    assert r.converged_iter == c["ref_iter"]
    # objective of the last assignment against the centroids that produced it:
    # recompute with the oracle from the final labels and the previous centroids
    it_o, lab_o, cen_o, ex_o = helpers.orc_lloyd(X, c["k"], c["tol"], c["seed"], c["maxiter"])
    np.testing.assert_array_equal(cen.view(np.uint32), cen_o.view(np.uint32))
    assert r.iterations == ex_o


@pytest.mark.parametrize("prec", PRECISIONS)
def test_lloyd_objective_fp64(km, gpu, prec):
    X, _ = helpers.synth_blobs_np(30000, 32, 24, -5, 5, 1.0, 41)
    k, maxiter = 24, 4
    m = km.Lloyd(30000, 32, k, tol=0.0, seed=4, maxiter=maxiter, precision=prec, conv="none").set_data(X)
    lab, cen, r = m.fit()
    m.close()
    # centroids before the last update: run the oracle maxiter-1 iterations
    _, _, cprev, _ = helpers.orc_lloyd(X, k, -1.0, 4, maxiter - 1)
    obj = helpers.orc_inertia(X, lab, cprev)
    assert abs(r.objective - obj) <= OBJ_RTOL * obj
    sx = float((X.astype(np.float64) ** 2).sum())
    assert abs(r.score - (obj - sx)) <= OBJ_RTOL * obj
    assert r.iterations == maxiter and r.converged_iter == maxiter


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("shape", [(1000, 1, 3), (129, 7, 129), (5000, 65, 100), (3333, 250, 17),
                                   (2048, 130, 256), (10007, 12, 2), (20000, 64, 300), (8000, 200, 777),
                                   (5000, 16, 2000), (6000, 256, 4096)])
def test_assign_exact_vs_oracle(km, gpu, prec, shape):
    import torch
    n, d, k = shape
    rng = np.random.default_rng(n + d + k)
    X = rng.standard_normal((n, d)).astype(np.float32) * 4
    Cc = X[rng.choice(n, k, replace=False)].copy()
    Cc[k // 2] = Cc[0]                      # duplicate centroid: exact ties, lowest index must win
    lab_o, md_o = helpers.orc_assign(X, Cc)
    Xt = torch.from_numpy(X).to(gpu)
    Ct = torch.from_numpy(Cc).to(gpu)
    lab, md, refined = km.assign(Xt, Ct, precision=prec, want_mindist=True)
    np.testing.assert_array_equal(lab.cpu().numpy().astype(np.uint32), lab_o)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_assign_near_ties(km, gpu, prec):
    """Points placed (almost) equidistant between centroid pairs force the
    refinement path; labels must still equal the reference formula's."""
    import torch
    rng = np.random.default_rng(7)
    k, d, n = 40, 24, 20000
    Cc = rng.standard_normal((k, d)).astype(np.float32) * 3
    a = rng.integers(0, k, n)
    b = (a + 1 + rng.integers(0, k - 1, n)) % k
    t = (0.5 + rng.standard_normal(n) * 1e-4)[:, None]
    X = (Cc[a] * t + Cc[b] * (1 - t)).astype(np.float32)
    X[: n // 4] = np.round(X[: n // 4] * 4) / 4
    lab_o, _ = helpers.orc_assign(X, Cc)
    lab, _, refined = km.assign(torch.from_numpy(X).to(gpu), torch.from_numpy(Cc).to(gpu), precision=prec)
    np.testing.assert_array_equal(lab.cpu().numpy().astype(np.uint32), lab_o)
    assert refined > 0


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("d", [4, 100, 132, 260])
def test_assign_dense_queue_shapes(km, gpu, prec, d):
    """Centroids in groups of 2..6 near-duplicates and points at the groups'
    centres: almost every row is queued, many with 3..4 candidates (the staged
    re-score's passes hit their row and pair limits) and the groups of 5..6
    send rows to the full re-score.  d = 4, 100, 132, 260 cover a chunk of
    fewer than 128 columns, a padded shared-memory row stride, and two or
    three 128-column chunks per pass.  Labels must equal the reference
    formula's."""
    import torch
    rng = np.random.default_rng(11 + d)
    sizes = [2, 3, 4, 5, 6, 2, 3, 4, 6, 5, 2, 4]
    base = rng.standard_normal((len(sizes), d)).astype(np.float32) * 4
    cs, owner = [], []
    for g, m in enumerate(sizes):
        for _ in range(m):
            cs.append(base[g] + rng.standard_normal(d).astype(np.float32) * 1e-5)
            owner.append(g)
    Cc = np.stack(cs).astype(np.float32)
    n = 9000
    grp = rng.integers(0, len(sizes), n)
    X = (base[grp] + rng.standard_normal((n, d)).astype(np.float32) * 1e-3).astype(np.float32)
    lab_o, _ = helpers.orc_assign(X, Cc)
    lab, _, refined = km.assign(torch.from_numpy(X).to(gpu), torch.from_numpy(Cc).to(gpu), precision=prec)
    np.testing.assert_array_equal(lab.cpu().numpy().astype(np.uint32), lab_o)
    assert refined > n // 2


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("shape", [(3000, 96, 200), (2000, 64, 700)])
def test_distances_vs_torch_fp32(km, gpu, prec, shape):
    """The fast-path distance stage against a plain PyTorch fp32 reference
    (FP64 for the comparison); tolerance = the bound the refinement uses.
    k = 700 runs the chunked tensor-core kernel."""
    import torch
    n, d, k = shape
    rng = np.random.default_rng(3)
    X = torch.from_numpy(rng.standard_normal((n, d)).astype(np.float32) * 2).to(gpu)
    Cc = torch.from_numpy(rng.standard_normal((k, d)).astype(np.float32) * 2).to(gpu)
    D = km.distances(X, Cc, precision=prec)
    torch.backends.cuda.matmul.allow_tf32 = False
    ref32 = (X * X).sum(1)[:, None] + (Cc * Cc).sum(1)[None] - 2.0 * (X @ Cc.T)
    ref = ((X.double()[:, None, :] - Cc.double()[None]) ** 2).sum(-1)
    nx = X.double().norm(dim=1)[:, None]
    nc = Cc.double().norm(dim=1)[None]
    u, ub, uacc = 2.0 ** -24, 2.0 ** -8, 2.0 ** -22
    eps = {"fp32": d * u, "bf16": 2 * ub + ub * ub + d * uacc, "bf16x3": 3.5 * ub * ub + 3 * d * uacc}[prec]
    # error envelope of the fast path (the bound the refinement relies on),
    # plus the rounding of the ||x||^2 term added for this probe
    tol = (2.02 * eps + 2.1 * u) * nx * nc + 2.1 * u * nc * nc + 4 * u * (nx ** 2 + nc ** 2)
    err = (D.double() - ref).abs()
    assert bool((err <= tol).all()), float((err / tol).max())
    # against the plain torch fp32 expansion: both sit inside the envelope
    tol32 = tol + (2.02 * d * u + 2.1 * u) * nx * nc + 4 * u * (nx ** 2 + nc ** 2)
    assert bool(((D.double() - ref32.double()).abs() <= tol32).all())


def test_update_exact_vs_oracle(km, gpu):
    import torch
    rng = np.random.default_rng(11)
    n, d, k = 50000, 37, 300
    X = (rng.standard_normal((n, d)) * 10).astype(np.float32)
    lab = rng.integers(0, k - 5, n).astype(np.uint32)        # clusters k-5.. stay empty
    C_o, cnt_o = helpers.orc_update(X, lab, k)
    Ct, cnt, perm, off = km.update(torch.from_numpy(X).to(gpu), torch.from_numpy(lab.astype(np.int32)).to(gpu), k)
    np.testing.assert_array_equal(Ct.cpu().numpy().view(np.uint32), C_o.view(np.uint32))
    np.testing.assert_array_equal(cnt.cpu().numpy().astype(np.uint32), cnt_o)
    p = perm.cpu().numpy()
    np.testing.assert_array_equal(p, np.argsort(lab, kind="stable"))
    np.testing.assert_array_equal(off.cpu().numpy()[:-1], np.concatenate([[0], np.cumsum(cnt_o)[:-1]]))


def test_update_rejects_bad_labels(km, gpu):
    import torch
    X = torch.zeros((100, 4), device=gpu)
    lab = torch.full((100,), 7, dtype=torch.int32, device=gpu)
    with pytest.raises(km.KmError) as e:
        km.update(X, lab, 5)
    assert e.value.status == km.KM_ERR_ARG


@pytest.mark.parametrize("prec", PRECISIONS)
def test_round_robin_init_score_rule(km, gpu, prec):
    """Reference GPU semantics: labels i % k, stop on |score - last| < tol."""
    X, _ = helpers.synth_blobs_np(8000, 10, 6, -4, 4, 1.0, 23)
    n, d, k = 8000, 10, 6
    lab0 = (np.arange(n) % k).astype(np.uint32)
    C0, _ = helpers.orc_update(X, lab0, k)
    m = km.Lloyd(n, d, k, tol=1e-3, maxiter=40, init="round_robin", precision=prec, conv="score").set_data(X)
    lab, cen, r = m.fit()
    m.close()
    it_o, lab_o, cen_o, ex_o = helpers.orc_lloyd(X, k, -1.0, 0, r.iterations, C0=C0)
    np.testing.assert_array_equal(lab, lab_o)
    assert r.converged_iter <= 40


def test_determinism_and_repeat_fit(km, gpu):
    X, _ = helpers.synth_blobs_np(40000, 20, 30, -5, 5, 1.0, 31)
    m = km.Lloyd(40000, 20, 30, tol=1e-4, seed=3, maxiter=50, precision="bf16").set_data(X)
    a = m.fit()
    b = m.fit()
    m.close()
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
    assert a[2].objective == b[2].objective and a[2].converged_iter == b[2].converged_iter


def test_profile_between_fits(km, gpu):
    """The per-stage timer runs iterations on the handle's state; a fit after
    it starts again from the seeded initialisation and matches the first fit
    (the device-side loop state, including the finalize ticket, is reset)."""
    X, _ = helpers.synth_blobs_np(30000, 16, 20, -5, 5, 1.0, 7)
    m = km.Lloyd(30000, 16, 20, tol=1e-4, seed=2, maxiter=30, precision="bf16x3").set_data(X)
    a = m.fit()
    st = m.profile(3)
    b = m.fit()
    m.close()
    assert len(st) == 5 and all(v > 0 for v in st)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
    assert a[2].objective == b[2].objective and a[2].iterations == b[2].iterations


def test_device_input_and_nonfinite_rejection(km, gpu):
    import torch
    X, _ = helpers.synth_blobs_np(5000, 8, 4, -3, 3, 1.0, 2)
    Xt = torch.from_numpy(X).to(gpu)
    m = km.Lloyd(5000, 8, 4, tol=1e-4, seed=1, maxiter=30).set_data(Xt)
    lab, cen, r = m.fit()
    it_o, lab_o, _, _ = helpers.orc_lloyd(X, 4, 1e-4, 1, 30)
    np.testing.assert_array_equal(lab, lab_o)
    assert r.converged_iter == it_o
    X[17, 3] = np.nan
    with pytest.raises(km.KmError) as e:
        m.set_data(X)
    assert e.value.status == km.KM_ERR_ARG
    m.close()


def test_too_few_distinct_points(km, gpu):
    X = np.zeros((100, 3), np.float32)
    X[:50] = 1.0
    m = km.Lloyd(100, 3, 3, maxiter=5).set_data(X)
    with pytest.raises(km.KmError) as e:
        m.fit()
    assert e.value.status == km.KM_ERR_ARG
    m.close()


def test_k_equals_n(km, gpu):
    rng = np.random.default_rng(5)
    X = rng.standard_normal((300, 5)).astype(np.float32)
    m = km.Lloyd(300, 5, 300, tol=1e-4, seed=2, maxiter=10).set_data(X)
    lab, cen, r = m.fit()
    m.close()
    it_o, lab_o, _, _ = helpers.orc_lloyd(X, 300, 1e-4, 2, 10)
    np.testing.assert_array_equal(lab, lab_o)
    assert r.converged_iter == it_o
