"""ORACLE — test infrastructure only (tests/ and bench.py's parity legs; never
loaded by the product library).

One iteration of the reference GPU path's kernel k-means in FP64, from given
labels, for n where the n x n kernel matrix does not fit host memory as FP64
(n = 65,536 is 34 GB): K is formed one row block at a time from the points
and folded straight into E = K V^T.  Semantics as oracle/km_oracle.cpp's
orc_kernel_kmeans, which restates
  src/kernels/kernels.cuh:43-118      kernel functions (stored without the -2)
  src/kernels/distances.cu:895-1002   D[i,c] = -2/|c| sum_{j in c} K_ij + ctilde_c,
                                      ctilde_c = (1/|c|^2) sum_{a,b in c} K_ab
  src/kernels/distances.cu:588-599    ctilde_c == 0 -> +inf (empty cluster)
  src/kmeans.cu:923-936               argmin from (0, FLT_MAX), lowest index on ties
  src/kmeans.cu:1054-1061             score = sum_i D[i, label_i] (K_ii left out)
plus the Gaussian kernel exp(-||x-y||^2 / (2 sigma^2)).
"""
from __future__ import annotations

import concurrent.futures as cf
import os

import numpy as np

FLT_MAX = float(np.finfo(np.float32).max)
KINDS = {"linear": 0, "polynomial": 1, "sigmoid": 2, "gaussian": 3}


def _kernel_rows(X64, nrm, b0, b1, kind, gamma, coef, degree, sigma):
    """K[b0:b1, :] in FP64, computed in place over the Gram block."""
    G = X64[b0:b1] @ X64.T
    if kind == 0:
        return G
    if kind == 1:
        G *= gamma
        G += coef
        return np.power(G, degree, out=G)
    if kind == 2:
        G *= gamma
        G += coef
        return np.tanh(G, out=G)
    G *= -2.0
    G += nrm[b0:b1, None]
    G += nrm[None, :]
    np.maximum(G, 0.0, out=G)
    G *= -1.0 / (2.0 * sigma * sigma)
    return np.exp(G, out=G)


def kernel_diag(X, kind, gamma=1.0, coef=1.0, degree=2, sigma=1.0):
    """K_ii in FP64."""
    X64 = np.asarray(X, np.float64)
    nrm = np.einsum("ij,ij->i", X64, X64)
    kind = KINDS.get(kind, kind)
    if kind == 0:
        return nrm
    if kind == 1:
        return (gamma * nrm + coef) ** degree
    if kind == 2:
        return np.tanh(gamma * nrm + coef)
    return np.ones_like(nrm)


def kkm_step_f64(X, labels, k, kind, gamma=1.0, coef=1.0, degree=2, sigma=1.0, block=1024, workers=None):
    """One kernel k-means iteration in FP64 from `labels` (n, values < k).
    Returns (new labels as uint32, score = sum_i D[i, new_label_i])."""
    X64 = np.ascontiguousarray(X, np.float64)
    n = X64.shape[0]
    kind = KINDS.get(kind, kind)
    labels = np.asarray(labels).astype(np.int64)
    nrm = np.einsum("ij,ij->i", X64, X64)
    cnt = np.bincount(labels, minlength=k).astype(np.float64)
    V = np.zeros((n, k), np.float64)
    V[np.arange(n), labels] = 1.0
    E = np.empty((n, k), np.float64)

    def work(b0):
        b1 = min(n, b0 + block)
        E[b0:b1] = _kernel_rows(X64, nrm, b0, b1, kind, gamma, coef, degree, sigma) @ V

    workers = workers or max(1, min(8, (os.cpu_count() or 4) // 2))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        list(ex.map(work, range(0, n, block)))
    ct = np.zeros(k, np.float64)
    np.add.at(ct, labels, E[np.arange(n), labels])
    with np.errstate(divide="ignore", invalid="ignore"):
        ct = np.where(cnt > 0, ct / (cnt * cnt), 0.0)
        add = np.where(ct == 0.0, np.inf, ct)
        D = np.where(cnt > 0, -2.0 * E / np.maximum(cnt, 1.0), 0.0) + add
    D = np.minimum(D, FLT_MAX)              # the argmin starts from (0, FLT_MAX)
    new = np.argmin(D, axis=1)               # first index of the minimum: lowest index on ties
    score = float(D[np.arange(n), new].sum())
    return new.astype(np.uint32), score
