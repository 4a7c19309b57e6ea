"""Generates the golden fixtures in this folder from the reference itself.

Each case is a seeded synthetic input (tests/helpers.synth_blobs_np, the numpy
twin of the library's generator) run through the reference's own CPU k-means
(comparisons/CPU_Kmeans, built from the reference sources into oracle/_ref by
oracle/build_ref.sh).  The fixture stores the case parameters, a SHA-256 of
the generated input (so that generator drift is detected before any parity
claim) and the reference's labels and returned iteration.

    python tests/golden/make_golden.py        (needs the reference tree)
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
import helpers  # noqa: E402

# name, n, d, blobs, lo, hi, sigma, round_clip, data_seed, k, tol, kmeans_seed, maxiter
CASES = [
    ("config1_s0", 1797, 64, 10, 0.0, 16.0, 3.0, True, 0, 10, 1e-4, 0, 300),
    ("config1_s1", 1797, 64, 10, 0.0, 16.0, 3.0, True, 0, 10, 1e-4, 1, 300),
    ("config1_s2", 1797, 64, 10, 0.0, 16.0, 3.0, True, 0, 10, 1e-4, 2, 300),
    ("float_d16_k7", 5000, 16, 7, -10.0, 10.0, 1.5, False, 3, 7, 1e-4, 3, 300),
    ("float_d128_k32", 20000, 128, 32, -10.0, 10.0, 1.0, False, 5, 32, 1e-4, 5, 100),
    ("float_d3_k64", 4096, 3, 40, -5.0, 5.0, 1.0, False, 7, 64, 1e-5, 7, 200),
    ("overlap_d8_k20", 8000, 8, 5, -1.0, 1.0, 2.0, False, 11, 20, 1e-5, 11, 60),
    ("k1_d8", 1000, 8, 3, -3.0, 3.0, 1.0, False, 13, 1, 1e-4, 13, 50),
    ("int_d2_k5", 3000, 2, 5, 0.0, 10.0, 2.0, True, 17, 5, 0.0, 17, 100),
    ("d200_k256", 6000, 200, 256, -10.0, 10.0, 1.0, False, 19, 256, 1e-4, 19, 30),
]


def x_hash(X: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(X, np.float32).tobytes()).hexdigest()


def main():
    if helpers.reference_lib() is None:
        raise SystemExit("reference build (oracle/_ref) unavailable")
    meta = []
    arrays = {}
    for (name, n, d, blobs, lo, hi, sigma, rc, dseed, k, tol, kseed, maxiter) in CASES:
        X, _ = helpers.synth_blobs_np(n, d, blobs, lo, hi, sigma, dseed, round_clip=rc)
        it, lab = helpers.ref_lloyd(X, k, tol, kseed, maxiter)
        meta.append(dict(name=name, n=n, d=d, blobs=blobs, lo=lo, hi=hi, sigma=sigma, round_clip=rc,
                         data_seed=dseed, k=k, tol=tol, seed=kseed, maxiter=maxiter,
                         ref_iter=it, x_sha256=x_hash(X),
                         counts=np.bincount(lab, minlength=k).tolist()))
        arrays[name] = lab.astype(np.uint16)
        print(f"{name}: reference run() = {it}")
    (HERE / "lloyd_cases.json").write_text(json.dumps(meta, indent=1) + "\n")
    np.savez_compressed(HERE / "lloyd_labels.npz", **arrays)


if __name__ == "__main__":
    main()
