"""Benchmark of the k-means iteration hot path on GB300.

Workload: Lloyd k-means, n = 1,048,576 points, d = 128, k = 256 (256 seeded
isotropic Gaussian blobs, centers U[-10,10]^128, sigma = 1, FP32 input).  One
step = one Lloyd iteration over all n points: distance stage with fused argmin,
exact near-tie refinement, label sort (one-hot V), centroid update V.X,
convergence and objective reductions.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision bf16|bf16x3|fp32]

--impl ours (default) prints one JSON line: `value` = iterations/s of the
split-BF16x3 tensor-core + exact-refinement path (hi*hi + hi*lo + lo*hi,
FP32 accumulate; --precision bf16 for the single-BF16 form) with the points
resident in HBM
(device-timed with CUDA events on the launching stream), the FP32 plain path
beside it, labels compared between the two, `roofline` for the dominant kernel,
`e2e` through the C ABI from pinned host memory, `cpu_baseline` (the oracle port
on this host's cores).  --impl reference times the reference's CPU k-means
algorithm on the host cores (the oracle port; the reference's own build where it
exists) on a bounded sample per step.  N > 1 (torchrun) runs independent
replicas, one per GPU ("replicas only": k-means here has no data-path exchange).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "tests"))

N, D, K = 1_048_576, 128, 256
BLOBS, LO, HI, SIGMA, DATA_SEED = 256, -10.0, 10.0, 1.0, 1000
KM_SEED, TOL = 0, 1e-4
E2E_ITERS = 20          # iterations of the end-to-end fit (one H2D of X per fit)
FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12   # nominal FP32 FMA rate (80.5 TFLOP/s)
METRIC = "iters/s (n=1M,d=128,k=256): BF16-TC vs FP32 plain at equal labels; % of peak"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        j = json.loads(p.read_text())
        return j["hbm_gbs"], j["bf16_tflops"], "measured"
    return 6800.0, 1900.0, "fallback"


class Clocks:
    """nvidia-smi sampling every 20 ms around the timed region: sampling has
    started (first sample read) before the region begins and runs until a
    sample after its end, so that short regions are bracketed."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
            t0 = time.time()
            while not self.rows and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.005)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            n0, t0 = len(self.rows), time.time()
            while len(self.rows) <= n0 and time.time() - t0 < 1.0 and self.proc.poll() is None:
                time.sleep(0.005)
            self.proc.terminate()
            try:
                self.proc.wait(2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) >= 9:
                for nm, v in zip(names, r[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        loaded = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def repo_libraries_loaded():
    """Shared libraries of this repository mapped into this process (from
    /proc/self/maps; empty where that file does not exist)."""
    try:
        maps = Path("/proc/self/maps").read_text().splitlines()
    except OSError:
        return []
    libs = {ln.split()[-1] for ln in maps if ln.endswith(".so") and str(ROOT) in ln}
    return sorted(str(Path(x).relative_to(ROOT)) for x in libs)


def bench_config(world):
    """The `config` object both arms print."""
    return {"workload": f"lloyd n={N} d={D} k={K} (256 gaussian blobs, sigma 1, centers U[-10,10])",
            "n": N, "d": D, "k": K, "maxiter": "steps (stop rule off)",
            "l2": "inputs larger than L2 (X fp32 512 MiB, bf16 256 MiB; L2 129 MB)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def make_data(km):
    return km.synth_blobs(N, D, BLOBS, LO, HI, SIGMA, DATA_SEED, nthreads=os.cpu_count() or 8)


def run_cpu_sample(X, threads, sample_rows, min_seconds, use_ref=False):
    """The reference CPU k-means iteration (comparisons/CPU_Kmeans/src/kmeans.cpp:86-155:
    assignment by the CPU distance formula, strict-< argmin, sum-then-scale
    update) on the first `sample_rows` points of the workload against k seeded
    sample centroids, repeated until `min_seconds` have passed; on `threads`
    host threads (the oracle port), or the reference's own single-threaded build
    where it exists.  Returns full-n iterations/s (scaled by n/sample_rows when
    the sample is smaller than n), the seconds of one repetition, and the
    repetitions run."""
    import helpers
    Xs = np.ascontiguousarray(X[:sample_rows])
    rng = np.random.default_rng(0)
    C0 = Xs[rng.choice(sample_rows, K, replace=False)].copy()
    t = []
    t_start = time.perf_counter()
    while not t or (time.perf_counter() - t_start < min_seconds and len(t) < 64):
        t0 = time.perf_counter()
        if use_ref:
            helpers.ref_lloyd(Xs, K, -1.0, KM_SEED, 1)
        else:
            lab, _ = helpers.orc_assign(Xs, C0, threads=threads)
            helpers.orc_update(Xs, lab, K, threads=threads)
        t.append(time.perf_counter() - t0)
    per_iter_full = statistics.median(t) * (N / sample_rows)
    return 1.0 / per_iter_full, statistics.median(t), len(t)


PARITY_ITERS = 5        # iterations of the full-size oracle comparison


def oracle_parity(km, X, Xd, dev, stream, precisions):
    """Full-size parity with the oracle on the bench's own points: a
    PARITY_ITERS-iteration fit per precision (seeded sample-pick init, the
    reference CPU's centroid-shift stop rule with tol) against
    (1) the oracle's restatement of the reference CPU k-means
        (comparisons/CPU_Kmeans/src/kmeans.cpp:49-200): labels and centroids
        bit for bit and the returned iteration;
    (2) the FP64 oracle from the same initial centroids: label agreement and
        the relative error of the last assignment's objective."""
    import torch
    import helpers
    threads = os.cpu_count() or 8
    t0 = time.perf_counter()
    it32, lab32, cen32, _ = helpers.orc_lloyd(X, K, TOL, KM_SEED, PARITY_ITERS, threads=threads)
    it64, lab64, _, _, obj64 = helpers.orc_lloyd64_obj(X, K, TOL, KM_SEED, PARITY_ITERS, threads=threads)
    cpu_s = time.perf_counter() - t0
    out = {"iterations": PARITY_ITERS, "oracle_seconds": cpu_s, "oracle_threads": threads}
    with torch.cuda.stream(stream):
        for prec in precisions:
            m = km.Lloyd(N, D, K, tol=TOL, seed=KM_SEED, maxiter=PARITY_ITERS, precision=prec, conv="shift",
                         device=dev, stream=stream.cuda_stream).set_data(Xd)
            lab, cen, r = m.fit()
            m.close()
            out[prec] = {
                "label_agreement_vs_oracle": float((lab == lab32).mean()),
                "centroids_bitwise_equal_vs_oracle": bool(np.array_equal(cen.view(np.uint32), cen32.view(np.uint32))),
                "iteration_equal_vs_oracle": int(r.converged_iter) == it32,
                "label_agreement_vs_fp64": float((lab == lab64).mean()),
                "objective_rel_err_vs_fp64": abs(r.objective - obj64) / abs(obj64),
            }
    return out


def reference_arm(args, rank):
    import helpers
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    use_ref = helpers.reference_lib() is not None
    if use_ref:
        threads = 1                           # the reference CPU k-means is single-threaded
    # the port runs one whole iteration over all n points per step; the
    # single-threaded reference build (about 30 s per full iteration) a 1/16 slice
    sample = N if not use_ref else N // 16
    # the numpy twin of the product's generator (same values, checked in the
    # CPU tests), so that this arm loads no product library
    X, _ = helpers.synth_blobs_np_chunked(N, D, BLOBS, LO, HI, SIGMA, DATA_SEED)
    vals = []
    for i in range(args.warmup + args.steps):
        v, secs, _ = run_cpu_sample(X, threads, sample, 0.0, use_ref)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    kind = "reference" if use_ref else "port"
    what = ("the reference's comparisons/CPU_Kmeans built from its sources (oracle/_ref)" if use_ref else
            "the oracle port of comparisons/CPU_Kmeans/src/kmeans.cpp:86-155")
    line = {
        "metric": METRIC, "value": value, "unit": "iters/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "impl": "reference",
        "config": bench_config(args.gpus),
        "cpu_baseline": {"value": value, "unit": "iters/s", "cores": threads, "kind": kind,
                         "sample": f"{what}: one assignment+update of {sample} of the {N} points against "
                                   f"k={K} centroids per step on {threads} host threads"
                                   + (f", scaled by n/{sample}" if sample != N else "")},
        "e2e": {"value": value, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "repo_libraries_loaded": repo_libraries_loaded(),
    }
    return line


def ours_arm(args, rank, world):
    import torch
    import helpers
    km = helpers.km()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()
    X = make_data(km)
    Xd = torch.from_numpy(X).to(f"cuda:{dev}")
    res = {}
    labels = {}
    timing = {}
    barrier = (lambda: torch.distributed.barrier()) if world > 1 else (lambda: None)
    others = [q for q in ("bf16", "bf16x3") if q != args.precision]
    with torch.cuda.stream(stream):
        for prec in [args.precision, "fp32"] + others:
            m = km.Lloyd(N, D, K, tol=TOL, seed=KM_SEED, maxiter=args.warmup, precision=prec,
                         conv="none", device=dev, stream=stream.cuda_stream).set_data(Xd)
            m.fit(want_centroids=False)                         # warm-up iterations (graph built)
            m.p.maxiter = args.steps
            m.close()
            m = km.Lloyd(N, D, K, tol=TOL, seed=KM_SEED, maxiter=args.steps, precision=prec,
                         conv="none", device=dev, stream=stream.cuda_stream).set_data(Xd)
            m.fit(want_centroids=False)                         # builds this handle's graph
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            barrier()
            torch.cuda.synchronize()
            clk = Clocks(dev)
            with clk:
                ev0.record(stream)
                lab, _, r = m.fit(want_centroids=False)
                ev1.record(stream)
                torch.cuda.synchronize()
            barrier()
            ms = ev0.elapsed_time(ev1)
            # the fit above includes the seeded init; the library's own loop timer
            # brackets exactly the `steps` iterations
            timing[prec] = dict(ms_total=ms, ms_loop=r.fit_ms, iters=r.iterations, clocks=clk.summary(),
                                refined=r.refined_rows, full=r.full_rescore_rows, objective=r.objective,
                                launches=r.kernel_launches)
            labels[prec] = lab
            res[prec] = m
    ms_loop = timing[args.precision]["ms_loop"]
    if world > 1:
        t = torch.tensor([ms_loop], device=f"cuda:{dev}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_loop = float(t.item())
    iters = timing[args.precision]["iters"]
    value = world * iters / (ms_loop / 1000.0)
    fp32_ips = timing["fp32"]["iters"] / (timing["fp32"]["ms_loop"] / 1000.0)
    agree = float((labels[args.precision] == labels["fp32"]).mean())
    sizes = np.bincount(labels[args.precision], minlength=K)

    # per-stage timing with CUDA events on the launching stream
    with torch.cuda.stream(stream):
        stages = res[args.precision].profile(max(3, min(args.steps, 10)))
        stages32 = res["fp32"].profile(3)
    for m in res.values():
        m.close()
    names = ["distance+argmin", "refine", "label sort", "centroid sums", "finalize+control"]
    hbm, bf16, src = peaks()
    dp = (D + 63) // 64 * 64
    # algorithmic bytes of each stage per iteration: distance = BF16 point
    # copies (hi, and lo for the split form) + labels + minima; sort = labels
    # read three times + the permutation written; sums = X + permutation +
    # centroids in and out; finalize = three passes over k x d floats
    bytes_stage = [N * dp * 2 + N * 4 + N * 4, 0, 3 * N * 4 + N * 4,
                   N * D * 4 + N * 4 + 2 * K * D * 4, K * D * 4 * 3]
    if args.precision == "bf16x3":
        bytes_stage[0] += N * dp * 2
    flops_dist = 2.0 * N * K * D
    dom = int(np.argmax(stages))
    st_ms = stages[dom]
    if dom == 0:
        ach_tf = flops_dist / (st_ms / 1e3) / 1e12
        ach_gb = bytes_stage[0] / (st_ms / 1e3) / 1e9
        # the distance GEMM sits at the ridge: report the tighter of the two bounds
        if ach_gb / hbm >= ach_tf / bf16:
            roof = {"bound": "hbm", "achieved": ach_gb, "peak": hbm, "unit": "GB/s", "frac": ach_gb / hbm}
        else:
            roof = {"bound": "tensor", "achieved": ach_tf, "peak": bf16, "unit": "TFLOP/s", "frac": ach_tf / bf16}
    else:
        ach_gb = bytes_stage[dom] / (st_ms / 1e3) / 1e9
        roof = {"bound": "hbm", "achieved": ach_gb, "peak": hbm, "unit": "GB/s", "frac": ach_gb / hbm}
    roof.update({"kernel": names[dom], "ms": st_ms, "peak_source": src,
                 "ms_source": "km_lloyd_profile: one iteration captured as a CUDA graph with event-record "
                              "nodes between the stages, replayed on the launching stream",
                 "traffic": TRAFFIC.get((args.precision, names[dom]))})

    # e2e: the public C ABI from pinned host memory: set_data (H2D) + fit + labels D2H,
    # a fit of E2E_ITERS iterations whatever --steps is (the H2D is paid once per fit)
    e2e = None
    if rank == 0 or world > 1:
        Xp = torch.from_numpy(X).pin_memory()
        with torch.cuda.stream(stream):
            m = km.Lloyd(N, D, K, tol=TOL, seed=KM_SEED, maxiter=E2E_ITERS, precision=args.precision,
                         conv="none", device=dev, stream=stream.cuda_stream)
            import ctypes as C
            lab = np.empty(N, np.uint32)
            lab_p = torch.from_numpy(lab).pin_memory()
            r = km.Result()
            for rep in range(2):   # first call builds the graph
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                km.check(km.lib().km_lloyd_set_data(m.h, Xp.data_ptr(), 0), "set_data")
                km.check(km.lib().km_lloyd_fit(m.h, None, lab_p.data_ptr(), None, C.byref(r)), "fit")
                torch.cuda.synchronize()
                wall = time.perf_counter() - t0
            m.close()
        its = max(1, r.iterations)
        e2e = {"value": r.iterations / wall, "unit": "iters/s",
               "h2d_bytes_per_step": N * D * 4 / its, "d2h_bytes_per_step": N * 4 / its,
               "h2d_bytes_per_fit": N * D * 4, "d2h_bytes_per_fit": N * 4,
               "step": f"one km_lloyd_fit from pinned host memory: km_lloyd_set_data (H2D of X) + "
                       f"seeded init + {r.iterations} iterations + labels D2H; wall clock {wall * 1e3:.2f} ms; "
                       f"the fit's copies divided over its {r.iterations} iterations"}

    parity = oracle_parity(km, X, Xd, dev, stream, [args.precision, "fp32"] + others) if rank == 0 else None

    cpu = None
    if rank == 0:
        threads = os.cpu_count() or 1
        v, secs, reps = run_cpu_sample(X, threads, N, 10.0)
        cpu = {"value": v, "unit": "iters/s", "cores": threads, "kind": "port",
               "sample": f"whole iterations (assignment+update, oracle port of comparisons/CPU_Kmeans/src/"
                         f"kmeans.cpp:86-155) over all {N} points against k={K}: {reps} repetitions of "
                         f"{secs:.2f} s each, median"}
    clocks = timing[args.precision]["clocks"]
    line = {
        "metric": METRIC, "value": value, "unit": "iters/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_loop / iters, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16" if args.precision != "fp32" else "f32",
        "data": "synthetic",
        "config": bench_config(world),
        "precision": args.precision,
        "fp32_plain": {"value": fp32_ips, "unit": "iters/s", "stages_ms": stages32,
                       # the FP32 distance kernel (stage 0) on 2nkd FLOP against the nominal FP32 rate
                       "distance_tflops": (2.0 * N * K * D / (stages32[0] * 1e-3) / 1e12) if stages32 else None,
                       "distance_frac_of_nominal": (2.0 * N * K * D / (stages32[0] * 1e-3) / 1e12 / FP32_NOMINAL_TFLOPS)
                       if stages32 else None,
                       "nominal_tflops": FP32_NOMINAL_TFLOPS,
                       "nominal_source": "152 SMs x 128 FP32 lanes x 2 FLOP x 2.07 GHz; no measured FP32 figure"},
        "other_tc_forms": {q: {"value": timing[q]["iters"] / (timing[q]["ms_loop"] / 1000.0), "unit": "iters/s",
                               "label_agreement_vs_fp32": float((labels[q] == labels["fp32"]).mean()),
                               "refined_rows_per_iter": timing[q]["refined"] / max(1, timing[q]["iters"])}
                           for q in others},
        "speedup_vs_fp32_plain": value / world / fp32_ips,
        "label_agreement_vs_fp32": agree,
        "label_agreement_vs_oracle": parity[args.precision]["label_agreement_vs_oracle"] if parity else None,
        "objective_rel_err_vs_fp64": parity[args.precision]["objective_rel_err_vs_fp64"] if parity else None,
        "oracle_parity": parity,
        "refined_rows_per_iter": timing[args.precision]["refined"] / max(1, iters),
        "full_rescore_rows_per_iter": timing[args.precision]["full"] / max(1, iters),
        "objective": timing[args.precision]["objective"],
        "cluster_sizes": {"min": int(sizes.min()), "max": int(sizes.max()), "mean": float(sizes.mean()),
                          "empty": int((sizes == 0).sum())},
        "stages_ms": dict(zip(names, stages)),
        "roofline": roof,
        # The same distance kernel against the tensor peak counting the MMAs it
        # issues: three per K step in the split form (hi.hi, hi.lo, lo.hi), one
        # in the single-BF16 form; its MMA floor, not HBM, bounds the split form.
        "roofline_tensor_issued": {
            "bound": "tensor", "kernel": names[0], "ms": stages[0], "unit": "TFLOP/s", "peak": bf16,
            "mma_per_k_step": 3 if args.precision == "bf16x3" else 1,
            "achieved": (3 if args.precision == "bf16x3" else 1) * flops_dist / (stages[0] / 1e3) / 1e12,
            "frac": (3 if args.precision == "bf16x3" else 1) * flops_dist / (stages[0] / 1e3) / 1e12 / bf16,
            "peak_source": src} if args.precision != "fp32" else None,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": timing[args.precision]["launches"],
    }
    return line


# ---------------------------------------------------------------------------
# Secondary workloads (--workload bigk | kkm): the very-large-k Lloyd case and
# kernel k-means with a precomputed kernel matrix.  Same JSON contract, one GPU.
# ---------------------------------------------------------------------------
BIGK = dict(n=4_194_304, d=256, k=4096, lo=-20.0, hi=20.0, sigma_range=(0.2, 2.0), zipf=1.1, seed=5000,
            tol=1e-5)
KKM = dict(n=65_536, d=512, k=64, lo=-1.0, hi=1.0, sigma=0.25, seed=3000)


def _event_ms(fn, stream):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    out = fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), out


def stages_only(args):
    """Per-stage times of the lloyd workload on one GPU: a 5-iteration fit
    (graph built, warm) then Lloyd.profile(10)."""
    import torch
    import helpers
    km = helpers.km()
    n = args.rows or N
    X = make_data(km)[:n]
    Xd = torch.from_numpy(X).cuda()
    stream = torch.cuda.Stream()
    names = ["distance+argmin", "refine", "label sort", "centroid sums", "finalize+control"]
    with torch.cuda.stream(stream):
        m = km.Lloyd(n, D, K, tol=TOL, seed=KM_SEED, maxiter=5, precision=args.precision, conv="none",
                     stream=stream.cuda_stream).set_data(Xd)
        m.fit(want_centroids=False)
        st = m.profile(10)
        m.close()
    return {"workload": bench_config(1)["workload"], "rows": n, "precision": args.precision,
            "stages_ms": dict(zip(names, st))}


def bigk_arm(args):
    """Lloyd with n = 4,194,304, d = 256, k = 4096, BF16-stored points from a
    seeded mixture with Zipf(1.1) cluster sizes, per-cluster sigma U[0.2, 2],
    centers U[-20, 20]^256.  BF16 tensor cores + exact refinement against the
    FP32 plain path on the same points."""
    import torch
    import helpers
    km = helpers.km()
    c = BIGK
    n, d, k = (args.rows or c["n"]), c["d"], c["k"]
    stream = torch.cuda.Stream()
    X = km.synth_blobs(n, d, k, c["lo"], c["hi"], 1.0, c["seed"], sigma_range=c["sigma_range"],
                       zipf_s=c["zipf"], nthreads=os.cpu_count() or 8)
    with torch.cuda.stream(stream):
        bits = torch.from_numpy(X).cuda().to(torch.bfloat16).view(torch.int16)
    torch.cuda.synchronize()
    Xd = bits.view(torch.bfloat16).float()                 # the points as FP32 (exact)
    steps32 = 2
    res = {}
    with torch.cuda.stream(stream):
        for prec, steps in ((args.precision, args.steps), ("fp32", steps32)):
            m = km.Lloyd(n, d, k, tol=c["tol"], seed=1, maxiter=steps, precision=prec, conv="none",
                         stream=stream.cuda_stream).set_data_bf16(bits)
            m.fit(want_centroids=False)                    # warm-up fit (builds the graph)
            torch.cuda.synchronize()
            clk = Clocks(0)
            with clk:
                lab, _, r = m.fit(want_centroids=False)
            stages = m.profile(3) if prec != "fp32" else None
            res[prec] = dict(ms=r.fit_ms, iters=r.iterations, launches=r.kernel_launches, clocks=clk.summary(),
                             refined=r.refined_rows, full=r.full_rescore_rows, stages=stages)
            m.close()
        # label agreement after the same iterations from the same seeded start
        m = km.Lloyd(n, d, k, tol=c["tol"], seed=1, maxiter=steps32, precision=args.precision, conv="none",
                     stream=stream.cuda_stream).set_data_bf16(bits)
        lab_b, cen_b, _ = m.fit()
        m.close()
        lab_all, _, _ = km.assign(Xd, torch.from_numpy(cen_b).cuda(), precision=args.precision)
        lab_all = lab_all.cpu().numpy().astype(np.uint32)
        m = km.Lloyd(n, d, k, tol=c["tol"], seed=1, maxiter=steps32, precision="fp32", conv="none",
                     stream=stream.cuda_stream).set_data(Xd)
        lab_f, _, _ = m.fit(want_centroids=False)
        m.close()
    agree = float((lab_b == lab_f).mean())
    sizes = np.bincount(lab_b, minlength=k)
    # Oracle parity: (1) the fit's centroids against the oracle's update of its
    # labels over all n rows; (2) the assignment of all n rows to those
    # centroids against the oracle's (reference CPU formula) and against FP64
    # on 65,536 rows spread over the whole range.
    Xh = Xd.cpu().numpy()
    cen_o, _ = helpers.orc_update(Xh, lab_b, k, threads=os.cpu_count() or 8)
    rows = np.sort(np.random.default_rng(11).choice(n, min(n, 65536), replace=False))
    lab_s, _ = helpers.orc_assign(Xh[rows], cen_b, threads=os.cpu_count() or 8)
    X64, C64 = Xh[rows].astype(np.float64), cen_b.astype(np.float64)
    D64 = (X64 * X64).sum(1)[:, None] - 2.0 * X64 @ C64.T + (C64 * C64).sum(1)[None, :]
    lab64 = D64.argmin(1)
    obj_ours = float(D64[np.arange(len(rows)), lab_all[rows]].sum())
    obj64 = float(D64[np.arange(len(rows)), lab64].sum())
    parity = {"centroids_bitwise_equal_vs_oracle_update": bool(np.array_equal(cen_b.view(np.uint32),
                                                                             cen_o.view(np.uint32))),
              "sample_rows": int(len(rows)),
              "label_agreement_vs_oracle": float((lab_all[rows] == lab_s).mean()),
              "label_agreement_vs_fp64": float((lab_all[rows] == lab64).mean()),
              "objective_rel_err_vs_fp64": abs(obj_ours - obj64) / abs(obj64)}
    del Xh, X64, D64
    rb = res[args.precision]
    value = rb["iters"] / (rb["ms"] / 1e3)
    v32 = res["fp32"]["iters"] / (res["fp32"]["ms"] / 1e3)
    hbm, bf16, src = peaks()
    names = ["distance+argmin", "refine", "label sort", "centroid sums", "finalize+control"]
    st = rb["stages"]
    flops = 2.0 * n * k * d
    ach = flops / (st[0] / 1e3) / 1e12
    # e2e: BF16 bits from pinned host memory through the C ABI
    hb = bits.cpu().pin_memory()
    import ctypes as C
    lab = torch.empty(n, dtype=torch.int32).pin_memory()
    with torch.cuda.stream(stream):
        m = km.Lloyd(n, d, k, tol=c["tol"], seed=1, maxiter=args.steps, precision=args.precision, conv="none",
                     stream=stream.cuda_stream)
        r = km.Result()
        for _ in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            km.check(km.lib().km_lloyd_set_data_bf16(m.h, hb.data_ptr(), 0), "set_data_bf16")
            km.check(km.lib().km_lloyd_fit(m.h, None, lab.data_ptr(), None, C.byref(r)), "fit")
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        m.close()
    # CPU baseline: the oracle port on a row sample, scaled to n
    threads = os.cpu_count() or 1
    samp = 8192
    Xs = Xd[:samp].cpu().numpy()
    C0 = Xs[np.random.default_rng(0).choice(samp, k, replace=False)].copy()
    t0 = time.perf_counter()
    lab_s, _ = helpers.orc_assign(Xs, C0, threads=threads)
    helpers.orc_update(Xs, lab_s, k, threads=threads)
    secs = time.perf_counter() - t0
    cpu_v = 1.0 / (secs * n / samp)
    return {
        "metric": "iters/s (n=4M,d=256,k=4096, BF16 points): BF16-TC vs FP32 plain at equal labels",
        "value": value, "unit": "iters/s", "n_gpus": 1, "steps": args.steps, "warmup": args.steps,
        "ms_per_step": rb["ms"] / rb["iters"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16", "data": "synthetic",
        "config": {"workload": f"lloyd n={n} d=256 k=4096, BF16-stored points, Zipf(1.1) sizes, "
                               "sigma U[0.2,2], centers U[-20,20]", "n": n, "d": d, "k": k,
                   "l2": "inputs larger than L2 (BF16 X 2 GiB)", "parallelism": "single GPU"},
        "precision": args.precision,
        "fp32_plain": {"value": v32, "unit": "iters/s", "iters": res["fp32"]["iters"]},
        "speedup_vs_fp32_plain": value / v32,
        "label_agreement_vs_fp32": agree,
        "label_agreement_vs_oracle": parity["label_agreement_vs_oracle"],
        "objective_rel_err_vs_fp64": parity["objective_rel_err_vs_fp64"],
        "oracle_parity": parity,
        "refined_rows_per_iter": rb["refined"] / max(1, rb["iters"]),
        "full_rescore_rows_per_iter": rb["full"] / max(1, rb["iters"]),
        "cluster_sizes": {"max": int(sizes.max()), "median": float(np.median(sizes)), "empty": int((sizes == 0).sum())},
        "stages_ms": dict(zip(names, st)),
        "roofline": {"bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s", "frac": ach / bf16,
                     "kernel": "distance+argmin (assign_tc_chunked_kernel)", "ms": st[0], "peak_source": src,
                     "traffic": None},
        "e2e": {"value": r.iterations / wall, "unit": "iters/s", "h2d_bytes_per_step": n * d * 2,
                "d2h_bytes_per_step": n * 4,
                "step": f"km_lloyd_set_data_bf16 from pinned host + seeded init + {r.iterations} iterations + "
                        f"labels D2H; wall {wall * 1e3:.1f} ms"},
        "cpu_baseline": {"value": cpu_v, "unit": "iters/s", "cores": threads, "kind": "port",
                         "sample": f"one assignment+update of {samp} rows against k={k} (oracle port), "
                                   f"{secs:.2f} s, scaled by n/{samp}"},
        "clocks": rb["clocks"],
        "gpu_launches": rb["launches"],
    }


def kkm_arm(args):
    """Kernel k-means with a precomputed kernel matrix: n = 65,536, d = 512,
    k = 64, 64 seeded blobs (centers U[-1,1]^512, sigma 0.25); polynomial
    (x.y/d + 1)^2 and Gaussian (sigma 0.5) kernels; K stored FP32 (16 GiB)
    or BF16 (8 GiB); K built on the tensor cores (split-BF16x3 for FP32
    storage, BF16 for BF16 storage)."""
    import torch
    import helpers
    import importlib.util
    km = helpers.km()
    spec = importlib.util.spec_from_file_location("kkm_step", ROOT / "oracle" / "kkm_step.py")
    ks = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ks)
    c = KKM
    n, d, k = c["n"], c["d"], c["k"]
    X = km.synth_blobs(n, d, k, c["lo"], c["hi"], c["sigma"], c["seed"], nthreads=os.cpu_count() or 8)
    Xd = torch.from_numpy(X).cuda()
    stream = torch.cuda.current_stream()
    hbm, bf16, src = peaks()
    rows = {}
    for kern, params in (("polynomial", dict(gamma=1.0 / d, coef=1.0, degree=2)), ("gaussian", dict(sigma=0.5))):
        for kb16 in (False, True):
            prec = "bf16" if kb16 else "bf16x3"
            m = km.KernelKMeans(n, d, k, kernel=kern, maxiter=args.steps, precision=prec, k_bf16=kb16,
                                **params).set_data(Xd)
            kb_ms = [m.build_ms()]
            m.set_data(Xd)                                 # second build: warm
            kb_ms.append(m.build_ms())
            m.fit()                                        # warm-up
            clk = Clocks(0)
            with clk:
                lab, r = m.fit()
            # one more iteration from the fit's labels, against the FP64 oracle's
            km.check(km.lib().km_kkm_configure(m.h, 1, m.p.tol, 0), "km_kkm_configure")
            lab1, r1 = m.fit(init_labels=lab)
            m.close()
            new, score = ks.kkm_step_f64(X, lab, k, kern, **params, workers=max(1, (os.cpu_count() or 8) // 2))
            trace = float(ks.kernel_diag(X, kern, **params).sum())
            torch.cuda.empty_cache()
            ips = r.iterations / (r.fit_ms / 1e3)
            kbytes = n * n * (2 if kb16 else 4)
            it_ms = r.fit_ms / r.iterations
            rows[f"{kern}/{'bf16' if kb16 else 'fp32'}K"] = {
                "iters_per_s": ips, "ms_per_iter": it_ms, "k_build_ms": min(kb_ms),
                "k_build_tflops": 2.0 * n * n * d / (min(kb_ms) / 1e3) / 1e12,
                "iter_gbs": (kbytes + 4 * n + 4 * n * k) / (it_ms / 1e3) / 1e9,
                "score": r.score, "clocks": clk.summary(), "launches": r.kernel_launches,
                "one_step_vs_fp64": {"label_agreement": float((lab1 == new).mean()),
                                     "objective_rel_err": abs((r1.score + trace) - (score + trace)) / abs(score + trace)}}
    head = rows["polynomial/fp32K"]
    # e2e through the public API from host memory: set_data (H2D of X and the
    # K build) + fit + labels D2H, the headline variant
    Xp = torch.from_numpy(X).pin_memory()
    m = km.KernelKMeans(n, d, k, kernel="polynomial", maxiter=args.steps, precision="bf16x3", k_bf16=False,
                        gamma=1.0 / d, coef=1.0, degree=2)
    for rep in range(2):                                   # first round: allocation and warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m.set_data(Xp.numpy())
        _, r = m.fit()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    m.close()
    torch.cuda.empty_cache()
    e2e = {"value": r.iterations / wall, "unit": "iters/s", "h2d_bytes_per_step": n * d * 4,
           "d2h_bytes_per_step": n * 4,
           "step": f"one fit from host memory: set_data (H2D of X + K build) + {r.iterations} iterations "
                   f"+ labels D2H; wall clock {wall * 1e3:.1f} ms"}
    return {
        "metric": "iters/s (kernel k-means n=65536,d=512,k=64, precomputed K)",
        "value": head["iters_per_s"], "unit": "iters/s", "n_gpus": 1, "steps": args.steps, "warmup": args.steps,
        "ms_per_step": head["ms_per_iter"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "kernel k-means n=65536 d=512 k=64, polynomial (x.y/d+1)^2, K FP32 16 GiB",
                   "n": n, "d": d, "k": k, "l2": "K larger than L2", "parallelism": "single GPU"},
        "variants": rows,
        "label_agreement_vs_fp64": head["one_step_vs_fp64"]["label_agreement"],
        "objective_rel_err_vs_fp64": head["one_step_vs_fp64"]["objective_rel_err"],
        "oracle_parity_note": "one iteration from the timed fit's labels against the FP64 oracle (K formed block "
                              "by block), per variant; the reference GPU path itself cannot be built here",
        "roofline": {"bound": "hbm", "achieved": head["iter_gbs"], "peak": hbm, "unit": "GB/s",
                     "frac": head["iter_gbs"] / hbm, "kernel": "kkm_vk_kernel (V.K streaming of K)",
                     "peak_source": src, "traffic": None},
        "clocks": head["clocks"], "gpu_launches": head["launches"], "e2e": e2e,
    }


KKM_PANEL = dict(n=262_144, d=512, k=64, lo=-1.0, hi=1.0, sigma=0.25, seed=3100, panel=8192)


def kkm_panel_arm(args):
    """Kernel k-means where the kernel matrix does not fit the device: n =
    262,144, d = 512, k = 64, 64 seeded blobs (centers U[-1,1]^512, sigma
    0.25), polynomial (x.y/d + 1)^2, split-BF16x3 on the tensor cores.  The
    FP32 K would be 275 GB (the reference's n*n buffer, src/kmeans.cu:143).
    Two ways without it, both timed: K rebuilt every iteration in panels of
    8192 rows (8 GiB) streamed into E = K V^T (fits identical to a resident
    K), and the fused kernel that keeps no K (X against a label-sorted copy of
    X, kernel values summed per cluster in the epilogue).  `value` is the
    faster of the two."""
    import torch
    import helpers
    km = helpers.km()
    c = KKM_PANEL
    n, d, k = c["n"], c["d"], c["k"]
    X = km.synth_blobs(n, d, k, c["lo"], c["hi"], c["sigma"], c["seed"], nthreads=os.cpu_count() or 8)
    Xd = torch.from_numpy(X).cuda()
    hbm, bf16, src = peaks()
    pj = ROOT / "MEASURED_PEAKS.json"
    bf16_sus = (json.loads(pj.read_text()).get("bf16_tflops_sustained") if pj.exists() else None) or 1700.0
    params = dict(gamma=1.0 / d, coef=1.0, degree=2)
    mma_flops = 3 * 2.0 * n * n * d                           # split-BF16x3: three BF16 products per K entry
    modes, labs = {}, {}
    for mode, pr in (("panels", c["panel"]), ("fused", "fused")):
        m = km.KernelKMeans(n, d, k, kernel="polynomial", maxiter=args.warmup, precision="bf16x3", k_bf16=False,
                            panel_rows=pr, **params).set_data(Xd)
        m.fit()                                              # warm-up iterations
        km.check(km.lib().km_kkm_configure(m.h, args.steps, m.p.tol, 0), "km_kkm_configure")
        clk = Clocks(0)
        with clk:
            lab, r = m.fit()
        m.close()
        torch.cuda.empty_cache()
        it_ms = r.fit_ms / r.iterations
        labs[mode] = lab
        modes[mode] = {"iters_per_s": r.iterations / (r.fit_ms / 1e3), "ms_per_iter": it_ms,
                       "mma_tflops": mma_flops / (it_ms / 1e3) / 1e12, "score": r.score,
                       "iterations": r.iterations, "launches": r.kernel_launches, "clocks": clk.summary()}
    modes["panels"]["panel_rows"] = c["panel"]
    modes["panels"]["panel_hbm_gbs"] = 2 * n * n * 4 / (modes["panels"]["ms_per_iter"] / 1e3) / 1e9
    agree = float((labs["panels"] == labs["fused"]).mean())
    best = max(modes, key=lambda md: modes[md]["iters_per_s"])
    head = modes[best]
    # e2e through the public API from host memory: set_data (H2D of X) + fit + labels D2H
    Xp = torch.from_numpy(X).pin_memory()
    m = km.KernelKMeans(n, d, k, kernel="polynomial", maxiter=args.steps, precision="bf16x3", k_bf16=False,
                        panel_rows=c["panel"] if best == "panels" else "fused", **params)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m.set_data(Xp.numpy())
    _, r2 = m.fit()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    m.close()
    torch.cuda.empty_cache()
    kern = ("kkm_fused_tc_kernel (X against the label-sorted X copy, per-cluster sums in the epilogue)"
            if best == "fused" else
            "whole iteration: kmat_tc_kernel panel builds then kkm_vk_kernel panel streams, in sequence")
    return {
        "metric": "iters/s (kernel k-means n=262144,d=512,k=64, no resident kernel matrix)",
        "value": head["iters_per_s"], "unit": "iters/s", "n_gpus": 1, "steps": head["iterations"],
        "warmup": args.warmup, "ms_per_step": head["ms_per_iter"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "kernel k-means n=262144 d=512 k=64, polynomial (x.y/d+1)^2, split-BF16x3, "
                               f"{best} (resident FP32 K would be 275 GB)",
                   "n": n, "d": d, "k": k, "mode": best, "l2": "operands and panels larger than L2",
                   "parallelism": "single GPU"},
        "variants": modes, "label_agreement_panels_vs_fused": agree,
        "roofline": {"bound": "tensor", "achieved": head["mma_tflops"], "peak": bf16_sus, "unit": "TFLOP/s",
                     "frac": head["mma_tflops"] / bf16_sus,
                     "kernel": kern + "; BF16 MMA flops, 3 per K entry, over the whole iteration",
                     "peak_source": src + " (bf16 sustained)", "traffic": None},
        "clocks": head["clocks"], "gpu_launches": head["launches"],
        "e2e": {"value": r2.iterations / wall, "unit": "iters/s", "h2d_bytes_per_step": n * d * 4,
                "d2h_bytes_per_step": n * 4,
                "step": f"one fit from host memory ({best}): set_data (H2D of X) + {r2.iterations} iterations + "
                        f"labels D2H; wall clock {wall * 1e3:.1f} ms"},
    }


def batch_arm(args):
    """512 independent Lloyd problems, n log-uniform in [1024, 65536], d in
    {2, 8, 16, 32, 64, 128, 256}, k uniform in [2, 128] (k < n), one seeded
    Gaussian blob per cluster (sigma 1, centers U[-5, 5]^d), FP32, 8 seeded
    restarts each, all in one persistent launch; against a sequential loop of
    single-problem fits (the FP32 Lloyd handle, one instance after another)."""
    import helpers
    km = helpers.km()
    P, R = 512, 8
    shapes = helpers.batch_problems(P)
    Xs = helpers.batch_points(shapes, nthreads=os.cpu_count() or 8)
    b = km.Batch(shapes, restarts=R, seed=0, tol=1e-4, maxiter=300).set_data(Xs)
    v, tune_ms = b.tune()
    b.fit()                                          # warm-up
    clk = Clocks(0)
    with clk:
        best, results, ms = b.fit()
    # e2e through the public API from host memory: set_data (H2D of every
    # problem's points) + fit (labels and centroids back to the host)
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.set_data(Xs)
    b.fit()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    b.close()
    e2e = {"value": P / e2e_s, "unit": "problems/s",
           "h2d_bytes_per_step": int(sum(x.nbytes for x in Xs)), "d2h_bytes_per_step": int(sum(n * 4 + k * d * 4 for n, d, k in shapes)),
           "step": f"set_data of all {P} problems from host memory + one batched fit with results to the host; "
                   f"wall clock {e2e_s * 1e3:.1f} ms"}
    iters = sum(r[1] for pr in results for r in pr)
    # Oracle parity on the full-size problems: the four largest (n*d*k) and
    # twelve seeded others, restart 0 and the last restart of each.
    work = np.array([n * d * k for n, d, k in shapes])
    big = [int(p) for p in np.argsort(work)[::-1][:4]]
    others = [int(p) for p in np.random.default_rng(5).permutation(P) if int(p) not in big][:12]
    b2 = km.Batch(shapes, restarts=R, seed=0, tol=1e-4, maxiter=300).set_data(Xs)
    b2.fit()
    same, checked = 0, 0
    for p in big + others:
        n, d, k = shapes[p]
        for r in (0, R - 1):
            it_o, lab_o, cen_o, _ = helpers.orc_lloyd(Xs[p], k, 1e-4, p * R + r, 300, threads=os.cpu_count() or 8)
            lab, cen = b2.instance(p, r)
            same += int(np.array_equal(lab, lab_o) and np.array_equal(cen.view(np.uint32), cen_o.view(np.uint32))
                        and results[p][r][0] == it_o)
            checked += 1
    b2.close()
    # the assignment's arithmetic: 3 FP32 operations (sub, mul, add: the
    # reference formula, no FMA) per point, centroid and coordinate, per
    # iteration of every instance
    ops = 3.0 * sum(results[p][r][1] * shapes[p][0] * shapes[p][1] * shapes[p][2]
                    for p in range(P) for r in range(R))
    fp32_peak = 152 * 128 * 2.07e9 / 1e12          # nominal FP32 instructions/s (T/s)
    ach = ops / (ms / 1e3) / 1e12
    # sequential per-problem loop on a sample of problems (all restarts), scaled
    sample = list(range(0, P, P // 16))[:16]
    t0 = time.perf_counter()
    seq_iters = 0
    for p in sample:
        n, d, k = shapes[p]
        for r in range(R):
            m = km.Lloyd(n, d, k, tol=1e-4, seed=p * R + r, maxiter=300, precision="fp32").set_data(Xs[p])
            _, _, res = m.fit(want_centroids=False)
            seq_iters += res.iterations
            m.close()
    seq_s = time.perf_counter() - t0
    work = [n * k * d for (n, d, k) in shapes]
    seq_frac = sum(work[p] for p in sample) / sum(work)
    seq_pps = len(sample) / seq_s
    value = P / (ms / 1e3)
    names = ["128x8", "128x16", "128x32", "256x8", "256x16", "256x32"]
    return {
        "metric": "problems/s (512 uneven Lloyd problems x 8 restarts, one persistent launch)",
        "value": value, "unit": "problems/s", "n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batched lloyd: 512 problems, n log-U[1024,65536], d in {2..256}, k U[2,128], "
                               "8 restarts, blobs sigma 1 centers U[-5,5]", "problems": P, "restarts": R,
                   "points_total": int(sum(n for n, _, _ in shapes)), "parallelism": "single GPU"},
        "instance_iterations": int(iters),
        "autotune": {"chosen": names[v], "ms_on_sample": dict(zip(names, tune_ms))},
        "sequential_loop": {"value": seq_pps, "unit": "problems/s", "sample_problems": len(sample),
                            "sample_work_fraction": seq_frac,
                            "note": "km_lloyd FP32 handle per instance, one after another, same seeds"},
        "speedup_vs_sequential": value / seq_pps,
        "oracle_parity": {"instances_checked": checked, "instances_identical": same,
                          "label_agreement_vs_oracle": same / checked,
                          "what": "labels, centroids bit for bit and the returned iteration against the oracle's "
                                  "single run, the 4 largest and 12 other problems, restarts 0 and 7"},
        "roofline": {"bound": "fp32", "achieved": ach, "peak": fp32_peak, "unit": "T FP32 instr/s",
                     "frac": ach / fp32_peak, "kernel": "batch_lloyd_kernel (exact reference-formula assignment)",
                     "peak_source": "nominal (152 SMs x 128 FP32 lanes x 2.07 GHz; no measured FP32 figure)",
                     "traffic": None},
        "clocks": clk.summary(), "gpu_launches": 1, "e2e": e2e,
    }


# dram__bytes_read.sum + dram__bytes_write.sum per launch of the stage's
# dominant kernel, from one ncu capture of this command
# (profiles/lloyd_iteration_n1M_d128_k256_launches.md; averages over the
# launches of each arm).  Keys: (precision, stage).
TRAFFIC = {
    ("bf16x3", "distance+argmin"): 551.8e6,      # assign_tc_kernel<1, false>
    ("bf16x3", "refine"): 44.0e6,                # refine_staged_kernel<true>
    ("bf16x3", "label sort"): 10.6e6,            # seg_hist + seg_scan + seg_scatter
    ("bf16x3", "centroid sums"): 541.6e6,        # update_sums_bulk_kernel
    ("bf16x3", "finalize+control"): 0.7e6,
    ("bf16", "distance+argmin"): 283.1e6,        # assign_tc_kernel<0>
    ("bf16", "centroid sums"): 541.6e6,
    ("fp32", "distance+argmin"): 549.1e6,        # assign_f32_kernel<1>
    ("fp32", "centroid sums"): 541.6e6,
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 200 for the lloyd workload, whose iterations take "
                         "~0.4 ms, so that clock samples fall inside the timed region; 20 otherwise)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="bf16x3", choices=["bf16", "bf16x3", "fp32"],
                    help="tensor-core form of the timed arm (default bf16x3: the faster form end to end, "
                         "a fit from its seeded start; single BF16 is faster once the centroids settle; "
                         "for bigk's BF16-stored points bf16x3 is the two-term split)")
    ap.add_argument("--workload", default="lloyd", choices=["lloyd", "bigk", "kkm", "kkm-panel", "batch"],
                    help="lloyd: the headline n=1M d=128 k=256 workload (default); bigk: n=4M d=256 "
                         "k=4096 BF16 points; kkm: kernel k-means n=65536 d=512 k=64; kkm-panel: kernel "
                         "k-means n=262144 d=512 k=64 with K rebuilt in panels; batch: 512 uneven "
                         "problems x 8 restarts in one launch")
    ap.add_argument("--stages-only", action="store_true",
                    help="lloyd only: a 5-iteration fit and the per-stage timer (Lloyd.profile) of "
                         "--precision, printed as one JSON line (a short command for profilers)")
    ap.add_argument("--rows", type=int, default=0,
                    help="bigk and --stages-only: the first ROWS points of the workload instead of all n "
                         "(a smaller case for profilers)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = (200 if (args.workload == "lloyd" and args.impl == "ours")
                      else 5 if args.workload == "kkm-panel" else 20)
    args.warmup = max(args.warmup, 3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        line = reference_arm(args, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if args.stages_only:
        print(json.dumps(stages_only(args)), flush=True)
        return
    if args.workload != "lloyd":
        if rank == 0:
            line = {"bigk": bigk_arm, "kkm": kkm_arm, "kkm-panel": kkm_panel_arm,
                    "batch": batch_arm}[args.workload](args)
            print(json.dumps(line), flush=True)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    line = ours_arm(args, rank, world)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
