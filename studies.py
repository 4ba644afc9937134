"""Reproducible studies on the GPU engine (run on a CUDA host, from the
repository root):

    python studies.py precision   [--out FILE]
    python studies.py batch       [--coding msc|ssc] [--out FILE]
    python studies.py large       [--out FILE]
    python studies.py reference_large [--out FILE]
    python studies.py populations [--coding msc|ssc] [--out FILE]
    python studies.py small       [--out FILE]
    python studies.py large_clusters [--out FILE]
    python studies.py sweeps      [--out FILE]

precision: L in {32, 64, 128} (R = 1e6 at L=32, 1e5 at L=64 and 128), 100
    sweeps, dbeta=0.005, beta 0 -> 1, MSC, native stream; FP32 compensated
    resampling weights (FP64 lnQ) against all-FP64 weights; errors of betaF/N,
    E/N and C/N against the exact finite-lattice solution (Kaufman) at every
    beta, from the oracle's FP64 evaluation (the studies' checker).
batch: 64 populations with L drawn from {16,32,48,64,96,128}, R uniform in
    [1000, 20000], dbeta from {0.0025, 0.005, 0.01}, beta_final 1, 20 sweeps
    (seed 2026), annealed as one batch and as 64 sequential plain runs, MSC
    or SSC (native stream: bit planes at every one of these sizes).
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import paising_gb300 as pa  # noqa: E402
from oracle import pa_oracle  # noqa: E402


# ------------------------------------------------ exact solution (Kaufman)
def kaufman(L: int, beta: float):
    """(betaF/N, E/N, C/N) of the L x L torus from the oracle's exact
    partition function (oracle/kaufman.c, checked against enumeration and
    mpmath by tests/test_kaufman.py); the studies use it as the checker."""
    lz, e, c = pa_oracle.kaufman(L, beta)
    N = L * L
    return -lz / N, e / N, c / N


# ----------------------------------------------------------------- studies
def precision(seed: int = 31) -> dict:
    out = {"workload": "MSC, 100 sweeps, dbeta=0.005, beta 0->1, native stream", "cases": []}
    for L, R in ((32, 1_000_000), (64, 100_000), (128, 100_000)):
        case = {"L": L, "R": R}
        ex = None
        for w in ("fp32", "fp64"):
            with pa.Engine(L=L, R=R, sweeps=100, dbeta=0.005, coding="msc", weights=w, seed=seed) as e:
                e.run()
                rows = e.rows(0)
                ms, att = e.timing()
            if ex is None:
                ex = np.array([kaufman(L, b) for b in rows[:, 0]])
            case[w] = {
                "max_abs_err_betaF_per_site": float(np.max(np.abs(rows[:, 6] - ex[:, 0]))),
                "max_abs_err_E_per_site": float(np.max(np.abs(rows[1:, 1] - ex[1:, 1]))),
                "max_abs_err_C_per_site": float(np.max(np.abs(rows[1:, 2] - ex[1:, 2]))),
                "final_betaF_per_site": float(rows[-1, 6]),
                "seconds": ms / 1e3, "attempts_per_ns": att / (ms * 1e6),
                "lnQ": rows[:, 9].tolist(),
            }
        d = np.abs(np.array(case["fp32"]["lnQ"]) - np.array(case["fp64"]["lnQ"]))
        case["max_abs_lnQ_fp32_minus_fp64"] = float(d.max())
        for w in ("fp32", "fp64"):
            del case[w]["lnQ"]
        out["cases"].append(case)
        print(json.dumps(case), flush=True)
    return out


def batch(seed: int = 2026, coding: str = "msc") -> dict:
    rng = np.random.default_rng(seed)
    pops = [dict(L=int(rng.choice([16, 32, 48, 64, 96, 128])), R=int(rng.integers(1000, 20001)),
                 dbeta=float(rng.choice([0.0025, 0.005, 0.01])), sweeps=20, seed=seed + k) for k in range(64)]
    res = {"coding": coding, "populations": pops}
    for form, tune in (("batched", True), ("batched_model_tiles", False)):
        with pa.Engine.batch(pops, coding=coding) as e:
            t0 = time.perf_counter()
            tiles = e.autotune() if tune else None
            tune_s = time.perf_counter() - t0
            e.run()  # warm (graph upload)
            t0 = time.perf_counter()
            e.run()
            wall = time.perf_counter() - t0
            ms, att = e.timing()
            spw = e.sweep_form(0)["spins_per_word"]
            prof = e.profile()
        tot = sum(v[1] for v in prof.values())
        res[form] = {"device_s": ms / 1e3, "wall_s": wall, "attempts_per_ns": att / (ms * 1e6),
                     "spins_per_word": spw,
                     "kernel_share": {k: round(v[1] / tot, 4) for k, v in prof.items()}}
        if tune:
            res[form]["autotune_s"] = tune_s
            res[form]["tiles_by_L"] = {str(p["L"]): t for p, t in zip(pops, tiles)}
    tot_ms = tot_att = 0.0
    t0 = time.perf_counter()
    for p in pops:
        with pa.Engine(coding=coding, **p) as e:
            e.run()
            m, a = e.timing()
            tot_ms += m
            tot_att += a
    wall = time.perf_counter() - t0
    res["sequential_plain"] = {"device_s": tot_ms / 1e3, "wall_s_including_setup": wall,
                               "attempts_per_ns": tot_att / (tot_ms * 1e6)}
    res["speedup_device"] = res["batched"]["attempts_per_ns"] / res["sequential_plain"]["attempts_per_ns"]
    print(json.dumps({k: v for k, v in res.items() if k != "populations"}), flush=True)
    return res


def large(seed: int = 256, variants=(2, 4), sweeps: int = 50) -> dict:
    """L=256, R=131072 MSC (one group: 256 KB, swept by a thread-block
    cluster), dbeta=0.005, beta 0->1: throughput per cluster size, the
    per-kernel split of one run timed launch by launch, and betaF/N against
    the exact solution."""
    L, R = 256, 131072
    res = {"workload": f"MSC L={L} R={R} {sweeps} sweeps dbeta=0.005 beta 0->1, native stream, FP32 weights",
           "variants": {}}
    for v in variants:
        with pa.Engine(L=L, R=R, sweeps=sweeps, dbeta=0.005, coding="msc", seed=seed, sweep_variant=v) as e:
            e.run()
            rows = e.rows(0)
            ms, att = e.timing()
            prof = e.profile()
        ex = np.array([kaufman(L, b) for b in rows[:, 0]])
        r = {"seconds": ms / 1e3, "attempts_per_ns": att / (ms * 1e6),
             "max_abs_err_betaF_per_site": float(np.max(np.abs(rows[:, 6] - ex[:, 0]))),
             "max_abs_err_E_per_site": float(np.max(np.abs(rows[1:, 1] - ex[1:, 1]))),
             "kernels_ms": {k: [n, t] for k, (n, t) in prof.items()}}
        res["variants"][str(v)] = r
        print(json.dumps({"variant": v, **r}), flush=True)
    return res


def reference_large(seed: int = 256, sweeps: int = 50) -> dict:
    """The reference's own MSC program (PAisingMSC.cu with #define L 256,
    cuRAND, built by oracle/ref_build.py) on the same workload as large():
    its whole-anneal seconds and attempts/ns as it reports them, and the
    errors of its results file against the exact solution."""
    import re
    import subprocess
    import tempfile
    from oracle import ref_build
    L, R = 256, 131072
    binp = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle", "_ref", "bin",
                        f"PAisingMSC_L{L}_curand")
    if not os.path.exists(binp):
        ref_build.main(["--sizes", str(L)])
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([binp, "-R", str(R), "-t", str(sweeps), "-d", "0.005", "-s", str(seed), "-o", d],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stdout[-800:] + r.stderr[-800:])
        rows = np.loadtxt(os.path.join(d, "PA_results_run_0.dat"))
    el = float(re.search(r"Elapsed time:\s*([0-9.eE+-]+)", r.stdout).group(1))
    tpf = float(re.search(r"Time per spin-flip:\s*([0-9.eE+-]+)", r.stdout).group(1))
    ex = np.array([kaufman(L, b) for b in rows[:, 0]])
    res = {"program": f"PAisingMSC.cu, L={L}, cuRAND (its own build)", "R": R, "sweeps": sweeps, "seed": seed,
           "seconds": el, "attempts_per_ns": 1.0 / tpf,
           "max_abs_err_betaF_per_site": float(np.max(np.abs(rows[:, 6] - ex[:, 0]))),
           "max_abs_err_E_per_site": float(np.max(np.abs(rows[1:, 1] - ex[1:, 1]))),
           "beta_at_max_betaF_err": float(rows[np.argmax(np.abs(rows[:, 6] - ex[:, 0])), 0]),
           "rows": len(rows)}
    print(json.dumps(res), flush=True)
    return res


def populations(counts=(1, 2, 4, 8, 16, 32), coding: str = "msc") -> dict:
    """The headline anneal (L=64, R=20000, 100 sweeps, dbeta=0.005) with P
    independent populations per launch sequence: attempts/ns as P grows (the
    batched form's gain over the plain one-population form)."""
    import torch
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    res = {"workload": f"{coding.upper()} L=64 R=20000 100 sweeps dbeta=0.005 beta 0->1, native stream, FP32 "
                       "weights, graph", "by_populations": {}}
    for P in counts:
        with pa.Engine(L=64, R=20000, sweeps=100, dbeta=0.005, runs=P, seed=500 + P, coding=coding) as e:
            e.run()
            ms = att = 0.0
            for _ in range(2):
                flush.zero_()
                torch.cuda.synchronize()
                e.run()
                m, a = e.timing()
                ms += m
                att += a
        r = {"attempts_per_ns": att / (ms * 1e6), "s_per_population_anneal": ms / 2 / 1e3 / P}
        res["by_populations"][str(P)] = r
        print(json.dumps({"P": P, **r}), flush=True)
    return res


def small(cases=((64, (2500, 5000, 7500, 10000, 12500, 15000, 20000, 25000, 30000, 40000, 100000)),
                  (96, (2000, 5000, 10000, 20000)),
                  (128, (1000, 2000, 5000, 10000, 15000, 20000, 30000, 40000, 100000)),
                  (48, (5000, 20000)))) -> dict:
    """Single populations too small to fill the GPU with one CTA per group:
    the one-CTA sweep (sweep_variant=1) against the engine's automatic form
    (clusters of 2 or 4 CTAs per group where the groups are too few) and
    against each cluster size forced; MSC, native stream, 100 sweeps up to
    L=64, 50 above, dbeta=0.005."""
    import torch
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    res = {"cases": []}
    for L, Rs in cases:
        for R in Rs:
            row = {"L": L, "R": R, "groups": (R + 31) // 32}
            for name, v in (("one_cta", 1), ("automatic", 0), ("clusters2", 2), ("clusters4", 4)):
                with pa.Engine(L=L, R=R, sweeps=100 if L <= 64 else 50, dbeta=0.005, seed=7, coding="msc",
                               sweep_variant=v) as e:
                    e.run()
                    ms = att = 0.0
                    for _ in range(2):
                        flush.zero_()
                        torch.cuda.synchronize()
                        e.run()
                        m, a = e.timing()
                        ms += m
                        att += a
                    row[name] = round(att / (ms * 1e6), 1)
                    if v == 0:
                        row["automatic_cluster_ctas"] = e.sweep_form(0)["cluster_ctas"]
            res["cases"].append(row)
            print(json.dumps(row), flush=True)
    return res


def large_clusters(cases=((256, (1000, 2000, 2600, 3000, 8000, 20000, 65536)), (224, (3000, 20000)),
                           (192, (1000, 3000, 8000, 30000)), (160, (1000, 5000, 20000)), (144, (3000,)))) -> dict:
    """Lattices above L = 128 (a group needs a cluster) with few groups:
    clusters of 2 CTAs (1024 threads) against clusters of 4 (512 threads),
    the engine's automatic choice and pa_autotune's; MSC, native stream, 50
    sweeps, dbeta=0.05 up to beta = 1 (20 temperatures, whole anneals)."""
    import torch
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    res = {"cases": []}
    for L, Rs in cases:
        for R in Rs:
            row = {"L": L, "R": R, "groups": (R + 31) // 32}
            for name, v in (("automatic", 0), ("clusters2", 2), ("clusters4", 4), ("autotuned", 0)):
                with pa.Engine(L=L, R=R, sweeps=50, dbeta=0.05, seed=7, coding="msc", sweep_variant=v) as e:
                    if name == "autotuned":
                        e.autotune()
                    e.run()
                    ms = att = 0.0
                    for _ in range(2):
                        flush.zero_()
                        torch.cuda.synchronize()
                        e.run()
                        m, a = e.timing()
                        ms += m
                        att += a
                    row[name] = round(att / (ms * 1e6), 1)
                    if v == 0:
                        row[name + "_cluster_ctas"] = e.sweep_form(0)["cluster_ctas"]
            res["cases"].append(row)
            print(json.dumps(row), flush=True)
    return res


def sweeps(cases=((64, 524288), (128, 131072), (256, 32768), (16, 524288)), counts=(5, 20, 100)) -> dict:
    """Whole anneals with few and many sweeps per temperature: MSC, native
    stream, FP32 weights, dbeta=0.05 up to beta = 1 (20 temperatures: strong
    reweighting, so a few replicas take many copies), one population of each
    size; attempts/ns (best of three runs after a warm-up, L2 flushed before
    each) and the per-kernel device time of one further run."""
    import torch
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    res = {"cases": []}
    for L, R in cases:
        for sw in counts:
            with pa.Engine(L=L, R=R, sweeps=sw, dbeta=0.05, beta_final=1.0, seed=7, coding="msc") as e:
                e.run()
                best = None
                for _ in range(3):
                    flush.zero_()
                    torch.cuda.synchronize()
                    e.run()
                    m, a = e.timing()
                    if best is None or m < best[0]:
                        best = (m, a)
                prof = e.profile()
            row = {"L": L, "R": R, "sweeps": sw, "attempts_per_ns": round(best[1] / (best[0] * 1e6), 1),
                   "anneal_ms": round(best[0], 2),
                   "kernels_ms": {k: round(v[1], 3) for k, v in prof.items()}}
            res["cases"].append(row)
            print(json.dumps(row), flush=True)
    return res


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["precision", "batch", "large", "reference_large", "populations", "small",
                                          "large_clusters", "sweeps"])
    ap.add_argument("--out", default=None)
    ap.add_argument("--coding", choices=["msc", "ssc"], default="msc", help="batch study: spin coding")
    a = ap.parse_args(argv)
    r = batch(coding=a.coding) if a.study == "batch" else \
        {"precision": precision, "large": large, "reference_large": reference_large,
         "populations": lambda: populations(coding=a.coding), "small": small,
         "large_clusters": large_clusters, "sweeps": sweeps}[a.study]()
    if a.out:
        json.dump(r, open(a.out, "w"), indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
