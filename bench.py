#!/usr/bin/env python
"""Headline benchmark: spin-flip attempts per ns of a full population-annealing
run of the 2D Ising ferromagnet at L=64, R=20000, 100 sweeps per temperature,
dbeta=0.005, beta 0 -> 1 (199 temperatures), the reference's sample shape.

One "step" is one full anneal of the batch (P independent populations run
concurrently by one engine; P=1 is the plain single-population form).  The
metric is the reference's own (PAisingSSC.cu:632,806):
    attempts = sweeps * N * sum_{i>=1} R_i,   value = attempts / device ns.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference runs the reference's own CUDA program (PAisingMSC.cu built
with cuRAND by oracle/ref_build.py) on the same GPU, the same number of
populations per step (its -M flag), and reports its own timing; the SSC
program's figure rides along as "other_coding".  Under torchrun with N > 1 each rank anneals its own populations
(replicas only; the path has no data-parallel exchange) and rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PROFILES = os.path.join(ROOT, "profiles")
METRIC = "spin-flip attempts/ns (full anneal, L=64 R=20000 100 sweeps dbeta=0.005)"
UNIT = "attempts/ns"


# ----------------------------------------------------------------- helpers
def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--coding", choices=["msc", "ssc"], default="msc")
    ap.add_argument("--populations", type=int, default=8,
                    help="independent populations per engine launch (the batched form; 1 = plain)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain single-population comparison")
    ap.add_argument("--L", type=int, default=64)
    ap.add_argument("--R", type=int, default=20000)
    ap.add_argument("--sweeps", type=int, default=100)
    ap.add_argument("--dbeta", type=float, default=0.005)
    ap.add_argument("--beta-final", type=float, default=1.0)
    ap.add_argument("--graph", type=int, default=1)
    ap.add_argument("--cpu-sample-steps", type=int, default=12,
                    help="temperatures in the CPU baseline sample (about 10 s of CPU work on 16 cores)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-profile", action="store_true")
    return ap.parse_args(argv)


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.proc, self.lines = gpu, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_profile_traffic(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary."""
    p = os.path.join(PROFILES, "ncu_summary.json")
    try:
        d = json.load(open(p))
        return d[kernel][workload]["dram_bytes_per_launch"]
    except (OSError, KeyError, ValueError):
        return None


def dist_init():
    """(rank, local rank, world size, torch.distributed or None) of a
    torchrun launch; one rank per GPU (NCCL), gloo where no GPU is present."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws == 1:
        return 0, 0, 1, None
    import torch
    import torch.distributed as dist
    rank, lrank = int(os.environ["RANK"]), int(os.environ.get("LOCAL_RANK", "0"))
    if torch.cuda.is_available():
        torch.cuda.set_device(lrank)
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, lrank, ws, dist


def rank_seed(rank: int) -> int:
    """Seed of the populations rank `rank` anneals: the ranks run independent
    replicas of the workload (no data-parallel exchange on this path)."""
    return 1000 + 97 * rank


def reduce_over_ranks(dist, device, elapsed: float, attempts: float):
    """Whole-job figures of a multi-rank run: the slowest rank's time and the
    attempts of all ranks (MAX and SUM all-reduces; identity on one rank)."""
    if not dist:
        return elapsed, attempts
    import torch
    t = torch.tensor([elapsed, attempts], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return mx[0].item(), t[1].item()


# ------------------------------------------------------------- the workload
def schedule_steps(dbeta: float, beta_final: float) -> int:
    """Temperatures after beta = 0 of the reference's schedule: beta
    accumulated as B[i] = B[i-1] + dbeta while B[i] <= beta_final
    (PAisingSSC.cu:508-510)."""
    b, n = 0.0, 0
    while b + dbeta <= beta_final and n < 10000:
        b += dbeta
        n += 1
    return n


def workload_config(a, ws: int) -> dict:
    """The workload both arms run, described identically: P independent
    populations of the anneal per step (how an arm schedules them is
    reported outside this dict)."""
    P = a.populations
    nsteps = schedule_steps(a.dbeta, a.beta_final)
    return {"workload": f"PA anneal {a.coding.upper()} L={a.L} R={a.R} sweeps={a.sweeps} dbeta={a.dbeta} beta 0->"
                        f"{a.beta_final} ({nsteps} temperatures), {P} independent population(s) per step",
            "L": a.L, "R": a.R, "sweeps": a.sweeps, "dbeta": a.dbeta, "beta_final": a.beta_final,
            "coding": a.coding, "populations": P, "parallelism": f"replicas x{ws}",
            "l2": "flushed between timed steps (256 MB write)"}


# ------------------------------------------------------------- our engine
def engine_kwargs(a, seed: int, device: int) -> dict:
    """The timed engine: P populations of the workload in one launch
    sequence, native stream, FP32-compensated weights, CUDA graph."""
    return dict(L=a.L, R=a.R, sweeps=a.sweeps, dbeta=a.dbeta, beta_final=a.beta_final, runs=a.populations,
                seed=seed, coding=a.coding, rng="native", weights="fp32", graph=bool(a.graph), device=device)


def cpu_baseline(a) -> dict:
    """The oracle (C restatement of the reference's MSC/SSC loop, OpenMP over
    replicas) on this host's cores, over the first few temperatures of the
    same workload."""
    from oracle import pa_oracle
    threads = os.cpu_count() or 1
    pa_oracle.set_threads(threads)
    t0 = time.perf_counter()
    _, att = pa_oracle.anneal(a.coding, a.L, a.R, a.sweeps, a.dbeta, a.beta_final, 1, 7,
                              max_steps=a.cpu_sample_steps)
    dt = time.perf_counter() - t0
    return {"value": att / (dt * 1e9), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{a.coding.upper()} L={a.L} R={a.R} {a.sweeps} sweeps, initialisation + first "
                      f"{a.cpu_sample_steps} temperatures ({att:.3g} attempts in {dt:.1f} s)"}


def run_ours(a):
    import numpy as np
    import torch

    import paising_gb300 as pa

    rank, lrank, ws, dist = dist_init()
    dev = lrank
    torch.cuda.set_device(dev)
    P = a.populations
    eng = pa.Engine(**engine_kwargs(a, rank_seed(rank), dev))
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{dev}")  # > L2 (129 MB)
    for _ in range(a.warmup):
        eng.run()
    nsteps = eng.num_rows() - 1
    # one launch sequence serves all P populations: 5 kernels to initialise,
    # 8 per temperature (q, copy numbers, scatter, gather plan, gather, sweep
    # plan, sweep, finish), 9 for MSC (the gather's pair-list pass)
    launches_per_run = 5 + (9 if a.coding == "msc" else 8) * nsteps

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)

    ms_steps, att_steps = [], []
    with ClockSampler(dev) as clk:
        barrier()
        for _ in range(a.steps):
            flush.zero_()  # evict L2 between timed steps (outside the timed region)
            torch.cuda.synchronize(dev)
            eng.run()
            ms, att = eng.timing()
            ms_steps.append(ms)
            att_steps.append(att)
        barrier()
    tot_ms_max, tot_att_all = reduce_over_ranks(dist, f"cuda:{dev}", sum(ms_steps), sum(att_steps))
    value = tot_att_all / (tot_ms_max * 1e6)

    # end to end through the C ABI with host buffers: every step uploads the
    # initial populations from pinned host memory (pa_set_population), runs,
    # and reads the result rows back (pa_get_rows); host wall clock.
    N = a.L * a.L
    pop_bytes = P * (((a.R + 31) // 32) * N * 4 if a.coding == "msc" else a.R * N)
    host_pop = torch.empty(pop_bytes, dtype=torch.uint8, pin_memory=True)
    rng = np.random.default_rng(rank)
    host_np = host_pop.numpy()
    if a.coding == "msc":
        host_np[:] = rng.integers(0, 256, pop_bytes, dtype=np.uint8)
    else:
        host_np[:] = np.where(rng.integers(0, 2, pop_bytes) > 0, 1, -1).astype(np.int8).view(np.uint8)
    e2e_s, e2e_att = [], 0.0
    rows_bytes = 0
    for i in range(a.steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        eng.set_population(host_pop.data_ptr())
        eng.run()
        rows = [eng.rows(r) for r in range(P)]
        e2e_s.append(time.perf_counter() - t0)
        e2e_att += eng.timing()[1]
        rows_bytes = sum(r.nbytes for r in rows)
    eng.set_population(None)
    e2e_tot, e2e_att = reduce_over_ranks(dist, f"cuda:{dev}", sum(e2e_s), e2e_att)
    e2e_value = e2e_att / (e2e_tot * 1e9)

    out = None
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": tot_ms_max / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u32 bit-planes (int32 energies, fp32-compensated weights, fp64 lnQ)" if a.coding == "msc"
            else "i8 spins (int32 energies, fp32-compensated weights, fp64 lnQ)",
            "data": "synthetic (random initial spins from the seed, native Philox stream)",
            "config": workload_config(a, ws),
            "schedule": {"populations_per_launch": P, "graph": bool(a.graph),
                         "how": "all populations of a step in the same launches (persistent kernels), the whole "
                                "schedule one CUDA graph"},
            "full_anneal_s": tot_ms_max / a.steps / 1e3,
            "full_anneal_s_per_population": tot_ms_max / a.steps / 1e3 / P,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": pop_bytes,
                    "d2h_bytes_per_step": rows_bytes + 4 * P},
            "gpu_launches": launches_per_run * a.steps,
            "clocks": clk.summary(),
        }
        if not a.no_profile:
            out.update(profile_leg(a, eng, pa))
        if not a.no_plain and P > 1:
            out["plain"] = plain_leg(a, dev, flush)
            out["other_coding"] = other_coding_leg(a, dev, flush)
        if not a.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(a)
    eng.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return out


def plain_leg(a, dev, flush) -> dict:
    """The plain form on the same GPU: one population per launch sequence,
    the host stepping every temperature and synchronising after it."""
    import torch

    import paising_gb300 as pa
    out = {}
    for graph in (False, True):
        with pa.Engine(L=a.L, R=a.R, sweeps=a.sweeps, dbeta=a.dbeta, beta_final=a.beta_final, runs=1, seed=4242,
                       coding=a.coding, rng="native", weights="fp32", graph=graph, device=dev) as e:
            e.run()
            ms, att = [], []
            for _ in range(a.steps):
                flush.zero_()
                torch.cuda.synchronize(dev)
                e.run()
                t, n = e.timing()
                ms.append(t)
                att.append(n)
        key = "graph" if graph else "host_stepped"
        out[key] = {"value": sum(att) / (sum(ms) * 1e6), "unit": UNIT, "ms_per_anneal": sum(ms) / len(ms)}
    return out


def other_coding_leg(a, dev, flush) -> dict:
    """The same workload in the other coding (SSC for an MSC run and vice
    versa): batched like the headline and plain (one population, graph)."""
    import torch

    import paising_gb300 as pa
    coding = "ssc" if a.coding == "msc" else "msc"
    out = {"coding": coding}
    for key, runs in (("batched", a.populations), ("plain_graph", 1)):
        with pa.Engine(L=a.L, R=a.R, sweeps=a.sweeps, dbeta=a.dbeta, beta_final=a.beta_final, runs=runs, seed=777,
                       coding=coding, rng="native", weights="fp32", graph=True, device=dev) as e:
            e.run()
            ms, att = [], []
            for _ in range(max(1, a.steps // 2)):
                flush.zero_()
                torch.cuda.synchronize(dev)
                e.run()
                t, n = e.timing()
                ms.append(t)
                att.append(n)
        out[key] = {"value": sum(att) / (sum(ms) * 1e6), "unit": UNIT, "ms_per_anneal": sum(ms) / len(ms),
                    "populations": runs}
    return out


def profile_leg(a, eng, pa) -> dict:
    """Per-kernel device times of one run (CUDA events around each launch on
    the engine's stream) and the roofline of the dominant kernel."""
    prof = eng.profile()
    tot = sum(v[1] for v in prof.values())
    N = a.L * a.L
    # replicas swept per launch: all populations of the batch at one temperature
    Rs = sum(eng.rows(k)[1:, 8] for k in range(eng.num_sets()))
    sweep = f"{a.coding}_sweep"
    n_launch, sweep_ms = prof[sweep]
    avg_ms = sweep_ms / n_launch
    attempts_per_launch = a.sweeps * N * Rs.mean()
    # algorithmic INT32 operations per spin-flip attempt: MSC ~5 (bitsliced
    # neighbour count and acceptance mask shared by 32 replicas), SSC ~33 (a
    # 32-bit Philox word, ~25 operations, plus the update of one site).  The
    # native SSC sweep on bit planes (32 sites per word) does the bitsliced
    # work of the MSC figure.
    ssc_bits = a.coding == "ssc" and eng.sweep_form(0)["spins_per_word"] == 32
    ops_per_attempt = 5.0 if a.coding == "msc" or ssc_bits else 33.0
    achieved = attempts_per_launch * ops_per_attempt / (avg_ms * 1e-3) / 1e12
    from bench_probe import build as probe
    peaks = probe.probe_int_issue(eng.config.device)
    peak = max(peaks) / 1e12
    workload = f"L{a.L}_R{a.R}_sw{a.sweeps}"
    return {
        "kernels": {k: {"launches": v[0], "total_ms": v[1], "share": v[1] / tot} for k, v in prof.items()},
        "roofline": {"kernel": sweep, "bound": "int32", "achieved": achieved, "peak": peak, "unit": "Tops/s",
                     "frac": achieved / peak,
                     # ncu DRAM bytes of one single-population launch, scaled by the populations per launch
                     "traffic": (lambda t: None if t is None else t * eng.num_sets())(load_profile_traffic(sweep, workload)),
                     "ops_per_attempt": ops_per_attempt, "attempts_per_launch": attempts_per_launch,
                     "avg_launch_ms": avg_ms,
                     "peak_source": "measured in-process: integer lane-op issue rate of independent LOP3 (ALU "
                                    f"pipe) and IMAD (FMA pipe) chains, ALU-only {peaks[0] / 1e12:.1f}, FMA-only "
                                    f"{peaks[1] / 1e12:.1f}, alternating {peaks[2] / 1e12:.1f} Tops/s; the sweep "
                                    "uses both pipes: peak = the largest"},
    }


# -------------------------------------------------------- reference program
def _reference_binary(prog: str, L: int):
    """oracle/_ref/bin/PAising<prog>_L<L>_curand, built from the patched
    reference sources when missing; (path, None) or (None, why)."""
    from oracle import ref_build
    binp = os.path.join(ROOT, "oracle", "_ref", "bin", f"PAising{prog}_L{L}_curand")
    if not os.path.exists(binp):
        try:
            ref_build.main(["--sizes", str(L)])
        except Exception as ex:  # noqa: BLE001
            return None, f"reference build failed: {str(ex)[:200]}"
    if not os.path.exists(binp):
        return None, f"reference sources for L={L} not present"
    return binp, None


def _reference_once(binp: str, a, seed: int, runs: int):
    """One invocation of the reference program: `runs` populations one after
    the other (its -M flag); (elapsed s, spin-flip attempts) as it reports
    them (PAisingMSC.cu:956-957: Elapsed time, Time per spin-flip over the
    attempts of all runs)."""
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([binp, "-R", str(a.R), "-t", str(a.sweeps), "-d", str(a.dbeta), "-f",
                            str(a.beta_final), "-s", str(seed), "-M", str(runs), "-o", d],
                           capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-500:] + r.stderr[-500:])
    el = float(re.search(r"Elapsed time:\s*([0-9.eE+-]+)", r.stdout).group(1))
    tpf = float(re.search(r"Time per spin-flip:\s*([0-9.eE+-]+)", r.stdout).group(1))
    return el, el * 1e9 / tpf


def run_reference(a):
    """The reference's own CUDA program on the same GPU and workload: each
    step is one invocation annealing the same number of populations as our
    batch, one after the other (-M populations), timed by the program itself.
    The other coding's program is timed once on one population as an extra
    figure."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    prog = "MSC" if a.coding == "msc" else "SSC"
    binp, why = _reference_binary(prog, a.L)
    if binp is None:
        return {"impl": "reference", "unavailable": why}
    P = a.populations
    flush = None
    try:  # the same L2 flush between steps as our arm (L2 is the GPU's, whichever process writes it)
        import torch
        if torch.cuda.is_available():
            flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    except ImportError:
        pass
    for w in range(a.warmup):
        _reference_once(binp, a, 1 + w, 1)
    els, atts = [], []
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for k in range(a.steps):
            if flush is not None:
                flush.zero_()
                torch.cuda.synchronize()
            el, att = _reference_once(binp, a, 100 + k, P)
            els.append(el)
            atts.append(att)
    value = sum(atts) / (sum(els) * 1e9)
    sample = f"PAising{prog}.cu (L={a.L}, MSbits=32) built with cuRAND, {P} population(s) per step (-M {P}), " \
             "timed by the program's own CUDA events (Elapsed time / Time per spin-flip)"
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1e3 * sum(els) / len(els), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32 bit-planes" if a.coding == "msc" else "i8 spins",
        "data": "synthetic (random initial spins from the seed, cuRAND Philox)",
        "config": workload_config(a, 1),
        "schedule": {"how": f"one invocation of the program per step with -M {P}: the populations one after the "
                            "other, each with the reference's own launches and host synchronisation"},
        "full_anneal_s": sum(els) / len(els),
        "full_anneal_s_per_population": sum(els) / len(els) / P,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "reference",
                         "sample": sample + " (GPU program; one host thread drives it)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "clocks": clk.summary(),
    }
    if not a.no_plain:
        other = "SSC" if prog == "MSC" else "MSC"
        ob, why = _reference_binary(other, a.L)
        if ob is None:
            out["other_coding"] = {"coding": other.lower(), "unavailable": why}
        else:
            el, att = _reference_once(ob, a, 100, 1)
            out["other_coding"] = {"coding": other.lower(), "value": att / (el * 1e9), "unit": UNIT,
                                   "full_anneal_s": el, "populations": 1,
                                   "program": f"PAising{other}.cu built with cuRAND (one population)"}
    return out


def main(argv=None) -> int:
    a = parse_args(argv)
    out = run_reference(a) if a.impl == "reference" else run_ours(a)
    if out is not None:
        print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
