"""Adaptive temperature step (the reference's AdaptiveStep build): after every
temperature the device chooses the next one from the overlap of the energy
histogram, in the same kernel sequence (graph chunks or host steps).  Under
the reference stream the schedule, population sizes and observables must
equal the reference program built with -DAdaptiveStep."""
import numpy as np
import pytest

import paising_gb300 as pa
from conftest import compare_rows, load_dat

pytestmark = pytest.mark.gpu


def run(**kw):
    with pa.Engine(**kw) as e:
        e.run()
        return [e.rows(r) for r in range(e.num_sets())], e.num_rows()


@pytest.mark.parametrize("coding", ["ssc", "msc"])
@pytest.mark.parametrize("graph", [True, False])
def test_adaptive_reference(cuda, coding, graph):
    rows, n = run(L=16, R=1000, sweeps=10, seed=100, coding=coding, rng="reference", weights="fp64", graph=graph,
                  adaptive=True)
    ref = load_dat(f"ref/inj_{coding.upper()}_L16_R1000_t10_d0.005_s100_adaptive.dat")
    assert n == len(ref) == len(rows[0])
    compare_rows(rows[0], ref, rtol=2e-10)


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_adaptive_two_runs_replay_schedule(cuda, coding):
    rows, _ = run(L=16, R=1000, sweeps=10, seed=7, runs=2, dbeta=0.01, coding=coding, rng="reference",
                  weights="fp64", adaptive=True)
    for r in range(2):
        compare_rows(rows[r], load_dat(f"ref/inj_{coding.upper()}_L16_R1000_t10_d0.01_s7_M2_adaptive_run{r}.dat"),
                     rtol=2e-10)
    assert np.array_equal(rows[0][:, 0], rows[1][:, 0])


def test_adaptive_in_a_batch(cuda, oracle):
    """Adaptive and fixed-schedule populations in one batch, each equal to
    the oracle's run of it.  Successive pa_run calls continue the handle's
    sequence of runs: the stream goes on and the first run's schedule is
    replayed, as the reference's later runs do."""
    pops = [dict(L=16, R=800, sweeps=4, dbeta=0.01, seed=11, adaptive=True),
            dict(L=24, R=400, sweeps=3, dbeta=0.05, seed=12),
            dict(L=32, R=600, sweeps=2, dbeta=0.02, beta_final=0.7, seed=13, adaptive=True, min_overlap=0.6,
                 max_overlap=0.7)]
    refs = [oracle.anneal("msc", p["L"], p["R"], p["sweeps"], p["dbeta"], p.get("beta_final", 1.0), 2, p["seed"],
                          adaptive=p.get("adaptive", False), min_overlap=p.get("min_overlap", 0.85),
                          max_overlap=p.get("max_overlap", 0.87))[0] for p in pops]
    with pa.Engine.batch(pops, coding="msc", rng="reference", weights="fp64") as e:
        for run_index in range(2):
            e.run()
            for k in range(len(pops)):
                compare_rows(e.rows(k), refs[k][run_index], rtol=1e-9)


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_adaptive_native_free_energy(cuda, oracle, coding):
    """Native stream, FP32 weights, L=32, R=20000: the adaptive schedule ends
    on beta=1 and betaF/N stays within 1e-4 of the exact value."""
    rows, _ = run(L=32, R=20000, sweeps=20, seed=3, coding=coding, adaptive=True)
    r = rows[0]
    assert r[-1, 0] == 1.0 and np.all(np.diff(r[:, 0]) > 0)
    exact = np.array([-oracle.kaufman(32, b)[0] / 1024 for b in r[:, 0]])
    assert np.max(np.abs(r[:, 6] - exact)) < 1e-4


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_cli_adaptive(cuda, tmp_path, coding):
    """The command-line driver's -a switch (and -T, the autotuner) against the
    AdaptiveStep build's results file."""
    import os
    import subprocess
    from conftest import ROOT
    exe = os.path.join(ROOT, "paising_gb300", "_lib", "paising")
    r = subprocess.run([exe, "-R", "1000", "-t", "10", "-L", "16", "-s", "100", "-c", coding, "-m", "reference",
                        "-w", "fp64", "-a", "-T", "-o", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.loadtxt(tmp_path / "PA_results_run_0.dat")
    compare_rows(got, load_dat(f"ref/inj_{coding.upper()}_L16_R1000_t10_d0.005_s100_adaptive.dat"), rtol=2e-10)
