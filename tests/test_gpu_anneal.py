"""Whole-anneal parity: the engine (through pa_create / pa_run) against the
reference programs' own outputs under the injected stream.  With the
reference-coordinate stream and FP64 weights every population size R_i must
match exactly and every other column to print precision, for all 200
temperatures.  Plus size-independent invariants and physics checks of the
native (production) configuration."""
import numpy as np
import pytest

import paising_gb300 as pa
from conftest import compare_rows, load_dat

pytestmark = pytest.mark.gpu


def run(**kw):
    with pa.Engine(**kw) as e:
        e.run()
        rows = [e.rows(r) for r in range(e.num_sets())]
        return rows, e.timing()


@pytest.mark.parametrize("coding", ["ssc", "msc"])
@pytest.mark.parametrize("graph", [True, False])
def test_reference_C1(cuda, coding, graph):
    rows, _ = run(L=16, R=1000, sweeps=10, seed=100, coding=coding, rng="reference", weights="fp64", graph=graph)
    compare_rows(rows[0], load_dat(f"ref/inj_{coding.upper()}_L16_R1000_t10_d0.005_s100.dat"), rtol=2e-10)


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_reference_two_runs(cuda, coding):
    rows, _ = run(L=16, R=1000, sweeps=10, seed=7, runs=2, coding=coding, rng="reference", weights="fp64")
    for r in range(2):
        compare_rows(rows[r], load_dat(f"ref/inj_{coding.upper()}_L16_R1000_t10_d0.005_s7_M2_run{r}.dat"), rtol=2e-10)


@pytest.mark.slow
@pytest.mark.parametrize("coding", ["msc", "ssc"])
def test_reference_C2_L64(cuda, coding):
    """The reference's sample shape: L=64, R=20000, 100 sweeps, seed 100."""
    rows, _ = run(L=64, R=20000, sweeps=100, seed=100, coding=coding, rng="reference", weights="fp64")
    compare_rows(rows[0], load_dat(f"ref/inj_{coding.upper()}_L64_R20000_t100_d0.005_s100.dat"), rtol=2e-10)


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_fp32_weights_track_fp64(cuda, coding):
    """Same stream, FP32 compensated weights: lnQ per step within 1e-6 of the
    FP64 run while the populations coincide, betaF/N within 1e-6 at the end."""
    a, _ = run(L=16, R=1000, sweeps=10, seed=100, coding=coding, rng="reference", weights="fp64")
    b, _ = run(L=16, R=1000, sweeps=10, seed=100, coding=coding, rng="reference", weights="fp32")
    a, b = a[0], b[0]
    same = np.cumprod(a[:, 8] == b[:, 8]).astype(bool)
    k = int(same.sum())
    assert k >= 5
    assert np.max(np.abs(a[1:k, 9] - b[1:k, 9])) < 1e-6


def test_invariants_native(cuda):
    """Population size stays within the buffer, energies per site within
    [-2, 2], |M| <= 1, and E/N is monotone-ish decreasing in beta."""
    rows, (ms, att) = run(L=32, R=5000, sweeps=20, seed=3, coding="msc")
    r = rows[0]
    assert np.all(r[:, 8] > 0) and np.all(r[:, 8] <= 1.25 * 5000 + 256)
    assert np.all(np.abs(r[1:, 1]) <= 2) and np.all((r[1:, 3] >= 0) & (r[1:, 3] <= 1))
    assert r[-1, 1] < -1.9 and ms > 0 and att == pytest.approx(20 * 1024 * r[1:, 8].sum())


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_native_free_energy_vs_kaufman_L16(cuda, oracle, coding):
    """Native stream, FP32 weights, L=16, R=20000, 20 sweeps: betaF/N against
    the exact finite-lattice value within 3e-4 at every beta (the finite-R
    bias of population annealing at this size is ~1e-4)."""
    rows, _ = run(L=16, R=20000, sweeps=20, seed=12, coding=coding)
    r = rows[0]
    exact = np.array([-oracle.kaufman(16, b)[0] / 256 for b in r[:, 0]])
    assert np.max(np.abs(r[:, 6] - exact)) < 3e-4


@pytest.mark.slow
@pytest.mark.parametrize("coding", ["msc", "ssc"])
def test_native_free_energy_vs_kaufman_C2(cuda, oracle, coding):
    """The accuracy target at L=64, R=20000, 100 sweeps, dbeta=0.005:
    |betaF/N - exact| <= 1e-4 at every beta, native stream, FP32 weights."""
    rows, _ = run(L=64, R=20000, sweeps=100, seed=2026, coding=coding)
    r = rows[0]
    exact = np.array([-oracle.kaufman(64, b)[0] / 4096 for b in r[:, 0]])
    err = np.abs(r[:, 6] - exact)
    assert err.max() <= 1e-4, (err.max(), r[np.argmax(err), 0])
    eE = np.array([oracle.kaufman(64, b)[1] / 4096 for b in r[1:, 0]])
    assert np.max(np.abs(r[1:, 1] - eE)) < 5e-3


@pytest.mark.slow
def test_benchmarked_configuration_every_population_vs_kaufman(cuda, oracle):
    """The headline workload exactly as bench.py builds it (L=64, R=20000,
    100 sweeps, dbeta=0.005, 8 populations per launch, native stream, FP32
    weights, CUDA graph): every population meets |betaF/N - exact| <= 1e-4
    at every beta and |E/N - exact| < 5e-3, against Kaufman's finite-torus
    solution in FP64."""
    import bench
    a = bench.parse_args([])
    with pa.Engine(**bench.engine_kwargs(a, seed=bench.rank_seed(0), device=0)) as e:
        e.run()
        assert e.num_sets() == a.populations == 8
        rows = [e.rows(k) for k in range(e.num_sets())]
    N = a.L * a.L
    betas = rows[0][:, 0]
    exact = np.array([oracle.kaufman(a.L, b) for b in betas])
    bf_exact, e_exact = -exact[:, 0] / N, exact[:, 1] / N
    assert len({tuple(r[1:20, 8]) for r in rows}) == len(rows)
    for k, r in enumerate(rows):
        assert np.array_equal(r[:, 0], betas)
        err = np.abs(r[:, 6] - bf_exact)
        assert err.max() <= 1e-4, (k, err.max(), r[np.argmax(err), 0])
        assert np.max(np.abs(r[1:, 1] - e_exact[1:])) < 5e-3, k


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_population_roundtrip(cuda, coding):
    """pa_set_population / pa_get_population: with no temperature step
    (dbeta > beta_final) the final population is the uploaded one, and its
    energies give the beta=0 row's statistics."""
    L, R = 16, 100
    rng = np.random.default_rng(5)
    if coding == "ssc":
        pop = np.where(rng.integers(0, 2, (R, L * L)) > 0, 1, -1).astype(np.int8)
    else:
        pop = rng.integers(0, 2**32, ((R + 31) // 32, L * L), dtype=np.uint32)
    with pa.Engine(L=L, R=R, sweeps=5, dbeta=2.0, beta_final=1.0, coding=coding) as e:
        e.set_population(pop)
        e.run()
        assert e.num_rows() == 1
        assert np.array_equal(e.population(), pop)
        e.set_population(None)
        e.run()
        assert not np.array_equal(e.population(), pop)


BATCH = [dict(L=16, R=300, sweeps=5, dbeta=0.05, seed=100), dict(L=24, R=500, sweeps=3, dbeta=0.1, seed=7),
         dict(L=8, R=90, sweeps=7, dbeta=0.04, beta_final=0.6, seed=3), dict(L=32, R=200, sweeps=2, dbeta=0.2, seed=11)]


@pytest.mark.parametrize("coding", ["ssc", "msc"])
@pytest.mark.parametrize("graph", [True, False])
def test_batch_uneven_reference_stream(cuda, oracle, coding, graph):
    """Uneven populations (L, R, sweeps, dbeta, beta_final, seed) annealed in
    one batch: each result set equals the oracle's run of that population
    alone, bit for bit in R and to print precision elsewhere."""
    pops = BATCH if coding == "ssc" else [dict(p, L=p["L"] if p["L"] != 24 else 10) for p in BATCH]
    with pa.Engine.batch(pops, coding=coding, rng="reference", weights="fp64", graph=graph) as e:
        e.run()
        assert e.num_sets() == len(pops)
        for k, p in enumerate(pops):
            ref, _ = oracle.anneal(coding, p["L"], p["R"], p["sweeps"], p["dbeta"], p.get("beta_final", 1.0), 1,
                                   p["seed"])
            compare_rows(e.rows(k), ref[0], rtol=1e-9)


def test_native_runs_are_independent(cuda):
    """runs=4 with the native stream: four concurrent populations with
    disjoint streams -- different trajectories, same physics."""
    rows, (ms, att) = run(L=16, R=2000, sweeps=10, runs=4, seed=9, coding="msc")
    assert len(rows) == 4
    assert len({tuple(r[1:6, 8]) for r in rows}) == 4
    bf = np.array([r[-1, 6] for r in rows])
    assert bf.std() < 2e-3
    assert att == pytest.approx(10 * 256 * sum(r[1:, 8].sum() for r in rows))


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_cli_reference_C1(cuda, tmp_path, coding):
    """The command-line driver with the reference's flags writes the
    reference's results file (same directory layout, 11 digits)."""
    import os
    import subprocess
    from conftest import ROOT
    exe = os.path.join(ROOT, "paising_gb300", "_lib", "paising")
    r = subprocess.run([exe, "-R", "1000", "-t", "10", "-L", "16", "-s", "100", "-c", coding, "-m", "reference",
                        "-w", "fp64", "-o", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Time per spin-flip" in r.stdout and "RNG initial seed: 100" in r.stdout
    got = np.loadtxt(tmp_path / "PA_results_run_0.dat")
    ref_name = f"ref/inj_{coding.upper()}_L16_R1000_t10_d0.005_s100.dat"
    compare_rows(got, load_dat(ref_name), rtol=2e-10)
    from conftest import GOLDEN
    mine = open(tmp_path / "PA_results_run_0.dat").read().split("\n")
    theirs = open(os.path.join(GOLDEN, ref_name)).read().split("\n")
    for a, b in zip(mine[:50], theirs[:50]):  # beta, E/N and R print identically
        fa, fb = a.split(), b.split()
        assert fa[0] == fb[0] and fa[1] == fb[1] and fa[8] == fb[8]


def test_failed_allocation_is_reported(cuda):
    """A population far larger than the device (about 80 TB of spins): the
    allocation fails, pa_create returns PA_ERR_CUDA with a message and frees
    what it had allocated, and the device stays usable."""
    with pytest.raises(pa.PaisingError) as ei:
        pa.Engine(L=256, R=1_000_000_000, coding="ssc")
    assert ei.value.status == 2
    rows, _ = run(L=16, R=200, sweeps=2, dbeta=0.25, seed=1, coding="msc")
    assert rows[0].shape[0] == 5
