"""The MSC sweep by thread-block clusters (sweep_variant 2 or 4: each group
split into stripes over 2 or 4 CTAs that read their neighbours' boundary rows
from distributed shared memory).  Under the reference-coordinate stream it
must reproduce the reference's and the oracle's runs exactly, like the
one-CTA sweep; it is the only MSC sweep for L > 128."""
import numpy as np
import pytest

import paising_gb300 as pa
from conftest import compare_rows, load_dat

pytestmark = pytest.mark.gpu


def run(**kw):
    with pa.Engine(**kw) as e:
        e.run()
        return [e.rows(r) for r in range(e.num_sets())]


@pytest.mark.parametrize("variant", [2, 4])
@pytest.mark.parametrize("graph", [True, False])
def test_cluster_reference_C1(cuda, variant, graph):
    rows = run(L=16, R=1000, sweeps=10, seed=100, coding="msc", rng="reference", weights="fp64", graph=graph,
               sweep_variant=variant)
    compare_rows(rows[0], load_dat("ref/inj_MSC_L16_R1000_t10_d0.005_s100.dat"), rtol=2e-10)


@pytest.mark.slow
@pytest.mark.parametrize("variant", [2, 4])
def test_cluster_reference_C2_L64(cuda, variant):
    rows = run(L=64, R=20000, sweeps=100, seed=100, coding="msc", rng="reference", weights="fp64",
               sweep_variant=variant)
    compare_rows(rows[0], load_dat("ref/inj_MSC_L64_R20000_t100_d0.005_s100.dat"), rtol=2e-10)


@pytest.mark.parametrize("variant", [0, 2, 4])
def test_cluster_L256_reference_stream(cuda, oracle, variant):
    """L = 256 (one group is 256 KB, more than a CTA's shared memory): the
    automatic choice (0) and both cluster sizes against the oracle."""
    L, R, sweeps, dbeta, bfin, seed = 256, 100, 2, 0.25, 1.0, 21
    ref, _ = oracle.anneal("msc", L, R, sweeps, dbeta, bfin, 1, seed)
    rows = run(L=L, R=R, sweeps=sweeps, dbeta=dbeta, beta_final=bfin, seed=seed, coding="msc", rng="reference",
               weights="fp64", sweep_variant=variant)
    compare_rows(rows[0], ref[0], rtol=1e-9)


@pytest.mark.parametrize("variant", [2, 4])
def test_cluster_batch_uneven_reference_stream(cuda, oracle, variant):
    """Uneven populations swept by one cluster kernel, each equal to the
    oracle's run of that population alone."""
    pops = [dict(L=16, R=300, sweeps=5, dbeta=0.05, seed=100), dict(L=24, R=500, sweeps=3, dbeta=0.1, seed=7),
            dict(L=8, R=90, sweeps=7, dbeta=0.04, beta_final=0.6, seed=3), dict(L=32, R=200, sweeps=2, dbeta=0.2, seed=11)]
    with pa.Engine.batch(pops, coding="msc", rng="reference", weights="fp64", sweep_variant=variant) as e:
        e.run()
        for k, p in enumerate(pops):
            ref, _ = oracle.anneal("msc", p["L"], p["R"], p["sweeps"], p["dbeta"], p.get("beta_final", 1.0), 1,
                                   p["seed"])
            compare_rows(e.rows(k), ref[0], rtol=1e-9)


@pytest.mark.parametrize("variant", [2, 4])
def test_cluster_native_free_energy_vs_kaufman_L16(cuda, oracle, variant):
    """Native stream through the cluster sweep: betaF/N against the exact
    finite-lattice value within 3e-4 at every beta (as for the one-CTA sweep)."""
    r = run(L=16, R=20000, sweeps=20, seed=12, coding="msc", sweep_variant=variant)[0]
    exact = np.array([-oracle.kaufman(16, b)[0] / 256 for b in r[:, 0]])
    assert np.max(np.abs(r[:, 6] - exact)) < 3e-4


def test_cluster_native_L256_physics(cuda, oracle):
    """L = 256, native stream, FP32 weights, beta 0 -> 0.3 in steps of
    0.0025 (the step must stay near 1/sqrt(2N) for the free-energy estimator
    to be unbiased at this size): betaF/N within 1e-4 and E/N within 3e-3 of
    the exact values at every beta (the oracle's run of the same schedule
    reaches 1.0e-5 and 6.1e-4), populations inside their buffers."""
    R = 4096
    r = run(L=256, R=R, sweeps=5, dbeta=0.0025, beta_final=0.3, seed=5, coding="msc")[0]
    N = 256 * 256
    assert np.all(r[:, 8] > 0) and np.all(r[:, 8] <= 1.25 * R + 256)
    exact_f = np.array([-oracle.kaufman(256, b)[0] / N for b in r[:, 0]])
    exact_e = np.array([oracle.kaufman(256, b)[1] / N for b in r[1:, 0]])
    assert np.max(np.abs(r[:, 6] - exact_f)) < 1e-4
    assert np.max(np.abs(r[1:, 1] - exact_e)) < 3e-3
