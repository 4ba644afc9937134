"""Family statistics (no counterpart in the reference): every replica
carries the initial replica it descends from through the resampling, and
every temperature reports the number of surviving families, rho_t and the
family entropy.  Under the reference stream the engine must equal the
oracle's restatement of the same definition; the resampling it follows is
the one pinned on the reference's fixtures."""
import os

import numpy as np
import pytest

import paising_gb300 as pa

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("coding", ["ssc", "msc"])
@pytest.mark.parametrize("graph", [True, False])
def test_family_reference_stream(cuda, oracle, coding, graph):
    rows_ref, fam_ref, _ = oracle.anneal_family(coding, 16, 1000, 10, 0.05, 1.0, 1, 100)
    with pa.Engine(L=16, R=1000, sweeps=10, dbeta=0.05, seed=100, coding=coding, rng="reference", weights="fp64",
                   graph=graph, family=True) as e:
        e.run()
        f = e.family_rows(0)
        assert np.array_equal(e.rows(0)[:, 8], rows_ref[0][:, 8])
    ref = fam_ref[0]
    assert f.shape == ref.shape
    assert np.array_equal(f[:, 0], ref[:, 0])                 # family counts: exact
    assert np.allclose(f[:, 1:], ref[:, 1:], rtol=1e-12, atol=1e-12)
    assert f[0, 0] == 1000 and f[0, 1] == 1.0 and np.all(np.diff(f[:, 0]) <= 0)


def test_family_batch_adaptive_and_files(cuda, oracle, tmp_path):
    """Family statistics in a batch, one population with the adaptive step,
    and the PA_family_run_<r>.dat file."""
    pops = [dict(L=16, R=500, sweeps=4, dbeta=0.05, seed=11, family=True),
            dict(L=32, R=300, sweeps=3, dbeta=0.02, seed=12, family=True, adaptive=True)]
    with pa.Engine.batch(pops, coding="msc", rng="reference", weights="fp64") as e:
        e.run()
        for k, p in enumerate(pops):
            _, ref, _ = oracle.anneal_family("msc", p["L"], p["R"], p["sweeps"], p["dbeta"], 1.0, 1, p["seed"],
                                             adaptive=p.get("adaptive", False))
            f = e.family_rows(k)
            assert np.array_equal(f[:, 0], ref[0][:, 0])
            assert np.allclose(f[:, 1:], ref[0][:, 1:], rtol=1e-12, atol=1e-12)
        e.write_results(str(tmp_path))
        got = np.loadtxt(tmp_path / "PA_family_run_0.dat")
        assert np.array_equal(got[:, 1], e.family_rows(0)[:, 0])
        assert np.allclose(got[:, 0], e.rows(0)[:, 0])
