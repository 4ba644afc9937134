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


def _family_stats_of(sizes: np.ndarray):
    """The definitions themselves, from family sizes c_f (sum R): number of
    families, rho_t = sum c_f^2 / R, S_f = ln R - sum c_f ln c_f / R."""
    sizes = sizes[sizes > 0].astype(np.float64)
    R = sizes.sum()
    return len(sizes), (sizes ** 2).sum() / R, np.log(R) - (sizes * np.log(sizes)).sum() / R


def _replica_lattices(coding: str, pop: np.ndarray, R: int, L: int) -> np.ndarray:
    """Active replicas of a population read back with pa_get_population, one
    row of bytes per replica.  With the engine's own stream MSC slot (g, b)
    holds offspring s = 32 g + b and is active when s < R."""
    if coding == "ssc":
        return pop[:R].astype(np.int8)
    rg = pop.shape[0]
    out = []
    for g in range(rg):
        for b in range(32):
            if 32 * g + b < R:
                out.append(((pop[g] >> np.uint32(b)) & np.uint32(1)).astype(np.int8))
    return np.array(out)


@pytest.mark.parametrize("coding", ["ssc", "msc"])
@pytest.mark.parametrize("R,steps", [(8, 2), (300, 4)])
def test_family_statistics_from_observed_ancestors(cuda, coding, R, steps):
    """Family statistics checked against ancestors observed directly, not
    against a restatement of the engine's bookkeeping.  With no Metropolis
    sweeps (sweeps = 0) a replica's lattice is an exact copy of its initial
    ancestor's, and every initial lattice is distinct, so after k
    temperatures each replica's family is found by matching its lattice
    against the uploaded initial population.  The family sizes counted that
    way give the three columns of row k through their definitions."""
    L, N, dB, seed = 8, 64, 0.05, 31 + R
    rng = np.random.default_rng(R * 10 + steps)
    rg0 = (R + 31) // 32
    if coding == "ssc":
        init = np.where(rng.integers(0, 2, (R, N)) > 0, 1, -1).astype(np.int8)
        slots = init
    else:
        init = rng.integers(0, 2**32, (rg0, N), dtype=np.uint32)
        slots = np.array([((init[g] >> np.uint32(b)) & np.uint32(1)).astype(np.int8)
                          for g in range(rg0) for b in range(32)])
    index = {row.tobytes(): i for i, row in enumerate(slots)}
    assert len(index) == len(slots)  # every initial lattice distinct
    longest = None
    for k in range(1, steps + 1):
        with pa.Engine(L=L, R=R, sweeps=0, dbeta=dB, beta_final=(k + 0.5) * dB, seed=seed, coding=coding,
                       family=True) as e:
            e.set_population(init)
            e.run()
            rows, fam, pop = e.rows(0), e.family_rows(0), e.population()
        assert rows.shape[0] == k + 1 and fam.shape[0] == k + 1
        Rk = int(rows[k, 8])
        lat = _replica_lattices(coding, pop, Rk, L)
        assert len(lat) == Rk
        anc = np.array([index[row.tobytes()] for row in lat])  # KeyError: a lattice that descends from none
        nf, rho, sf = _family_stats_of(np.bincount(anc))
        assert fam[k, 0] == nf, (k, fam[k], nf)
        assert fam[k, 1] == pytest.approx(rho, rel=1e-12) and fam[k, 2] == pytest.approx(sf, rel=1e-12, abs=1e-12)
        if longest is not None:  # the same trajectory: earlier rows repeat
            assert np.array_equal(fam[:k], longest)
        longest = fam
    assert fam[0, 0] == R and fam[0, 1] == 1.0 and fam[0, 2] == pytest.approx(np.log(R), rel=1e-12)
    if R > 100:
        assert fam[-1, 0] < R  # resampling removed families
