"""Per-temperature records: multi-histogram reweighting (the reference's MHR
build) and the energies of every temperature (its EnergiesPopStore build),
against the reference built with both switches and the injected stream."""
import os

import numpy as np
import pytest

import paising_gb300 as pa
from conftest import GOLDEN, compare_rows, load_dat

pytestmark = pytest.mark.gpu


def fixture_dir(coding):
    return os.path.join(GOLDEN, "ref", f"inj_{coding.upper()}_L16_R1000_t10_d0.05_s100_records")


@pytest.mark.parametrize("coding", ["ssc", "msc"])
@pytest.mark.parametrize("graph", [True, False])
def test_records_reference(cuda, tmp_path, coding, graph):
    d = fixture_dir(coding)
    with pa.Engine(L=16, R=1000, sweeps=10, seed=100, dbeta=0.05, coding=coding, rng="reference", weights="fp64",
                   graph=graph, mhr=True, store_energies=True) as e:
        e.run()
        compare_rows(e.rows(0), np.loadtxt(os.path.join(d, "PA_results_run_0.dat")), rtol=2e-10)
        m = e.mhr_rows(0)
        ref = np.loadtxt(os.path.join(d, "PA_MHR_results_run_0.dat"))
        assert m.shape == ref.shape
        assert np.allclose(m, ref, rtol=2e-10, atol=1e-12)
        for i in range(1, len(m)):
            assert np.array_equal(e.energies(0, i), np.loadtxt(os.path.join(d, f"PA_energies_{i}.dat"), dtype=np.int64))
        # the files the reference writes, byte for byte in the integers
        e.write_results(str(tmp_path))
        for i in range(1, len(m)):
            assert open(tmp_path / f"PA_energies_{i}.dat").read().split() == \
                open(os.path.join(d, f"PA_energies_{i}.dat")).read().split()
        assert np.allclose(np.loadtxt(tmp_path / "PA_MHR_results_run_0.dat"), ref, rtol=2e-10, atol=1e-12)


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_records_with_adaptive_schedule(cuda, coding):
    """Energies of an adaptive run come back through the device ring (one
    graph chunk at a time) and agree with the rows: count = R_i and mean =
    E/N * N at every temperature, in graph and host-stepped mode alike."""
    got = []
    for graph in (True, False):
        with pa.Engine(L=16, R=1000, sweeps=10, seed=100, coding=coding, rng="reference", weights="fp64",
                       adaptive=True, store_energies=True, mhr=True, graph=graph) as e:
            e.run()
            rows = e.rows(0)
            assert len(rows) == 57
            es = [e.energies(0, i) for i in range(len(rows))]
            for i in range(1, len(rows)):
                assert len(es[i]) == rows[i, 8]
                assert es[i].mean() / 256 == pytest.approx(rows[i, 1], rel=1e-12, abs=1e-12)
            got.append((es, e.mhr_rows(0)))
    for a, b in zip(got[0][0], got[1][0]):
        assert np.array_equal(a, b)
    assert np.array_equal(got[0][1], got[1][1])


def test_records_native_mhr_vs_exact(cuda, oracle):
    """Native stream, L=16, R=20000: the reweighted free energy agrees with
    the exact value as well as the plain estimate does."""
    with pa.Engine(L=16, R=20000, sweeps=20, seed=12, coding="msc", mhr=True) as e:
        e.run()
        m = e.mhr_rows(0)
        rows = e.rows(0)
    exact = np.array([-oracle.kaufman(16, b)[0] / 256 for b in m[:, 0]])
    assert np.max(np.abs(m[:, 3] - exact)) < 3e-4
    assert np.max(np.abs(rows[:, 6] - exact)) < 3e-4
