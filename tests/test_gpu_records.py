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


def test_lattice_dump_reference_bytes(cuda, tmp_path):
    """The LatticePopStore build's per-temperature population text, byte for
    byte, through the command-line driver's -S switch."""
    import subprocess
    from conftest import ROOT
    exe = os.path.join(ROOT, "paising_gb300", "_lib", "paising")
    r = subprocess.run([exe, "-R", "20", "-t", "5", "-s", "100", "-d", "0.25", "-L", "16", "-c", "ssc", "-m",
                        "reference", "-w", "fp64", "-S", "-o", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    d = os.path.join(GOLDEN, "ref", "inj_SSC_L16_R20_t5_d0.25_s100_lattice")
    for i in range(1, 5):
        assert open(tmp_path / f"PA_lattice_{i}.dat").read() == open(os.path.join(d, f"PA_lattice_{i}.dat")).read()


def test_lattice_dump_msc_matches_population(cuda, tmp_path):
    """MSC lattice dumps (an extension): the last temperature's text lists the
    final population's active replicas, group-major."""
    L, R = 16, 40
    with pa.Engine(L=L, R=R, sweeps=3, dbeta=0.25, seed=5, coding="msc") as e:
        e.set_lattice_dump(str(tmp_path))
        e.run()
        pop = e.population()
        n = e.num_rows()
    text = open(tmp_path / f"PA_lattice_{n - 1}.dat").read().strip().split("\n")
    reps = [l for l in text[1:] if l.startswith("P=")]
    assert len(reps) == int(text[0].split("R=")[1].rstrip(";"))
    # replica 0 of the text = group 0, bit 0: rebuild its lattice rows from the words
    h, W = L * L // 2, L // 2
    s = np.where((pop[0] >> 0) & 1, 1, -1)
    rows = []
    for y in range(L):
        row = []
        for i in range(W):
            a, b = s[y * W + i], s[h + y * W + i]
            row += [a, b] if y % 2 == 0 else [b, a]
        rows.append("{" + ",".join(str(v) for v in row) + "}")
    assert reps[0] == "P={" + ",".join(rows) + "};"
