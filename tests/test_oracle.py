"""The oracle (CPU restatement of the reference) pinned against the reference
programs' own outputs (injected-stream builds run on a GB300, committed under
tests/golden/ref) and against exact results.  CPU only."""
import numpy as np
import pytest

from conftest import compare_rows, load_dat


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_oracle_matches_reference_C1(oracle, coding):
    """L=16, R=1000, 10 sweeps, dbeta=0.005, seed 100: the reference's own
    output, all 200 rows (R exactly; other columns print-rounded at 11 digits)."""
    rows, att = oracle.anneal(coding, 16, 1000, 10, 0.005, 1.0, 1, 100)
    ref = load_dat(f"ref/inj_{coding.upper()}_L16_R1000_t10_d0.005_s100.dat")
    compare_rows(rows[0], ref, rtol=2e-10)
    assert att == pytest.approx(10 * 256 * ref[1:, 8].sum())


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_oracle_matches_reference_two_runs(oracle, coding):
    """-M 2 -s 7: the second run continues the subsequence counter."""
    rows, _ = oracle.anneal(coding, 16, 1000, 10, 0.005, 1.0, 2, 7)
    for r in range(2):
        ref = load_dat(f"ref/inj_{coding.upper()}_L16_R1000_t10_d0.005_s7_M2_run{r}.dat")
        compare_rows(rows[r], ref, rtol=2e-10)


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_oracle_adaptive_matches_reference(oracle, coding):
    """The AdaptiveStep build of the reference (-DAdaptiveStep): temperatures
    chosen from the energy-histogram overlap, 57 rows ending on beta=1; and
    with -M 2 the second run replays the first run's schedule."""
    rows, _ = oracle.anneal(coding, 16, 1000, 10, 0.005, 1.0, 1, 100, adaptive=True)
    ref = load_dat(f"ref/inj_{coding.upper()}_L16_R1000_t10_d0.005_s100_adaptive.dat")
    assert ref.shape[0] == 57 and ref[-1, 0] == 1.0
    compare_rows(rows[0], ref, rtol=2e-10)
    rows, _ = oracle.anneal(coding, 16, 1000, 10, 0.01, 1.0, 2, 7, adaptive=True)
    for r in range(2):
        ref = load_dat(f"ref/inj_{coding.upper()}_L16_R1000_t10_d0.01_s7_M2_adaptive_run{r}.dat")
        compare_rows(rows[r], ref, rtol=2e-10)


def test_injected_stream_known_values(oracle):
    # Philox4x32-10 known-answer vectors (Salmon et al., Random123 kat_vectors):
    # counter 0, key 0 and counter/key all-ones
    assert list(oracle.philox([0, 0], [0, 0, 0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(oracle.philox([0xFFFFFFFF] * 2, [0xFFFFFFFF] * 4)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert list(oracle.philox([0xA4093822, 0x299F31D0], [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344])) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]
    # H is word (ctr & 3) of block ctr >> 2
    blk = oracle.philox([100, 0], [1, 0, 5, 0])
    assert [oracle.H(100, 5, 4 + j) for j in range(4)] == list(blk)


def test_product_philox_equals_oracle(oracle):
    """The engine's Philox (paising_gb300/csrc/pa_device.cuh, host path) and the
    oracle's independent restatement give the same words."""
    import paising_gb300 as pa
    rng = np.random.default_rng(3)
    for _ in range(200):
        seed, sub, ctr = (int(x) for x in rng.integers(0, 2**63, 3))
        assert pa.ref_word(seed, sub, ctr) == oracle.H(seed, sub, ctr)


def test_ssc_energy_known_lattices(oracle):
    L = 8
    N = L * L
    up = np.ones((1, N), dtype=np.int8)
    E, M = oracle.ssc_energy(up, L)
    assert E[0] == -2 * N and M[0] == N
    # checkerboard antiferromagnet: A = +1, B = -1 -> every bond anti-parallel
    af = np.concatenate([np.ones(N // 2), -np.ones(N // 2)]).astype(np.int8)[None]
    E, M = oracle.ssc_energy(af, L)
    assert E[0] == 2 * N and M[0] == 0


def test_msc_energy_matches_ssc(oracle):
    """Bit k of an MSC group is an SSC replica: energies must agree."""
    L = 12
    w, act = oracle.msc_init(L, 64, seed=9, iseq=0)
    E, M = oracle.msc_energy(w, L)
    for k in (0, 5, 31):
        for g in range(w.shape[0]):
            s = np.where((w[g] >> k) & 1, 1, -1).astype(np.int8)[None]
            e2, m2 = oracle.ssc_energy(s, L)
            assert E[g * 32 + k] == e2[0] and M[g * 32 + k] == m2[0]


def test_scan_and_resample(oracle):
    rng = np.random.default_rng(0)
    roff = rng.integers(0, 3, 50).astype(np.uint32)
    offs, tot = oracle.scan(roff)
    assert tot == roff.sum() and offs[0] == 0 and np.all(np.diff(offs.astype(int)) == roff[:-1])
    L = 8
    old = oracle.ssc_init(L, 50, 1, 0)
    new = oracle.ssc_resample(old, L, roff, offs, tot)
    src = np.repeat(np.arange(50), roff)
    assert np.array_equal(new, old[src])


def test_schedule_has_200_rows(engine_lib):
    import paising_gb300 as pa
    b = pa.schedule(0.005, 1.0)
    assert len(b) == 200 and b[0] == 0.0 and abs(b[-1] - 0.995) < 1e-12
    ref = load_dat("ref/inj_SSC_L16_R1000_t10_d0.005_s100.dat")[:, 0]
    assert np.allclose(b, ref, rtol=1e-10, atol=0)
    for d in (0.01, 0.0025, 0.003):
        py = [0.0]
        while py[-1] + d <= 1.0:
            py.append(py[-1] + d)
        assert list(pa.schedule(d, 1.0)) == py


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_oracle_family_statistics_definition(oracle, coding):
    """Family statistics of the oracle (the definition the engine is checked
    against): R families at beta = 0 with rho_t = 1 and S_f = ln R; counts
    never grow; S_f <= ln(families); rho_t >= R / families (Cauchy-Schwarz)."""
    rows, fam, _ = oracle.anneal_family(coding, 16, 600, 5, 0.05, 1.0, 1, 9)
    f, r = fam[0], rows[0]
    assert f[0, 0] == 600 and f[0, 1] == 1.0 and f[0, 2] == pytest.approx(np.log(600))
    assert np.all(np.diff(f[:, 0]) <= 0)
    assert np.all(f[:, 2] <= np.log(f[:, 0]) + 1e-12)
    assert np.all(f[:, 1] >= r[:, 8] / f[:, 0] - 1e-9)
