"""The SSC bit-plane sweep (native stream): tiles of replicas packed to one
bit per site in shared memory -- a sublattice row as words of up to 32 sites,
or the rows of several replicas in one word when a row has at most 16 sites
-- bitsliced neighbour counts and digit-serial acceptance.  Packing and
unpacking must be exact, zero-temperature sweeps must equal the checkerboard
dynamics restated in numpy for every layout, the energy epilogue must equal
the oracle's energies, and the physics must match the exact solution like
the int8 sweep's."""
import numpy as np
import pytest

import paising_gb300 as pa

pytestmark = pytest.mark.gpu


# L -> (segments per word, sites per segment, words per row): every layout kind
LAYOUTS = {8: (8, 4, 1), 16: (4, 8, 1), 24: (2, 12, 1), 32: (2, 16, 1), 40: (1, 20, 1), 48: (1, 24, 1),
           56: (1, 28, 1), 64: (1, 32, 1), 72: (1, 12, 3), 80: (1, 20, 2), 96: (1, 24, 2), 112: (1, 28, 2),
           120: (1, 20, 3), 128: (1, 32, 2), 144: (1, 24, 3), 160: (1, 20, 4), 168: (1, 28, 3), 192: (1, 32, 3),
           200: (1, 20, 5), 224: (1, 28, 4), 240: (1, 24, 5), 256: (1, 32, 4)}


def _reps(L):
    # replicas leaving the last tile partly empty (and the last word's segments)
    return {8: 301, 16: 259, 24: 131, 32: 67, 40: 30, 48: 23}.get(L, 7 if L <= 128 else 3)


def checkerboard_zero_T(pop, L, sweeps):
    """Zero-temperature checkerboard Metropolis dynamics on the SSC layout
    (sublattice A = sites with x+y even first, site (x, y) at y*L/2 + x/2,
    PAisingSSC.cu:169): A then B, a site flips iff dE <= 0, i.e. iff it has
    at least two anti-parallel neighbours."""
    y, x = np.mgrid[0:L, 0:L]
    a = (x + y) % 2 == 0
    m = np.where(a, 0, L * L // 2) + y * (L // 2) + x // 2
    g = pop[:, m].astype(np.int32)
    for _ in range(sweeps):
        for sub in (a, ~a):
            nb = (np.roll(g, 1, 1) + np.roll(g, -1, 1) + np.roll(g, 1, 2) + np.roll(g, -1, 2))
            g = np.where(sub & (g * nb <= 0), -g, g)
    out = np.empty_like(pop)
    out[:, m.ravel()] = g.reshape(len(pop), -1).astype(np.int8)
    return out


@pytest.mark.parametrize("L", sorted(LAYOUTS))
def test_bits_zero_temperature_exact(cuda, st, oracle, L):
    """At beta = 1e4 both thresholds are 0: the bit-plane sweep is the
    deterministic zero-temperature dynamics, for every row layout, equal to
    the numpy restatement and to the int8 sweep; E and M equal the oracle's
    energies of the result."""
    torch = cuda
    R = _reps(L)
    rng = np.random.default_rng(L)
    pop = np.where(rng.integers(0, 2, (R, L * L)) > 0, 1, -1).astype(np.int8)
    want = checkerboard_zero_T(pop, L, 3)
    t = torch.from_numpy(pop).cuda()
    E, M = st.ssc_sweep_bits(t, L, 3, 1e4, seed=5)
    got = t.cpu().numpy()
    assert np.array_equal(got, want)
    oE, oM = oracle.ssc_energy(want, L)
    assert np.array_equal(E.cpu().numpy(), oE) and np.array_equal(M.cpu().numpy(), oM)
    t8 = torch.from_numpy(pop).cuda()
    st.ssc_sweep(t8, L, 3, 1e4, pa.RNG_NATIVE, 5)
    assert np.array_equal(t8.cpu().numpy(), want)


def test_bits_layout_table(cuda):
    """The engine's bit-plane form per lattice size: spins per word 32, one
    replica per word group of `segs` rows; sizes without a layout (L=104)
    keep the int8 form, and sparse layouts (fill < 3/4: L=40, 72) are only
    chosen by the autotuner."""
    for L, (segs, seg, wq) in LAYOUTS.items():
        with pa.Engine(L=L, R=64, coding="ssc") as e:
            f = e.sweep_form()
            fill = segs * seg / 32.0  # bits of a word that hold sites
            assert f["spins_per_word"] == (32 if fill >= 0.75 else 4), (L, f)
    with pa.Engine(L=104, R=64, coding="ssc") as e:
        assert e.sweep_form()["spins_per_word"] == 4
    with pytest.raises(pa.PaisingError):
        import paising_gb300.stages as st
        st.ssc_sweep_bits(cuda.zeros((2, 104 * 104), dtype=cuda.int8, device="cuda"), 104, 1, 0.4, 1)


@pytest.mark.parametrize("L", [8, 16, 24, 32, 48, 64, 96, 128, 144, 192, 240, 256])
def test_bits_pack_unpack_and_energies(cuda, oracle, L):
    """A caller-supplied population with no temperature step: the final
    population is the uploaded one bit for bit, and the energies the sweep
    kernel's epilogue computes (kept by store_energies) are the oracle's."""
    R = _reps(L)  # tiles left partly empty
    rng = np.random.default_rng(L)
    pop = np.where(rng.integers(0, 2, (R, L * L)) > 0, 1, -1).astype(np.int8)
    with pa.Engine(L=L, R=R, sweeps=3, dbeta=2.0, beta_final=1.0, coding="ssc", store_energies=True) as e:
        assert e.sweep_form()["spins_per_word"] == 32
        e.set_population(pop)
        e.run()
        assert np.array_equal(e.population(), pop)
        E, _ = oracle.ssc_energy(pop, L)
        assert np.array_equal(e.energies(0, 0), E)


@pytest.mark.parametrize("L", [24, 48])
def test_bits_segments_free_energy_vs_kaufman(cuda, oracle, L):
    """Segment layouts (L=24: two replicas' 12-site rows per word; L=48: one
    24-site row per word): R=20000, 20 sweeps, dbeta=0.01, betaF/N within
    3e-4 of the exact value at every beta."""
    with pa.Engine(L=L, R=20000, sweeps=20, dbeta=0.01, coding="ssc", seed=31) as e:
        assert e.sweep_form()["spins_per_word"] == 32
        e.run()
        r = e.rows(0)
    exact = np.array([-oracle.kaufman(L, b)[0] / (L * L) for b in r[:, 0]])
    assert np.max(np.abs(r[:, 6] - exact)) < 3e-4


def test_bits_sweep_matches_int8_sweep_statistically(cuda, oracle):
    """L=64, R=20000, 20 sweeps, dbeta=0.01: the bit-plane sweep and the
    int8 sweep (sweep_variant=1) both stay within 2e-4 of the exact betaF/N
    at every beta, and within 1e-2 of the exact E/N, with no bias: their mean
    deviation over the schedule is below 5e-4.  (With 20 sweeps the largest
    deviations sit at beta_c = 0.44, where two independent runs differ by
    about 1e-2.)"""
    out = []
    for variant in (0, 1):
        with pa.Engine(L=64, R=20000, sweeps=20, dbeta=0.01, coding="ssc", seed=21, sweep_variant=variant) as e:
            e.run()
            out.append(e.rows(0))
    ex = [oracle.kaufman(64, b) for b in out[0][:, 0]]
    bf = np.array([-x[0] / 4096 for x in ex])
    en = np.array([x[1] / 4096 for x in ex])
    for r in out:
        assert np.max(np.abs(r[:, 6] - bf)) < 2e-4
        dev = r[1:, 1] - en[1:]
        assert np.max(np.abs(dev)) < 1e-2 and abs(dev.mean()) < 5e-4, (np.max(np.abs(dev)), dev.mean())


def test_bits_batch_and_invariants(cuda):
    """Uneven SSC populations on bit planes in one batch: sizes stay within
    capacity, energies per site within [-2, 2], magnetisation within [0, 1],
    attempts counted from the rows."""
    pops = [dict(L=64, R=3000, sweeps=10, dbeta=0.02, seed=1), dict(L=128, R=700, sweeps=5, dbeta=0.05, seed=2),
            dict(L=256, R=50, sweeps=4, dbeta=0.1, seed=3), dict(L=16, R=2000, sweeps=10, dbeta=0.02, seed=4),
            dict(L=48, R=900, sweeps=6, dbeta=0.05, seed=5), dict(L=96, R=300, sweeps=5, dbeta=0.05, seed=6)]
    with pa.Engine.batch(pops, coding="ssc") as e:
        e.run()
        ms, att = e.timing()
        tot = 0.0
        for k, p in enumerate(pops):
            r = e.rows(k)
            assert np.all(r[:, 8] > 0) and np.all(r[:, 8] <= 1.25 * p["R"] + 256)
            assert np.all(np.abs(r[1:, 1]) <= 2) and np.all((r[1:, 3] >= 0) & (r[1:, 3] <= 1))
            assert r[-1, 1] < -1.5
            tot += p["sweeps"] * p["L"] ** 2 * r[1:, 8].sum()
        assert att == pytest.approx(tot)
