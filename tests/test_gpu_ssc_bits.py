"""The SSC bit-plane sweep (native stream, L = 64, 128, 256): tiles of
replicas packed to one bit per site in shared memory, 32 sites of a row per
word, bitsliced neighbour counts and digit-serial acceptance.  Packing and
unpacking must be exact, the energy epilogue must equal the oracle's
energies, and the physics must match the exact solution like the int8
sweep's."""
import numpy as np
import pytest

import paising_gb300 as pa

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("L", [64, 128, 256])
def test_bits_pack_unpack_and_energies(cuda, oracle, L):
    """A caller-supplied population with no temperature step: the final
    population is the uploaded one bit for bit, and the energies the sweep
    kernel's epilogue computes (kept by store_energies) are the oracle's."""
    R = 37 if L < 256 else 9  # tiles left partly empty
    rng = np.random.default_rng(L)
    pop = np.where(rng.integers(0, 2, (R, L * L)) > 0, 1, -1).astype(np.int8)
    with pa.Engine(L=L, R=R, sweeps=3, dbeta=2.0, beta_final=1.0, coding="ssc", store_energies=True) as e:
        e.set_population(pop)
        e.run()
        assert np.array_equal(e.population(), pop)
        E, _ = oracle.ssc_energy(pop, L)
        assert np.array_equal(e.energies(0, 0), E)


def test_bits_sweep_matches_int8_sweep_statistically(cuda, oracle):
    """L=64, R=20000, 20 sweeps, dbeta=0.01: the bit-plane sweep and the
    int8 sweep (sweep_variant=1) both stay within 2e-4 of the exact betaF/N
    and agree with each other in E/N at every beta."""
    out = []
    for variant in (0, 1):
        with pa.Engine(L=64, R=20000, sweeps=20, dbeta=0.01, coding="ssc", seed=21, sweep_variant=variant) as e:
            e.run()
            out.append(e.rows(0))
    exact = np.array([-oracle.kaufman(64, b)[0] / 4096 for b in out[0][:, 0]])
    for r in out:
        assert np.max(np.abs(r[:, 6] - exact)) < 2e-4
    assert np.max(np.abs(out[0][1:, 1] - out[1][1:, 1])) < 5e-3


def test_bits_batch_and_invariants(cuda):
    """Uneven SSC populations on bit planes in one batch: sizes stay within
    capacity, energies per site within [-2, 2], magnetisation within [0, 1],
    attempts counted from the rows."""
    pops = [dict(L=64, R=3000, sweeps=10, dbeta=0.02, seed=1), dict(L=128, R=700, sweeps=5, dbeta=0.05, seed=2),
            dict(L=256, R=50, sweeps=4, dbeta=0.1, seed=3)]
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
