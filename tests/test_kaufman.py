"""The statistical oracle: Kaufman's exact partition function of the L x L
torus (oracle/kaufman.c) against brute-force enumeration and against the
values the reference's sample outputs are checked with."""
import itertools
import math

import numpy as np
import pytest


def brute(L, beta):
    N = L * L
    s = np.array(list(itertools.product([-1, 1], repeat=N)), dtype=np.int64).reshape(-1, L, L)
    E = -(s * np.roll(s, 1, 1)).sum((1, 2)) - (s * np.roll(s, 1, 2)).sum((1, 2))
    Em = E.min()
    w = np.exp(-beta * (E - Em))
    Z = w.sum()
    e1 = (E * w).sum() / Z
    e2 = (E * E * w).sum() / Z
    return math.log(Z) - beta * Em, e1, beta * beta * (e2 - e1 * e1)


@pytest.mark.parametrize("beta", [0.05, 0.3, 0.4406868, 0.7, 1.0])
def test_kaufman_vs_enumeration_L4(oracle, beta):
    lz, e, c = oracle.kaufman(4, beta)
    blz, be, bc = brute(4, beta)
    assert lz == pytest.approx(blz, rel=1e-13)
    assert e == pytest.approx(be, rel=1e-11, abs=1e-11)
    assert c == pytest.approx(bc, rel=1e-7)


def test_kaufman_L64_values(oracle):
    # betaF/N = -lnZ/N at the two betas quoted for the reference samples
    assert -oracle.kaufman(64, 0.5)[0] / 4096 == pytest.approx(-1.0259620381, abs=2e-10)
    assert -oracle.kaufman(64, 0.995)[0] / 4096 == pytest.approx(-1.9905320044, abs=2e-10)


def test_kaufman_vs_mpmath_L16(oracle):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    L, K = 16, mp.mpf("0.42")

    def g(k):
        if k == 0:
            return 2 * K + mp.log(mp.tanh(K))
        return mp.acosh(mp.cosh(2 * K) / mp.tanh(2 * K) - mp.cos(mp.pi * k / L))
    Z1 = mp.fprod(2 * mp.cosh(L * g(2 * r + 1) / 2) for r in range(L))
    Z2 = mp.fprod(2 * mp.sinh(L * g(2 * r + 1) / 2) for r in range(L))
    Z3 = mp.fprod(2 * mp.cosh(L * g(2 * r) / 2) for r in range(L))
    Z4 = mp.fprod(2 * mp.sinh(L * g(2 * r) / 2) for r in range(L))
    lnZ = mp.log(mp.mpf(1) / 2 * (2 * mp.sinh(2 * K)) ** (L * L / 2) * (Z1 + Z2 + Z3 + Z4))
    assert oracle.kaufman(L, 0.42)[0] == pytest.approx(float(lnZ), rel=1e-14)


def test_reference_samples_meet_the_bar(oracle):
    """The reference's shipped sample outputs (L=64, R=20000, 100 sweeps) are
    within 1e-4 of the exact betaF/N at every beta."""
    import os
    from conftest import GOLDEN
    d = os.path.join(GOLDEN, "reference_sample_output")
    for f in sorted(os.listdir(d)):
        rows = np.loadtxt(os.path.join(d, f))
        err = max(abs(r[6] + oracle.kaufman(64, r[0])[0] / 4096) for r in rows[1:])
        assert err < 1e-4, (f, err)
