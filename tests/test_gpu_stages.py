"""Stage-level parity: each CUDA stage (through the C ABI) against the oracle
on the same seeded inputs.  Integer results (spins, energies, copy numbers,
offsets) must be bit-exact; lnQ / q to FP64 round-off."""
import numpy as np
import pytest

import paising_gb300 as pa

pytestmark = pytest.mark.gpu


def msc_words_np(t):
    return t.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("L,R", [(16, 37), (24, 5), (64, 9)])
def test_ssc_init(st, oracle, L, R):
    g = st.ssc_init(L, R, seed=100, iseq=12345)
    assert np.array_equal(g.cpu().numpy(), oracle.ssc_init(L, R, 100, 12345))


@pytest.mark.parametrize("L,R", [(16, 70), (10, 33), (64, 40)])
def test_msc_init(st, oracle, L, R):
    w, act = st.msc_init(L, R, seed=7, iseq=99)
    ow, oact = oracle.msc_init(L, R, 7, 99)
    assert np.array_equal(msc_words_np(w), ow)
    assert np.array_equal(act.cpu().numpy(), oact)


@pytest.mark.parametrize("L,R,sweeps,beta", [(16, 23, 3, 0.2), (16, 11, 2, 0.9), (24, 7, 2, 0.44),
                                             (48, 5, 1, 0.5), (64, 6, 2, 0.44), (64, 3, 1, 0.05)])
def test_ssc_sweep_reference_stream(st, oracle, L, R, sweeps, beta):
    """checkKerALL decisions under the reference-coordinate stream, then the
    fused energy epilogue against energyKer."""
    init = oracle.ssc_init(L, R, 5, 0)
    g = st.ssc_init(L, R, seed=5, iseq=0)
    E, M = st.ssc_sweep(g, L, sweeps, beta, pa.RNG_REFERENCE, seed=5, iseq=777)
    ref = oracle.ssc_sweep(init, L, sweeps, beta, 5, 777)
    got = g.cpu().numpy()
    assert np.array_equal(got, ref), f"{(got != ref).sum()} sites differ"
    oE, oM = oracle.ssc_energy(ref, L)
    assert np.array_equal(E.cpu().numpy(), oE) and np.array_equal(M.cpu().numpy(), oM)


@pytest.mark.parametrize("L,R,sweeps,beta", [(16, 64, 3, 0.2), (16, 40, 2, 0.9), (10, 33, 2, 0.44),
                                             (64, 96, 2, 0.44), (12, 32, 4, 0.05)])
def test_msc_sweep_reference_stream(st, oracle, L, R, sweeps, beta):
    w, act = st.msc_init(L, R, seed=11, iseq=0)
    ow, _ = oracle.msc_init(L, R, 11, 0)
    E, M = st.msc_sweep(w, act, L, sweeps, beta, pa.RNG_REFERENCE, seed=11, iseq=4242)
    ref = oracle.msc_sweep(ow, L, sweeps, beta, 11, 4242)
    got = msc_words_np(w)
    assert np.array_equal(got, ref), f"{(got != ref).sum()} words differ"
    oE, oM = oracle.msc_energy(ref, L)
    assert np.array_equal(E.cpu().numpy(), oE) and np.array_equal(M.cpu().numpy(), oM)


@pytest.mark.parametrize("coding,L", [("ssc", 16), ("ssc", 40), ("msc", 16), ("msc", 14)])
def test_energy_epilogue_random_lattices(st, oracle, coding, L):
    if coding == "ssc":
        g = st.ssc_init(L, 50, seed=3, iseq=1)
        E, M = st.ssc_sweep(g, L, 0, 0.4, pa.RNG_NATIVE, seed=3)
        oE, oM = oracle.ssc_energy(g.cpu().numpy(), L)
    else:
        w, act = st.msc_init(L, 100, seed=3, iseq=1)
        E, M = st.msc_sweep(w, act, L, 0, 0.4, pa.RNG_NATIVE, seed=3)
        oE, oM = oracle.msc_energy(msc_words_np(w), L)
    assert np.array_equal(E.cpu().numpy(), oE) and np.array_equal(M.cpu().numpy(), oM)


def _energies(oracle, coding, L, R, seed, beta):
    if coding == "ssc":
        s = oracle.ssc_sweep(oracle.ssc_init(L, R, seed, 0), L, 3, beta, seed, 10**6)
        E, M = oracle.ssc_energy(s, L)
        return s, E, None
    w, act = oracle.msc_init(L, R, seed, 0)
    w = oracle.msc_sweep(w, L, 3, beta, seed, 10**6)
    E, M = oracle.msc_energy(w, L)
    return w, E, act


@pytest.mark.parametrize("coding,L,R", [("ssc", 16, 1000), ("ssc", 16, 3000), ("msc", 16, 1000), ("msc", 16, 2500)])
def test_resample_plan_fp64(cuda, st, oracle, coding, L, R):
    """QKer + lnQ + CalcTauKer + CalcParSum with FP64 weights."""
    torch = cuda
    lat, E, act = _energies(oracle, coding, L, R, 21, 0.3)
    b0, b1, Emean, seed, iseq = 0.3, 0.305, float(E.mean()) + 3.0, 21, 555
    dB = b1 - b0
    if coding == "ssc":
        q = oracle.ssc_q(E, dB, Emean)
        lnQ = -dB * Emean + np.log(q) - np.log(R)
        roff, Rn = oracle.ssc_copy_numbers(E, R, lnQ, dB, seed, iseq)
    else:
        q = oracle.msc_q(E, act, dB, Emean)
        lnQ = -dB * Emean + np.log(q) - np.log(R)
        roff, Rn = oracle.msc_copy_numbers(E, act, R, R, lnQ, dB, seed, iseq)
    offs, tot = oracle.scan(roff)
    Et = torch.from_numpy(E).cuda()
    actt = None if act is None else torch.from_numpy(act).cuda()
    groff, goffs, gsrc, glnQ, gq, gRn = st.resample_plan(Et, actt, pa.SSC if coding == "ssc" else pa.MSC, R, R,
                                                         2 * R, b0, b1, Emean, pa.WEIGHTS_FP64, seed, iseq)
    assert gq == pytest.approx(q, rel=1e-13) and glnQ == pytest.approx(lnQ, rel=1e-12, abs=1e-14)
    assert gRn == Rn == tot
    assert np.array_equal(groff.cpu().numpy().view(np.uint32), roff)
    assert np.array_equal(goffs.cpu().numpy().view(np.uint32), offs)
    assert np.array_equal(gsrc[:Rn].cpu().numpy(), np.repeat(np.arange(len(roff)), roff))


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_resample_plan_concentrated_copies(cuda, st, oracle, coding):
    """A few replicas far below the others in energy take nearly all the
    copies (thousands each: one alone in its tile of 256, two in the same
    tile, one in the last tile), as a large dbeta against the energy spread
    makes them; the map of new to old replicas is still CalcParSum's."""
    torch = cuda
    L, R = 16, 6000
    _, E, act = _energies(oracle, coding, L, R, 33, 0.3)
    E = E.copy()
    heavy = [300, 1024, 1030, len(E) - 40]
    if act is not None:
        heavy = [int(np.flatnonzero(act[h:])[0]) + h for h in heavy]
    for k, h in enumerate(heavy):
        E[h] -= 900 + 40 * k
    b0, b1, seed, iseq = 0.3, 0.31, 5, 77
    dB = b1 - b0
    valid = E if act is None else E[act.astype(bool)]
    Emean = float(valid.mean())
    if coding == "ssc":
        q = oracle.ssc_q(E, dB, Emean)
        lnQ = -dB * Emean + np.log(q) - np.log(R)
        roff, Rn = oracle.ssc_copy_numbers(E, R, lnQ, dB, seed, iseq)
    else:
        q = oracle.msc_q(E, act, dB, Emean)
        lnQ = -dB * Emean + np.log(q) - np.log(R)
        roff, Rn = oracle.msc_copy_numbers(E, act, R, R, lnQ, dB, seed, iseq)
    assert roff[heavy].min() > 400 and roff[heavy].sum() > 0.9 * R, roff[heavy]
    offs, tot = oracle.scan(roff)
    Et = torch.from_numpy(E).cuda()
    actt = None if act is None else torch.from_numpy(act).cuda()
    groff, goffs, gsrc, glnQ, gq, gRn = st.resample_plan(Et, actt, pa.SSC if coding == "ssc" else pa.MSC, R, R,
                                                         2 * R, b0, b1, Emean, pa.WEIGHTS_FP64, seed, iseq)
    assert gRn == Rn == tot
    assert np.array_equal(groff.cpu().numpy().view(np.uint32), roff)
    assert np.array_equal(goffs.cpu().numpy().view(np.uint32), offs)
    assert np.array_equal(gsrc[:Rn].cpu().numpy(), np.repeat(np.arange(len(roff)), roff))


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_resample_plan_fp32_close_to_fp64(cuda, st, oracle, coding):
    """FP32 compensated weights: lnQ within 1e-6 of the FP64 value, copy
    numbers identical except where U falls within FP32 round-off of the
    fractional part (expected count << 1 at this size)."""
    torch = cuda
    L, R = 16, 4000
    lat, E, act = _energies(oracle, coding, L, R, 8, 0.42)
    Et = torch.from_numpy(E).cuda()
    actt = None if act is None else torch.from_numpy(act).cuda()
    c = pa.SSC if coding == "ssc" else pa.MSC
    valid = E if act is None else E[act.astype(bool)]
    r64 = st.resample_plan(Et, actt, c, R, R, 2 * R, 0.42, 0.43, float(valid.mean()), pa.WEIGHTS_FP64, 8, 0)
    r32 = st.resample_plan(Et, actt, c, R, R, 2 * R, 0.42, 0.43, float(valid.min()), pa.WEIGHTS_FP32, 8, 0)
    assert abs(r32[3] - r64[3]) < 1e-6
    diff = (r32[0] != r64[0]).sum().item()
    assert diff <= 2


@pytest.mark.parametrize("L,R", [(16, 50), (64, 30), (8, 700), (24, 130), (128, 9), (192, 7), (256, 5)])
def test_ssc_resample_gather(cuda, st, oracle, L, R):
    """Work units of whole replicas (L <= 128, the last one partial, e.g. L=24:
    56 replicas of 36 vectors) and of replica parts (L=192: 2048 + 256
    vectors, L=256: 2 x 2048) copy exactly what resampleKer copies."""
    torch = cuda
    old = oracle.ssc_init(L, R, 4, 0)
    rng = np.random.default_rng(1)
    roff = rng.integers(0, 3, R).astype(np.uint32)
    offs, tot = oracle.scan(roff)
    src = np.repeat(np.arange(R), roff).astype(np.int32)
    new = st.ssc_resample(torch.from_numpy(old).cuda(), L, torch.from_numpy(src).cuda(), tot)
    assert np.array_equal(new.cpu().numpy(), oracle.ssc_resample(old, L, roff, offs, tot))


@pytest.mark.parametrize("L,R", [(16, 200), (12, 70), (64, 100)])
def test_msc_resample_gather(cuda, st, oracle, L, R):
    """The gather places offspring s at group s % rg_new, bit s / rg_new,
    exactly like resampleKer's atomicXor scatter (PAisingMSC.cu:413-431)."""
    torch = cuda
    old, act = oracle.msc_init(L, R, 4, 0)
    rng = np.random.default_rng(2)
    roff = (rng.integers(0, 3, len(act)) * act).astype(np.uint32)
    offs, tot = oracle.scan(roff)
    src = np.repeat(np.arange(len(roff)), roff).astype(np.int32)
    new, nact = st.msc_resample(torch.from_numpy(old.view(np.int32)).cuda(), L, torch.from_numpy(src).cuda(), tot)
    onew, oact = oracle.msc_resample(old, L, roff, offs, tot)
    assert np.array_equal(msc_words_np(new), onew)
    assert np.array_equal(nact.cpu().numpy(), oact)


@pytest.mark.parametrize("L,R,kind", [(16, 200, "mixed"), (12, 70, "mixed"), (64, 3000, "mixed"),
                                      (64, 5000, "identity"), (32, 4000, "sparse"), (128, 700, "bursty"),
                                      (10, 33, "mixed"), (256, 100, "mixed"), (16, 900, "gap"),
                                      (16, 3000, "copies"), (64, 2000, "concentrated"), (24, 1500, "alternating")])
def test_msc_resample_gather_native(cuda, st, oracle, L, R, kind):
    """The native stream's gather (offspring s at slot s) equals the oracle's
    restatement bit for bit, active flags included: copy numbers of 0..3
    (mixed), all 1 (every word one shift), mostly 0 with some 4s (sparse:
    sources far apart, many per-bit fallbacks), and runs of 0 and of 3
    (bursty: long duplicate runs), and one run of 150 replicas without
    offspring (gap: sources beyond the four-word window, gathered bit by
    bit); 0..9 copies each (copies: runs of one source as broadcast pairs
    beside shifted single copies), a few parents with hundreds of copies
    among single ones (concentrated: whole words of one source), and 2 and 0
    copies in turn (alternating: runs of two beside every gap)."""
    torch = cuda
    old, act = oracle.msc_init(L, R, 4, 0)
    rng = np.random.default_rng(R + L)
    n = len(act)
    if kind == "mixed":
        roff = rng.integers(0, 4, n)
    elif kind == "identity":
        roff = np.ones(n, dtype=np.int64)
    elif kind == "sparse":
        roff = np.where(rng.random(n) < 0.2, 4, 0)
    elif kind == "bursty":
        roff = np.repeat(rng.choice([0, 1, 3], size=n // 40 + 1, p=[0.4, 0.3, 0.3]), 40)[:n]
    elif kind == "copies":
        roff = rng.integers(0, 10, n)
    elif kind == "concentrated":
        roff = np.where(rng.random(n) < 0.5, 1, 0)
        roff[rng.choice(n, 6, replace=False)] = [300, 150, 97, 64, 33, 500]
    elif kind == "alternating":
        roff = np.tile([2, 0], n // 2 + 1)[:n]
    else:  # one copy each, but 150 replicas in a row without offspring
        roff = np.ones(n, dtype=np.int64)
        roff[300:450] = 0
    roff = (roff * act).astype(np.uint32)
    offs, tot = oracle.scan(roff)
    assert tot > 0
    src = np.repeat(np.arange(n), roff).astype(np.int32)
    new, nact = st.msc_resample_native(torch.from_numpy(old.view(np.int32)).cuda(), L, R,
                                       torch.from_numpy(src).cuda(), tot)
    onew, oact = oracle.msc_resample_linear(old, L, roff, offs, tot)
    assert np.array_equal(nact.cpu().numpy(), oact)
    got = msc_words_np(new)
    bad = np.nonzero((got != onew).any(axis=1))[0]
    assert bad.size == 0, f"{bad.size} of {len(onew)} groups differ, first {bad[:5]}"


@pytest.mark.parametrize("coding", ["ssc", "msc"])
@pytest.mark.parametrize("beta", [0.25, 0.6])
def test_native_acceptance_probability(cuda, st, oracle, coding, beta):
    """Native stream: during the A half sweep every A site flips with
    probability 1 (dE <= 0), T4/2^32 (dE = 4) or T8/2^32 (dE = 8), given the
    initial B configuration.  The number of A flips after one sweep must match
    the expected count within 5 standard deviations."""
    L = 16
    N, h = L * L, L * L // 2
    T4, T8 = (int(x) for x in oracle.msc_thresholds(beta))
    p = {0: T8 / 2**32, 1: T4 / 2**32}
    if coding == "ssc":
        R = 4000
        g = st.ssc_init(L, R, seed=1, iseq=0)
        before = g.cpu().numpy().astype(np.int64)
        st.ssc_sweep(g, L, 1, beta, pa.RNG_NATIVE, seed=99)
        after = g.cpu().numpy().astype(np.int64)
        A, B = before[:, :h], before[:, h:]
        flips = (after[:, :h] != A).sum()
    else:
        R = 4000
        w, act = st.msc_init(L, R, seed=1, iseq=0)
        bw = msc_words_np(w).copy()
        st.msc_sweep(w, act, L, 1, beta, pa.RNG_NATIVE, seed=99)
        aw = msc_words_np(w)
        bits = lambda x: ((x[:, :, None] >> np.arange(32, dtype=np.uint32)) & 1).transpose(0, 2, 1).reshape(-1, N)
        before = bits(bw).astype(np.int64) * 2 - 1
        after = bits(aw).astype(np.int64) * 2 - 1
        A, B = before[:, :h], before[:, h:]
        flips = (after[:, :h] != A).sum()
    # anti-parallel neighbours of every A site in the initial configuration
    idx = np.arange(h)
    ty, tx = idx // (L // 2), idx % (L // 2)
    side = ty * (L // 2) + np.where(ty & 1, (tx + 1) % (L // 2), (tx - 1) % (L // 2))
    up, dn = ((ty - 1) % L) * (L // 2) + tx, ((ty + 1) % L) * (L // 2) + tx
    na = sum((A != B[:, j]).astype(np.int64) for j in (idx, side, up, dn))
    prob = np.where(na >= 2, 1.0, np.where(na == 1, p[1], p[0]))
    mean, var = prob.sum(), (prob * (1 - prob)).sum()
    assert abs(flips - mean) < 5 * np.sqrt(var), (flips, mean, np.sqrt(var))


def test_resample_plan_capacity_and_extinction(cuda, st, oracle):
    """The error paths of the resampling plan: a population that would
    outgrow its buffer raises the capacity error instead of writing past the
    buffer (the copy-number kernel publishes the flag, the scatter then
    writes nothing), and an empty new population the extinction error; the
    call returns the status.  With exactly enough room the plan succeeds."""
    torch = cuda
    L, R = 16, 1000
    _, E, _ = _energies(oracle, "ssc", L, R, 21, 0.3)
    Et = torch.from_numpy(E).cuda()
    b0, b1, Emean, iseq = 0.3, 0.305, float(E.mean()), 555
    dB = b1 - b0
    lnQ = -dB * Emean + np.log(oracle.ssc_q(E, dB, Emean)) - np.log(R)

    def plan(Rinit, Rcap, seed):
        return st.resample_plan(Et, None, pa.SSC, R, Rinit, Rcap, b0, b1, Emean, pa.WEIGHTS_FP64, seed, iseq)

    Rn = oracle.ssc_copy_numbers(E, R, lnQ, dB, 21, iseq)[1]
    assert plan(R, Rn, 21)[5] == Rn
    with pytest.raises(pa.PaisingError) as ei:
        plan(R, Rn - 1, 21)
    assert ei.value.status == 3
    # R_init = 1: about one copy expected in all, so some seeds draw none
    n_new = {s: oracle.ssc_copy_numbers(E, 1, lnQ, dB, s, iseq)[1] for s in range(1, 40)}
    dead = [s for s, n in n_new.items() if n == 0]
    alive = [s for s, n in n_new.items() if n > 0]
    assert dead and alive
    with pytest.raises(pa.PaisingError) as ei:
        plan(1, 2 * R, dead[0])
    assert ei.value.status == 4
    assert plan(1, 2 * R, alive[0])[5] == n_new[alive[0]]
