"""The engine's native random stream (no counterpart in the reference).

CPU: the oracle's restatement of the native acceptance (oracle/native_stream.c)
decides each replica's Metropolis test with probability exactly T/2^32 -- the
reference's thresholds -- and without correlation between replicas or sites.
The thresholds are chosen so that the single-bit finish after digit 7 carries
a visible share of the probability (T4 mod 2^24 = 2^24 - 1, T8 mod 2^24 = 0).

GPU: the production MSC and SSC bit-plane sweeps (native stream) equal that
restatement bit for bit, and its energy epilogue equals energyKer's; two
consecutive whole runs of one handle equal the oracle's anneal with the same
native sweeps row for row (the run number is part of the sweep counter).
"""
import numpy as np
import pytest

import paising_gb300 as pa

N_CALLS = 60000


def _accept_samples(oracle, T4, T8, n=N_CALLS, seed=3):
    """n batches of four word-sites, every bit undecided; replica bits of site
    k use T4 where a[k] is set.  Returns (accepted bits [n, 128], a bits)."""
    rng = np.random.default_rng(seed)
    a = rng.integers(0, 2**32, size=(n, 4), dtype=np.uint64).astype(np.uint32)
    und = np.full(4, 0xFFFFFFFF, dtype=np.uint32)
    zero = np.zeros(4, dtype=np.uint32)
    out = np.empty((n, 4), dtype=np.uint32)
    for i in range(n):
        site = np.array([4 * i, 4 * i + 1, 4 * i + 2, 4 * i + 3], dtype=np.uint32)
        out[i] = oracle.native_accept4(a[i], und, zero, site, 4, i, 0x50, 9, oracle.NATIVE_TAG_MSC | 7, 2026, T4, T8)
    bits = lambda x: ((x[:, :, None] >> np.arange(32, dtype=np.uint32)) & 1).reshape(len(x), 128)
    return bits(out).astype(np.float64), bits(a).astype(bool)


@pytest.mark.parametrize("T4,T8", [(0xA5FFFFFF, 0x3C000000), (0x2BFFFFFF, 0x07000000)])
def test_native_acceptance_is_exact(oracle, T4, T8):
    acc, use4 = _accept_samples(oracle, T4, T8)
    for mask, T in ((use4, T4), (~use4, T8)):
        p = T / 2**32
        n = mask.sum()
        f = acc[mask].mean()
        assert abs(f - p) < 5 * np.sqrt(p * (1 - p) / n), (hex(T), f, p, n)


def test_native_acceptance_finish_uses_each_bits_threshold(oracle):
    """With T4 and T8 equal in their first 8 digits, only the single-bit finish
    tells them apart: T4 mod 2^24 = 2^24 - 1, T8 mod 2^24 = 0, so the two
    classes must differ by 2^-8 in acceptance."""
    T4, T8 = 0x47FFFFFF, 0x47000000
    acc, use4 = _accept_samples(oracle, T4, T8, seed=11)
    f4, f8 = acc[use4].mean(), acc[~use4].mean()
    n4, n8 = use4.sum(), (~use4).sum()
    for f, T, n in ((f4, T4, n4), (f8, T8, n8)):
        p = T / 2**32
        assert abs(f - p) < 5 * np.sqrt(p * (1 - p) / n), (hex(T), f, p)
    assert f4 - f8 > 2**-8 - 10 * np.sqrt(0.28 * 0.72 / min(n4, n8))


def test_native_acceptance_uncorrelated(oracle):
    """No two of a batch's 128 decisions (4 word-sites x 32 replicas) share
    randomness: every pairwise correlation is within sampling noise."""
    acc, _ = _accept_samples(oracle, 0x40000000, 0x10000000, seed=5)
    c = np.corrcoef(acc.T)
    np.fill_diagonal(c, 0.0)
    assert np.abs(c).max() < 6.0 / np.sqrt(len(acc)), np.abs(c).max()


def test_native_acceptance_partial_batch(oracle):
    """Slots beyond nvalid draw nothing and keep their outright accepts."""
    a = np.array([0x0F0F0F0F, 0, 0xFFFF0000, 0x12345678], dtype=np.uint32)
    und = np.array([0xFFFFFFFF, 0xFFFFFFFF, 0, 0], dtype=np.uint32)
    acc0 = np.array([0, 0, 0xF0, 0x0F], dtype=np.uint32)
    site = np.arange(4, dtype=np.uint32)
    out = oracle.native_accept4(a, und, acc0, site, 2, 1, 0x30, 1, oracle.NATIVE_TAG_MSC, 5, 0x80000000, 0x20000000)
    assert out[2] == 0xF0 and out[3] == 0x0F
    # the first two sites drew: the same call is deterministic
    again = oracle.native_accept4(a, und, acc0, site, 2, 1, 0x30, 1, oracle.NATIVE_TAG_MSC, 5, 0x80000000,
                                  0x20000000)
    assert np.array_equal(out, again)


@pytest.mark.gpu
@pytest.mark.parametrize("L,R,sweeps,beta", [(16, 64, 3, 0.3), (10, 40, 2, 0.44), (12, 96, 2, 0.9),
                                             (24, 33, 2, 0.44), (64, 70, 2, 0.35), (128, 32, 1, 0.44)])
def test_msc_sweep_native_stream_bit_exact(cuda, st, oracle, L, R, sweeps, beta):
    seed, step = 777 + L, 5
    w, act = st.msc_init(L, R, seed=seed, iseq=0)
    ow, _ = oracle.msc_init(L, R, seed, 0)
    E, M = st.msc_sweep(w, act, L, sweeps, beta, pa.RNG_NATIVE, seed=seed, iseq=0, step=step)
    T4, T8 = (int(x) for x in oracle.msc_thresholds(beta))
    # the stage call runs temperature step 1 of population `step`
    ref = oracle.msc_sweep_native(ow, L, sweeps, T4, T8, seed, 1, oracle.NATIVE_TAG_MSC | step)
    got = w.cpu().numpy().view(np.uint32)
    assert (ref != ow).any()
    assert np.array_equal(got, ref), f"{(got != ref).sum()} of {got.size} words differ"
    oE, oM = oracle.msc_energy(ref, L)
    assert np.array_equal(E.cpu().numpy(), oE) and np.array_equal(M.cpu().numpy(), oM)


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [True, False])
@pytest.mark.parametrize("L,R,sweeps,dbeta", [(16, 200, 5, 0.05), (24, 700, 3, 0.1), (64, 1000, 4, 0.1),
                                              (96, 100, 2, 0.2), (128, 64, 2, 0.2)])
def test_msc_anneal_native_stream_two_runs(cuda, oracle, graph, L, R, sweeps, dbeta):
    """Whole anneals with the production stream: two runs of one handle
    (one-CTA sweep, one group per work unit, FP64 weights) equal the oracle's
    sequential runs row for row -- population sizes exactly -- and the second
    run draws sweep randomness of its own (temperature i of run r is native
    counter word i | r << 14)."""
    from conftest import compare_rows
    seed = 100 + L
    with pa.Engine(L=L, R=R, sweeps=sweeps, dbeta=dbeta, beta_final=1.0, seed=seed, coding="msc", rng="native",
                   weights="fp64", graph=graph, sweep_variant=1, tile_groups=1, device=0) as e:
        got = []
        for _ in range(2):
            e.run()
            got.append(e.rows(0))
    ref = oracle.anneal_msc_native(L, R, sweeps, dbeta, 1.0, 2, seed, seed, oracle.NATIVE_TAG_MSC | 0)
    for r in range(2):
        compare_rows(got[r], ref[r], rtol=2e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("L,R,tile", [(16, 300, 2), (16, 1000, 8), (32, 500, 4), (24, 400, 2), (32, 900, 8),
                                      (64, 200, 2)])
def test_msc_anneal_native_stream_stacked_tiles(cuda, oracle, L, R, tile):
    """Stacked tiles (several groups per work unit of the one-CTA sweep, the
    last tile short where the group count is not a multiple): every batch of
    four stacked rows is numbered by its tile, so the stream differs from the
    one-group sweep and must still equal the oracle's restatement."""
    from conftest import compare_rows
    seed = 31 + tile
    with pa.Engine(L=L, R=R, sweeps=3, dbeta=0.1, beta_final=1.0, seed=seed, coding="msc", rng="native",
                   weights="fp64", graph=True, sweep_variant=1, tile_groups=tile, device=0) as e:
        assert e.sweep_form(0)["tile"] == tile
        e.run()
        got = e.rows(0)
    ref = oracle.anneal_msc_native(L, R, 3, 0.1, 1.0, 1, seed, seed, oracle.NATIVE_TAG_MSC, 256, tile, 1)
    compare_rows(got, ref[0], rtol=2e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("L,R,cs", [(16, 200, 2), (16, 200, 4), (64, 100, 4), (64, 300, 2), (128, 90, 2),
                                     (256, 40, 2)])
def test_msc_anneal_native_stream_clusters(cuda, oracle, L, R, cs):
    """Thread-block clusters (cs CTAs per group, 256 threads each up to
    L = 128, else 1024 or 512, halo rows over distributed shared memory)
    under the native stream equal the oracle's restatement of the same thread
    layout row for row."""
    from conftest import compare_rows
    # threads per CTA: 256 up to L = 128, else 1024 (clusters of 2) or 512 (4)
    seed, threads = 57 + cs, 256 if L <= 128 else {2: 1024, 4: 512}[cs]
    sweeps, dbeta = (2, 0.25) if L == 256 else (3, 0.1)
    with pa.Engine(L=L, R=R, sweeps=sweeps, dbeta=dbeta, beta_final=1.0, seed=seed, coding="msc", rng="native",
                   weights="fp64", graph=True, sweep_variant=cs, device=0) as e:
        assert e.sweep_form(0)["cluster_ctas"] == cs
        e.run()
        got = e.rows(0)
    ref = oracle.anneal_msc_native(L, R, sweeps, dbeta, 1.0, 1, seed, seed, oracle.NATIVE_TAG_MSC, threads, 1, cs)
    compare_rows(got, ref[0], rtol=2e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("L,R,beta", [(8, 521, 0.44), (16, 303, 0.3), (24, 171, 0.44), (32, 130, 0.9),
                                      (40, 45, 0.44), (48, 50, 0.35), (64, 37, 0.44), (96, 11, 0.44),
                                      (128, 9, 0.5)])
def test_ssc_sweep_bits_native_stream_bit_exact(cuda, st, oracle, L, R, beta):
    """The SSC bit-plane sweep (pa_ssc_sweep_bits: largest tile, short last
    tiles, rows sharing a word as segments for L <= 32, rows of several words
    for L = 96, 128) equals the oracle's site-by-site restatement bit for bit,
    and its popcount energies equal energyKer's."""
    seed, step = 4000 + L, 3
    g = st.ssc_init(L, R, seed=seed, iseq=0)
    init = oracle.ssc_init(L, R, seed, 0)
    E, M = st.ssc_sweep_bits(g, L, 2, beta, seed=seed, step=step)
    T4, T8 = (int(x) for x in oracle.msc_thresholds(beta))
    ref = oracle.ssc_sweep_bits_native(init, L, 2, T4, T8, seed, 1, oracle.NATIVE_TAG_SSC | step,
                                       oracle.bits_max_tile(L))
    got = g.cpu().numpy()
    assert (ref != init).any()
    assert np.array_equal(got, ref), f"{(got != ref).sum()} of {got.size} sites differ"
    oE, oM = oracle.ssc_energy(ref, L)
    assert np.array_equal(E.cpu().numpy(), oE) and np.array_equal(M.cpu().numpy(), oM)


@pytest.mark.gpu
@pytest.mark.parametrize("L,R", [(16, 1000), (24, 500), (64, 700), (128, 300)])
def test_ssc_anneal_native_stream_bit_planes(cuda, oracle, L, R):
    """Whole SSC anneals on bit planes (the engine's automatic tile, two runs
    of one handle, FP64 weights) equal the oracle's anneal with the same
    native sweeps row for row."""
    from conftest import compare_rows
    seed = 900 + L
    with pa.Engine(L=L, R=R, sweeps=3, dbeta=0.1, beta_final=1.0, seed=seed, coding="ssc", rng="native",
                   weights="fp64", graph=True, device=0) as e:
        form = e.sweep_form(0)
        assert form["spins_per_word"] == 32
        got = []
        for _ in range(2):
            e.run()
            got.append(e.rows(0))
    ref = oracle.anneal_ssc_bits_native(L, R, 3, 0.1, 1.0, 2, seed, seed, oracle.NATIVE_TAG_SSC, form["tile"])
    for r in range(2):
        compare_rows(got[r], ref[r], rtol=2e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("L,R,beta", [(8, 60, 0.44), (16, 33, 0.3), (24, 20, 0.9), (40, 17, 0.44),
                                      (56, 9, 0.35), (64, 12, 0.44), (136, 3, 0.44)])
def test_ssc_sweep_int8_native_stream_bit_exact(cuda, st, oracle, L, R, beta):
    """The int8 SSC sweep's byte-at-a-time acceptance (pa_ssc_sweep, native
    stream) equals the oracle's restatement bit for bit, energies included."""
    seed, step = 5000 + L, 2
    g = st.ssc_init(L, R, seed=seed, iseq=0)
    init = oracle.ssc_init(L, R, seed, 0)
    E, M = st.ssc_sweep(g, L, 3, beta, pa.RNG_NATIVE, seed=seed, iseq=0, step=step)
    T4, T8 = (int(x) for x in oracle.msc_thresholds(beta))
    ref = oracle.ssc_sweep_native(init, L, 3, T4, T8, seed, 1, oracle.NATIVE_TAG_SSC | step)
    got = g.cpu().numpy()
    assert (ref != init).any()
    assert np.array_equal(got, ref), f"{(got != ref).sum()} of {got.size} sites differ"
    oE, oM = oracle.ssc_energy(ref, L)
    assert np.array_equal(E.cpu().numpy(), oE) and np.array_equal(M.cpu().numpy(), oM)


@pytest.mark.gpu
@pytest.mark.parametrize("L,R,variant", [(40, 600, 0), (64, 500, 1)])
def test_ssc_anneal_native_stream_int8(cuda, oracle, L, R, variant):
    """Whole SSC anneals on the int8 sweep (L=40, whose bit-plane words would
    be 5/8 full, by default; L=64 by sweep_variant=1) equal the oracle's
    anneal with the same native sweeps row for row."""
    from conftest import compare_rows
    seed = 700 + L
    with pa.Engine(L=L, R=R, sweeps=3, dbeta=0.1, beta_final=1.0, seed=seed, coding="ssc", rng="native",
                   weights="fp64", graph=True, sweep_variant=variant, device=0) as e:
        assert e.sweep_form(0)["spins_per_word"] == 4
        e.run()
        got = e.rows(0)
    ref = oracle.anneal_ssc_bits_native(L, R, 3, 0.1, 1.0, 1, seed, seed, oracle.NATIVE_TAG_SSC, 0)
    compare_rows(got, ref[0], rtol=2e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("coding,L,R,P,sweeps,dbeta", [
    ("msc", 64, 2000, 4, 2, 0.05), ("ssc", 64, 2000, 4, 2, 0.05),
    ("msc", 16, 700, 3, 3, 0.1), ("msc", 96, 300, 2, 2, 0.1), ("msc", 128, 200, 2, 2, 0.2),
    ("msc", 256, 64, 2, 1, 0.25), ("ssc", 32, 500, 3, 3, 0.1), ("ssc", 128, 150, 2, 2, 0.2)])
def test_native_batch_each_population_equals_oracle(cuda, oracle, coding, L, R, P, sweeps, dbeta):
    """The batched form the benchmark times (runs=P concurrent populations of
    one configuration in one launch sequence, native stream, graph), here
    with FP64 weights so that every R_i must agree exactly: population k
    equals the oracle's anneal started at subsequence k << 40 with sweep tag
    | k, row for row -- at the headline's L=64 in both codings and in the
    other sweep forms a batch can take (stacked MSC tiles at L=16, the L=96
    kernel, L=128, clusters at L=256, SSC segments at L=32, two-word SSC rows
    at L=128).  The reference's -M runs (PAisingMSC.cu:583,784) are
    the sequential form this batching generalises."""
    from conftest import compare_rows
    seed = 4242 + L
    with pa.Engine(L=L, R=R, sweeps=sweeps, dbeta=dbeta, beta_final=1.0, runs=P, seed=seed, coding=coding,
                   rng="native", weights="fp64", graph=True, device=0) as e:
        e.run()
        assert e.num_sets() == P
        forms = [e.sweep_form(k) for k in range(P)]
        got = [e.rows(k) for k in range(P)]
    assert len({tuple(g[1:, 8]) for g in got}) == P  # disjoint streams: different trajectories
    for k in range(P):
        f = forms[k]
        if coding == "msc":
            threads = 256 if L <= 128 else {2: 1024, 4: 512}.get(f["cluster_ctas"], 256)
            ref = oracle.anneal_msc_native(L, R, sweeps, dbeta, 1.0, 1, seed, seed, oracle.NATIVE_TAG_MSC | k,
                                           threads, f["tile"], max(1, f["cluster_ctas"]), iseq0=k << 40)
        else:
            assert f["spins_per_word"] == 32
            ref = oracle.anneal_ssc_bits_native(L, R, sweeps, dbeta, 1.0, 1, seed, seed, oracle.NATIVE_TAG_SSC | k,
                                                f["tile"], iseq0=k << 40)
        compare_rows(got[k], ref[0], rtol=2e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("L,R,cs", [(64, 2000, 4), (64, 20000, 2), (96, 600, 4), (128, 9000, 4), (128, 30000, 2),
                                     (64, 40000, 1)])
def test_automatic_clusters_for_small_populations(cuda, oracle, L, R, cs):
    """A population with too few groups to keep the resident one-CTA sweep
    slots busy is swept by clusters of 4 or 2 CTAs per group (256 threads
    each) without being asked; the anneal equals the oracle's restatement of
    that form.  40000 replicas at L=64 keep one CTA per group."""
    from conftest import compare_rows
    seed, sweeps, dbeta = 300 + L, 2, 0.1
    with pa.Engine(L=L, R=R, sweeps=sweeps, dbeta=dbeta, beta_final=0.5, seed=seed, coding="msc", rng="native",
                   weights="fp64", graph=True, device=0) as e:
        f = e.sweep_form(0)
        assert f["cluster_ctas"] == cs, f
        e.run()
        got = e.rows(0)
    ref = oracle.anneal_msc_native(L, R, sweeps, dbeta, 0.5, 1, seed, seed, oracle.NATIVE_TAG_MSC, 256,
                                   f["tile"], max(1, f["cluster_ctas"]))
    compare_rows(got, ref[0], rtol=2e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("sizes", [(96, 64, 32, 96), (96, 96, 96), (96, 128, 48)])
def test_one_cta_batches_with_l96(cuda, oracle, sizes):
    """One CTA per group (sweep_variant=1) for batches holding L = 96: all
    of them L = 96 (the kernel built for that size alone) or mixed with
    other sizes (the general kernel that also carries L = 96's compile-time
    form, beside L = 64's and 128's and the general paths of L = 32 and 48);
    each population equals the oracle's anneal of that population alone,
    with its subsequence base and sweep tag."""
    from conftest import compare_rows
    pops = [dict(L=L, R=700 + 150 * k, seed=90 + k) for k, L in enumerate(sizes)]
    common = dict(sweeps=2, dbeta=0.1, beta_final=0.5, coding="msc", rng="native", weights="fp64", graph=True,
                  sweep_variant=1)
    with pa.Engine.batch(pops, **common) as e:
        forms = [e.sweep_form(k) for k in range(len(pops))]
        assert all(f["cluster_ctas"] == 1 for f in forms), forms
        e.run()
        got = [e.rows(k) for k in range(len(pops))]
    for k, p in enumerate(pops):
        ref = oracle.anneal_msc_native(p["L"], p["R"], 2, 0.1, 0.5, 1, p["seed"], pops[0]["seed"],
                                       oracle.NATIVE_TAG_MSC | k, 256, forms[k]["tile"], 1, iseq0=k << 40)
        compare_rows(got[k], ref[0], rtol=2e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("L,R,cs", [(256, 1000, 2), (256, 5000, 4), (144, 3000, 4), (192, 3000, 4)])
def test_automatic_clusters_for_large_lattices(cuda, oracle, L, R, cs):
    """Above L = 128 a population left to the engine is swept by clusters of
    4 CTAs of 512 threads when its groups exceed one resident wave of
    clusters of 2 (1024 threads, one CTA per SM: about 72-76 clusters on a
    GB300) and stay within eight such waves, else by clusters of 2; the
    anneal equals the oracle's restatement of that form."""
    from conftest import compare_rows
    seed = 700 + L
    with pa.Engine(L=L, R=R, sweeps=2, dbeta=0.25, beta_final=0.5, seed=seed, coding="msc", rng="native",
                   weights="fp64", graph=True, device=0) as e:
        f = e.sweep_form(0)
        assert f["cluster_ctas"] == cs, f
        e.run()
        got = e.rows(0)
    ref = oracle.anneal_msc_native(L, R, 2, 0.25, 0.5, 1, seed, seed, oracle.NATIVE_TAG_MSC, {2: 1024, 4: 512}[cs],
                                   1, cs)
    compare_rows(got, ref[0], rtol=2e-10)


@pytest.mark.gpu
def test_automatic_clusters_for_many_large_groups(cuda):
    """2048 groups at L = 256 (far beyond eight waves of clusters of 2) keep
    clusters of 2, as does a population that asks for them."""
    with pa.Engine(L=256, R=65536, sweeps=1, dbeta=0.5, beta_final=0.5, coding="msc", device=0) as e:
        assert e.sweep_form(0)["cluster_ctas"] == 2
    with pa.Engine(L=256, R=5000, sweeps=1, dbeta=0.5, beta_final=0.5, coding="msc", sweep_variant=2,
                   device=0) as e:
        assert e.sweep_form(0)["cluster_ctas"] == 2


@pytest.mark.gpu
def test_automatic_clusters_in_a_mixed_batch(cuda, oracle):
    """Populations of L = 64, 96 and 128 in one small batch share one
    automatically chosen cluster form (compile-time paths for 64 and 128, the
    general one for 96 in the same launch); each equals the oracle's run of
    that population alone with its subsequence base and sweep tag."""
    from conftest import compare_rows
    pops = [dict(L=64, R=1000, seed=41), dict(L=96, R=500, seed=42), dict(L=128, R=300, seed=43)]
    common = dict(sweeps=2, dbeta=0.1, beta_final=0.5, coding="msc", rng="native", weights="fp64", graph=True)
    with pa.Engine.batch(pops, **common) as e:
        forms = [e.sweep_form(k) for k in range(3)]
        assert all(f["cluster_ctas"] == forms[0]["cluster_ctas"] > 1 for f in forms), forms
        e.run()
        got = [e.rows(k) for k in range(3)]
    for k, p in enumerate(pops):
        ref = oracle.anneal_msc_native(p["L"], p["R"], 2, 0.1, 0.5, 1, p["seed"], pops[0]["seed"],
                                       oracle.NATIVE_TAG_MSC | k, 256, 1, forms[k]["cluster_ctas"], iseq0=k << 40)
        compare_rows(got[k], ref[0], rtol=2e-10)
