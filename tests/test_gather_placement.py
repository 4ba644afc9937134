"""The native stream's MSC placement and the arithmetic its gather relies on
(CPU, no GPU): offspring s goes to slot s (group s // 32, bit s % 32), and a
new group's word at any site is OR_d ((W >> d) & M_d) over the distinct
shifts d = o_b - b of its bits, W being the four old words starting one
before the first source's, o_b the source's offset in W.  Checked against
the oracle's restatement of the placement (oracle/native_stream.c) and
against a bit-by-bit numpy gather, with the copy-number patterns of the
GPU stage test."""
import numpy as np
import pytest


def _copy_numbers(kind, n, rng):
    if kind == "mixed":
        return rng.integers(0, 4, n)
    if kind == "identity":
        return np.ones(n, dtype=np.int64)
    if kind == "sparse":
        return np.where(rng.random(n) < 0.2, 4, 0)
    if kind == "bursty":
        return np.repeat(rng.choice([0, 1, 3], size=n // 40 + 1, p=[0.4, 0.3, 0.3]), 40)[:n]
    roff = np.ones(n, dtype=np.int64)
    roff[300:450] = 0
    return roff


def _shift_gather(old, src, Rn):
    """New words from the distinct-shift decomposition (the kernel's method;
    groups whose sources leave the four-word window bit by bit)."""
    rgn, N = (Rn + 31) // 32, old.shape[1]
    new = np.zeros((rgn, N), dtype=np.uint32)
    fallbacks = 0
    for j in range(rgn):
        s = src[32 * j:32 * j + 32].astype(np.int64)
        first = s[0] >> 5
        d = s - 32 * (first - 1) - np.arange(len(s))
        assert (d >= 1).all()
        if (d >= 96).any():
            fallbacks += 1
            for b, lin in enumerate(s):
                new[j] |= ((old[lin >> 5] >> np.uint32(lin & 31)) & np.uint32(1)) << np.uint32(b)
            continue
        W = [old[min(max(first - 1 + q, 0), old.shape[0] - 1)].astype(np.uint64) for q in range(4)]
        for dv in np.unique(d):
            mask = int(np.bitwise_or.reduce(np.left_shift(1, np.nonzero(d == dv)[0])))
            k, sh = int(dv) >> 5, int(dv) & 31
            new[j] |= (((W[k + 1] << np.uint64(32)) | W[k]) >> np.uint64(sh)).astype(np.uint32) & np.uint32(mask)
    return new, fallbacks


@pytest.mark.parametrize("L,R,kind", [(16, 200, "mixed"), (64, 3000, "mixed"), (64, 5000, "identity"),
                                      (32, 4000, "sparse"), (128, 700, "bursty"), (10, 33, "mixed"),
                                      (16, 900, "gap")])
def test_native_placement_and_shift_decomposition(oracle, L, R, kind):
    old, act = oracle.msc_init(L, R, 4, 0)
    rng = np.random.default_rng(R + L)
    n = len(act)
    roff = (_copy_numbers(kind, n, rng) * act).astype(np.uint32)
    offs, tot = oracle.scan(roff)
    src = np.repeat(np.arange(n), roff)
    ref, ref_act = oracle.msc_resample_linear(old, L, roff, offs, tot)
    # the placement itself: new slot s holds old replica src[s]
    bits = lambda w, lin: (w[lin >> 5] >> (lin & 31).astype(np.uint32)) & np.uint32(1)
    for s in rng.choice(tot, size=min(tot, 64), replace=False):
        assert np.array_equal((ref[s // 32] >> np.uint32(s % 32)) & np.uint32(1), bits(old, np.array([src[s]]))[0])
    assert np.array_equal(ref_act[:tot], np.ones(tot, np.uint8)) and not ref_act[tot:].any()
    got, fallbacks = _shift_gather(old, src, tot)
    assert np.array_equal(got, ref)
    if kind == "gap":
        assert fallbacks >= 1  # sources more than the window apart
    if kind == "identity":
        assert fallbacks == 0
