"""ctypes bindings of the oracle library oracle/_build/libpaoracle.so.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() to
verify the engine's results and by bench.py's cpu_baseline / reference legs.
The product package never imports this module.

Every function restates one stage of the reference (see pa_oracle.c for the
file:line of each) on numpy arrays in the reference's own layouts.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpaoracle.so")

_vp, _i, _u64, _d, _u32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_double, ctypes.c_uint32
_SIGS = {
    "or_H": ([_u64, _u64, _u64], _u32),
    "or_philox": ([_vp, _vp, _vp], None),
    "or_set_threads": ([_i], None),
    "or_max_threads": ([], _i),
    "or_ssc_init": ([_vp, _i, _i, _u64, _u64], None),
    "or_ssc_boltz": ([_d, _vp], None),
    "or_ssc_sweep": ([_vp, _i, _i, _i, _vp, _u64, _u64], None),
    "or_ssc_energy": ([_vp, _i, _i, _vp, _vp], None),
    "or_ssc_q": ([_vp, _i, _d, _d], _d),
    "or_ssc_copy_numbers": ([_vp, _i, _i, _d, _d, _u64, _u64, _vp], _u32),
    "or_scan": ([_vp, _i, _vp], _u32),
    "or_ssc_resample": ([_vp, _i, _i, _vp, _vp, _vp], None),
    "or_averages": ([_vp, _vp, _vp, _i, _vp], None),
    "or_msc_init": ([_vp, _vp, _i, _i, _i, _u64, _u64], None),
    "or_msc_thresholds": ([_d, _vp], None),
    "or_msc_sweep": ([_vp, _i, _i, _i, _vp, _u64, _u64], None),
    "or_msc_energy": ([_vp, _i, _i, _vp, _vp], None),
    "or_msc_q": ([_vp, _vp, _i, _d, _d], _d),
    "or_msc_copy_numbers": ([_vp, _vp, _i, _i, _i, _d, _d, _u64, _u64, _vp], _u32),
    "or_msc_resample": ([_vp, _vp, _i, _i, _vp, _vp, _i, _vp, _vp, _vp], None),
    "or_msc_resample_linear": ([_vp, _vp, _i, _i, _vp, _vp, _i, _vp, _vp, _vp], None),
    "or_anneal": ([_i, _i, _i, _i, _d, _d, _i, _u64, _i, _vp, _i, _vp], _i),
    "or_anneal2": ([_i, _i, _i, _i, _d, _d, _i, _u64, _i, _i, _d, _d, _vp, _i, _vp, _vp], _i),
    "or_kaufman": ([_i, _d, _vp, _vp, _vp], None),
    "or_anneal_msc_native": ([_i, _i, _i, _d, _d, _i, _u64, _u64, _u32, _u64, _i, _i, _i, _vp, _i, _vp], _i),
    "or_anneal_ssc_bits_native": ([_i, _i, _i, _d, _d, _i, _u64, _u64, _u32, _u64, _i, _vp, _i, _vp], _i),
    "or_ssc_sweep_native": ([_vp, _i, _i, _i, _u32, _u32, _u64, _u32, _u32], None),
    "or_ssc_sweep_bits_native": ([_vp, _i, _i, _i, _u32, _u32, _u64, _u32, _u32, _i], _i),
    "or_native_accept4": ([_vp, _vp, _vp, _vp, _i, _u32, _u32, _u32, _u32, _u64, _u32, _u32], None),
    "or_msc_sweep_native": ([_vp, _i, _i, _i, _u32, _u32, _u64, _u32, _u32, _i], None),
}

_lib = None


def build() -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or any(
                os.path.getmtime(os.path.join(HERE, f)) > os.path.getmtime(LIB_PATH)
                for f in ("pa_oracle.c", "native_stream.c", "kaufman.c", "inj_stream.h")):
            build()
        L = ctypes.CDLL(LIB_PATH)
        for n, (a, r) in _SIGS.items():
            f = getattr(L, n)
            f.argtypes = a
            f.restype = r
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags.c_contiguous
    return a.ctypes.data


def H(seed: int, subseq: int, ctr: int) -> int:
    return int(lib().or_H(seed, subseq, ctr))


def philox(key, ctr) -> np.ndarray:
    k = np.asarray(key, dtype=np.uint32)
    c = np.asarray(ctr, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().or_philox(_p(k), _p(c), _p(o))
    return o


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def max_threads() -> int:
    return int(lib().or_max_threads())


# ------------------------------------------------------------------ SSC
def ssc_init(L: int, R: int, seed: int, iseq: int) -> np.ndarray:
    s = np.zeros((R, L * L), dtype=np.int8)
    lib().or_ssc_init(_p(s), L, R, seed, iseq)
    return s


def ssc_boltz(beta: float) -> np.ndarray:
    t = np.zeros(10)
    lib().or_ssc_boltz(beta, _p(t))
    return t


def ssc_sweep(spins: np.ndarray, L: int, sweeps: int, beta: float, seed: int, iseq: int) -> np.ndarray:
    s = np.ascontiguousarray(spins, dtype=np.int8).copy()
    lib().or_ssc_sweep(_p(s), L, s.shape[0], sweeps, _p(ssc_boltz(beta)), seed, iseq)
    return s


def ssc_energy(spins: np.ndarray, L: int):
    s = np.ascontiguousarray(spins, dtype=np.int8)
    E = np.zeros(s.shape[0], dtype=np.int32)
    M = np.zeros(s.shape[0], dtype=np.int32)
    lib().or_ssc_energy(_p(s), L, s.shape[0], _p(E), _p(M))
    return E, M


def ssc_q(E: np.ndarray, dB: float, Emean: float) -> float:
    E = np.ascontiguousarray(E, dtype=np.int32)
    return float(lib().or_ssc_q(_p(E), len(E), dB, Emean))


def ssc_copy_numbers(E, Rinit, lnQ, dB, seed, iseq):
    E = np.ascontiguousarray(E, dtype=np.int32)
    roff = np.zeros(len(E), dtype=np.uint32)
    Rn = lib().or_ssc_copy_numbers(_p(E), len(E), Rinit, lnQ, dB, seed, iseq, _p(roff))
    return roff, int(Rn)


def scan(roff: np.ndarray):
    roff = np.ascontiguousarray(roff, dtype=np.uint32)
    offs = np.zeros(len(roff), dtype=np.uint32)
    tot = lib().or_scan(_p(roff), len(roff), _p(offs))
    return offs, int(tot)


def ssc_resample(old: np.ndarray, L: int, roff, offs, Rnew: int) -> np.ndarray:
    old = np.ascontiguousarray(old, dtype=np.int8)
    new = np.zeros((Rnew, L * L), dtype=np.int8)
    lib().or_ssc_resample(_p(old), L, old.shape[0], _p(np.ascontiguousarray(roff, np.uint32)),
                          _p(np.ascontiguousarray(offs, np.uint32)), _p(new))
    return new


def averages(E, M, active=None) -> np.ndarray:
    E = np.ascontiguousarray(E, dtype=np.int32)
    M = np.ascontiguousarray(M, dtype=np.int32)
    a = np.zeros(5)
    act = None if active is None else np.ascontiguousarray(active, dtype=np.uint8)
    lib().or_averages(_p(E), _p(M), None if act is None else _p(act), len(E), _p(a))
    return a


# ------------------------------------------------------------------ MSC
def msc_init(L: int, R: int, seed: int, iseq: int):
    rg = (R + 31) // 32
    w = np.zeros((rg, L * L), dtype=np.uint32)
    act = np.zeros(rg * 32, dtype=np.uint8)
    lib().or_msc_init(_p(w), _p(act), L, R, rg, seed, iseq)
    return w, act


def msc_thresholds(beta: float) -> np.ndarray:
    t = np.zeros(2, dtype=np.uint32)
    lib().or_msc_thresholds(beta, _p(t))
    return t


def msc_sweep(words: np.ndarray, L: int, sweeps: int, beta: float, seed: int, iseq: int) -> np.ndarray:
    w = np.ascontiguousarray(words, dtype=np.uint32).copy()
    lib().or_msc_sweep(_p(w), L, w.shape[0], sweeps, _p(msc_thresholds(beta)), seed, iseq)
    return w


def msc_energy(words: np.ndarray, L: int):
    w = np.ascontiguousarray(words, dtype=np.uint32)
    E = np.zeros(w.shape[0] * 32, dtype=np.int32)
    M = np.zeros(w.shape[0] * 32, dtype=np.int32)
    lib().or_msc_energy(_p(w), L, w.shape[0], _p(E), _p(M))
    return E, M


def msc_q(E, active, dB, Emean) -> float:
    E = np.ascontiguousarray(E, dtype=np.int32)
    act = np.ascontiguousarray(active, dtype=np.uint8)
    return float(lib().or_msc_q(_p(E), _p(act), len(E) // 32, dB, Emean))


def msc_copy_numbers(E, active, Rinit, R, lnQ, dB, seed, iseq):
    E = np.ascontiguousarray(E, dtype=np.int32)
    act = np.ascontiguousarray(active, dtype=np.uint8)
    roff = np.zeros(len(E), dtype=np.uint32)
    Rn = lib().or_msc_copy_numbers(_p(E), _p(act), len(E) // 32, Rinit, R, lnQ, dB, seed, iseq, _p(roff))
    return roff, int(Rn)


def msc_resample(old: np.ndarray, L: int, roff, offs, Rnew: int):
    old = np.ascontiguousarray(old, dtype=np.uint32)
    rgn = (Rnew + 31) // 32
    new = np.zeros((rgn, L * L), dtype=np.uint32)
    act = np.zeros(rgn * 32, dtype=np.uint8)
    E0 = np.zeros(old.shape[0] * 32, dtype=np.int32)
    lib().or_msc_resample(_p(old), _p(E0), L, old.shape[0], _p(np.ascontiguousarray(roff, np.uint32)),
                          _p(np.ascontiguousarray(offs, np.uint32)), rgn, _p(new), _p(act), None)
    return new, act


def msc_resample_linear(old: np.ndarray, L: int, roff, offs, Rnew: int):
    """The native stream's MSC placement: offspring s at slot s (group s // 32,
    bit s % 32); native_stream.c."""
    old = np.ascontiguousarray(old, dtype=np.uint32)
    rgn = (Rnew + 31) // 32
    new = np.zeros((rgn, L * L), dtype=np.uint32)
    act = np.zeros(rgn * 32, dtype=np.uint8)
    E0 = np.zeros(old.shape[0] * 32, dtype=np.int32)
    lib().or_msc_resample_linear(_p(old), _p(E0), L, old.shape[0], _p(np.ascontiguousarray(roff, np.uint32)),
                                 _p(np.ascontiguousarray(offs, np.uint32)), rgn, _p(new), _p(act), None)
    return new, act


# ------------------------------------------------- the engine's native stream
# (native_stream.c: no counterpart in the reference; pins the engine's
# production sweep bit for bit)
NATIVE_TAG_MSC = 0x4D << 24     # 'M' in the top byte of counter word 3
NATIVE_TAG_SSC = 0x53 << 24     # 'S': the SSC sweeps
FINISH_TAG_FLIP = 0x20 << 24    # single-bit finishing words: 'M' -> 'm'


def native_accept4(a, und, acc, site, nvalid, chain, c1, step, tag, key, T4, T8) -> np.ndarray:
    """Accepted bits of a batch of four word-sites (uint32[4])."""
    a = np.ascontiguousarray(a, dtype=np.uint32)
    und = np.ascontiguousarray(und, dtype=np.uint32)
    out = np.ascontiguousarray(acc, dtype=np.uint32).copy()
    site = np.ascontiguousarray(site, dtype=np.uint32)
    lib().or_native_accept4(_p(a), _p(und), _p(out), _p(site), nvalid, chain, c1, step, tag, key, T4, T8)
    return out


def msc_sweep_native(words: np.ndarray, L: int, sweeps: int, T4: int, T8: int, key: int, step: int, tag: int,
                     threads: int = 256) -> np.ndarray:
    """Native-stream MSC sweeps of the engine's one-CTA sweep (one group per
    work unit) on a copy of words [rg][N]."""
    w = np.ascontiguousarray(words, dtype=np.uint32).copy()
    lib().or_msc_sweep_native(_p(w), L, w.shape[0], sweeps, T4, T8, key, step, tag, threads)
    return w


# ---------------------------------------------------------- full anneal
def anneal(coding: str, L: int, R: int, sweeps: int, dbeta: float = 0.005, beta_final: float = 1.0,
           runs: int = 1, seed: int = 1, max_steps: int = 0, adaptive: bool = False, min_overlap: float = 0.85,
           max_overlap: float = 0.87):
    """Rows of PA_results_run_<r>.dat for every run (shape runs x nrows x 10)
    and the spin-flip attempt count.  adaptive: the AdaptiveStep build, with
    dbeta the first step."""
    rows, _, att = anneal_family(coding, L, R, sweeps, dbeta, beta_final, runs, seed, max_steps, adaptive,
                                 min_overlap, max_overlap, family=False)
    return rows, att


def anneal_family(coding: str, L: int, R: int, sweeps: int, dbeta: float = 0.005, beta_final: float = 1.0,
                  runs: int = 1, seed: int = 1, max_steps: int = 0, adaptive: bool = False,
                  min_overlap: float = 0.85, max_overlap: float = 0.87, family: bool = True):
    """anneal() plus the family statistics of every temperature (runs x nrows
    x 3: families, rho_t, S_f)."""
    maxr = 10000 if adaptive else int(beta_final / dbeta) + 8
    rows = np.zeros((runs, maxr, 10))
    fam = np.zeros((runs, maxr, 3)) if family else None
    att = ctypes.c_double()
    n = lib().or_anneal2(1 if coding == "msc" else 0, L, R, sweeps, dbeta, beta_final, runs, seed, max_steps,
                         int(adaptive), min_overlap, max_overlap, _p(rows), maxr,
                         _p(fam) if family else None, ctypes.byref(att))
    if n < 0:
        raise RuntimeError("oracle anneal failed")
    return rows[:, :n], (fam[:, :n] if family else None), att.value


def bits_layout(L: int):
    """(words per sublattice row, sites per segment, segments per word) of the
    SSC bit-plane sweep, or None where L has no layout."""
    if L < 8 or L % 8 or L > 256:
        return None
    S = L // 2
    for w in range((S + 31) // 32, 9):
        if S % w == 0 and (S // w) % 4 == 0:
            return w, S // w, (32 // (S // w) if w == 1 else 1)
    return None


def bits_max_tile(L: int) -> int:
    """Replicas per tile of the bit-plane sweep when none is asked for: the
    word groups of 1024 words per sublattice plane (at least one), at most
    256 replicas."""
    Wq, seg, segs = bits_layout(L)
    gw = max(1, 1024 // (L * Wq))
    if gw * segs > 256:
        gw = 256 // segs
    return gw * segs


def ssc_sweep_bits_native(spins: np.ndarray, L: int, sweeps: int, T4: int, T8: int, key: int, step: int, tag: int,
                          tile: int) -> np.ndarray:
    """Native-stream SSC sweeps on bit planes with `tile` replicas per work
    unit, on a copy of spins [R][N] (int8 +-1)."""
    s = np.ascontiguousarray(spins, dtype=np.int8).copy()
    if not lib().or_ssc_sweep_bits_native(_p(s), L, s.shape[0], sweeps, T4, T8, key, step, tag, tile):
        raise ValueError(f"no bit-plane layout for L={L} with {tile} replicas per tile")
    return s


def anneal_msc_native(L: int, R: int, sweeps: int, dbeta: float, beta_final: float, runs: int, seed: int,
                      key: int, tag: int, threads: int = 256, tile: int = 1, cluster: int = 1, iseq0: int = 0):
    """Rows of `runs` sequential MSC runs whose sweeps use the engine's
    native stream: runs x nrows x 10.  tile: groups per work unit of the
    one-CTA sweep; cluster: CTAs per group (threads = threads per CTA);
    iseq0: first subsequence of the reference-coordinate draws (population k
    of an engine batch: k << 40, with tag | k)."""
    maxr = int(beta_final / dbeta) + 8
    rows = np.zeros((runs, maxr, 10))
    att = ctypes.c_double()
    n = lib().or_anneal_msc_native(L, R, sweeps, dbeta, beta_final, runs, seed, key, tag, iseq0, threads, tile,
                                   cluster, _p(rows), maxr, ctypes.byref(att))
    if n < 0:
        raise RuntimeError("oracle anneal failed")
    return rows[:, :n]


def ssc_sweep_native(spins: np.ndarray, L: int, sweeps: int, T4: int, T8: int, key: int, step: int,
                     tag: int) -> np.ndarray:
    """Native-stream SSC sweeps one int8 spin per site, on a copy of spins."""
    s = np.ascontiguousarray(spins, dtype=np.int8).copy()
    lib().or_ssc_sweep_native(_p(s), L, s.shape[0], sweeps, T4, T8, key, step, tag)
    return s


def anneal_ssc_bits_native(L: int, R: int, sweeps: int, dbeta: float, beta_final: float, runs: int, seed: int,
                           key: int, tag: int, tile: int, iseq0: int = 0):
    """Rows of `runs` sequential SSC runs swept on bit planes with the
    engine's native stream, `tile` replicas per work unit (0: the int8 sweep):
    runs x nrows x 10.  iseq0 as in anneal_msc_native."""
    maxr = int(beta_final / dbeta) + 8
    rows = np.zeros((runs, maxr, 10))
    att = ctypes.c_double()
    n = lib().or_anneal_ssc_bits_native(L, R, sweeps, dbeta, beta_final, runs, seed, key, tag, iseq0, tile,
                                        _p(rows), maxr, ctypes.byref(att))
    if n < 0:
        raise RuntimeError("oracle anneal failed")
    return rows[:, :n]


def kaufman(L: int, beta: float):
    """(ln Z, <E>, C) of the L x L torus, whole lattice."""
    a, e, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    lib().or_kaufman(L, beta, ctypes.byref(a), ctypes.byref(e), ctypes.byref(c))
    return a.value, e.value, c.value
