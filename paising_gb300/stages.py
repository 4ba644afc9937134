"""Stage entry points of the C ABI on torch CUDA tensors (torch provides the
device memory; every call goes through libpaising.so).

Each function replaces one reference kernel (group); see include/paising.h
for the file:line of the reference code each one replaces.
"""
from __future__ import annotations

import ctypes

import torch

from . import SSC, MSC, PaisingError, lib

__all__ = ["ssc_init", "ssc_sweep", "ssc_sweep_bits", "msc_init", "msc_sweep", "resample_plan", "ssc_resample", "msc_resample",
           "msc_resample_native"]


def _ptr(t: torch.Tensor | None):
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check(st: int) -> None:
    if st != 0:
        m = lib().pa_last_error(None)
        raise PaisingError(st, m.decode() if m else "")


def ssc_init(L: int, R: int, seed: int, iseq: int = 0, device="cuda") -> torch.Tensor:
    s = torch.empty((R, L * L), dtype=torch.int8, device=device)
    _check(lib().pa_ssc_init(_ptr(s), L, R, seed, iseq, _stream()))
    return s


def ssc_sweep(spins: torch.Tensor, L: int, sweeps: int, beta: float, rng: int, seed: int, iseq: int = 0,
              step: int = 1):
    """In place on spins [R, N] int8; returns (E, M) int32 tensors."""
    R = spins.shape[0]
    E = torch.empty(R, dtype=torch.int32, device=spins.device)
    M = torch.empty(R, dtype=torch.int32, device=spins.device)
    _check(lib().pa_ssc_sweep(_ptr(spins), L, R, sweeps, beta, rng, seed, iseq, step, _ptr(E), _ptr(M), _stream()))
    return E, M


def ssc_sweep_bits(spins: torch.Tensor, L: int, sweeps: int, beta: float, seed: int, step: int = 1):
    """The bit-plane sweep (native stream) in place on spins [R, N] int8;
    returns (E, M) int32 tensors."""
    R = spins.shape[0]
    E = torch.empty(R, dtype=torch.int32, device=spins.device)
    M = torch.empty(R, dtype=torch.int32, device=spins.device)
    _check(lib().pa_ssc_sweep_bits(_ptr(spins), L, R, sweeps, beta, seed, step, _ptr(E), _ptr(M), _stream()))
    return E, M


def msc_init(L: int, R: int, seed: int, iseq: int = 0, device="cuda"):
    rg = (R + 31) // 32
    w = torch.empty((rg, L * L), dtype=torch.int32, device=device)
    act = torch.empty(rg * 32, dtype=torch.uint8, device=device)
    _check(lib().pa_msc_init(_ptr(w), _ptr(act), L, R, seed, iseq, _stream()))
    return w, act


def msc_sweep(words: torch.Tensor, active: torch.Tensor, L: int, sweeps: int, beta: float, rng: int, seed: int,
              iseq: int = 0, step: int = 1):
    rg = words.shape[0]
    E = torch.empty(rg * 32, dtype=torch.int32, device=words.device)
    M = torch.empty(rg * 32, dtype=torch.int32, device=words.device)
    _check(lib().pa_msc_sweep(_ptr(words), _ptr(active), L, rg, sweeps, beta, rng, seed, iseq, step, _ptr(E),
                              _ptr(M), _stream()))
    return E, M


def resample_plan(E: torch.Tensor, active: torch.Tensor | None, coding: int, R_prev: int, Rinit: int, Rcap: int,
                  beta_prev: float, beta: float, e_ref: float, weights: int, seed: int, iseq: int):
    """Returns (roff, offs, src, lnQ, q, R_new)."""
    n = E.shape[0]
    dev = E.device
    roff = torch.empty(n, dtype=torch.int32, device=dev)
    offs = torch.empty(n, dtype=torch.int32, device=dev)
    src = torch.empty(Rcap + 1, dtype=torch.int32, device=dev)
    o = (ctypes.c_double * 3)()
    _check(lib().pa_resample_plan(_ptr(E), _ptr(active), coding, R_prev, Rinit, Rcap, beta_prev, beta, e_ref,
                                  weights, seed, iseq, _ptr(roff), _ptr(offs), _ptr(src), o, _stream()))
    return roff, offs, src, float(o[0]), float(o[1]), int(o[2])


def ssc_resample(old: torch.Tensor, L: int, src: torch.Tensor, R_new: int) -> torch.Tensor:
    new = torch.empty((R_new, L * L), dtype=torch.int8, device=old.device)
    _check(lib().pa_ssc_resample(_ptr(old), L, _ptr(src), R_new, _ptr(new), _stream()))
    return new


def msc_resample(old: torch.Tensor, L: int, src: torch.Tensor, R_new: int):
    rgn = (R_new + 31) // 32
    new = torch.empty((rgn, L * L), dtype=torch.int32, device=old.device)
    act = torch.empty(rgn * 32, dtype=torch.uint8, device=old.device)
    _check(lib().pa_msc_resample(_ptr(old), L, _ptr(src), R_new, _ptr(new), _ptr(act), _stream()))
    return new, act


def msc_resample_native(old: torch.Tensor, L: int, R_old: int, src: torch.Tensor, R_new: int):
    """The native stream's gather: offspring s at slot s (group s // 32, bit s % 32)."""
    rgn = (R_new + 31) // 32
    new = torch.empty((rgn, L * L), dtype=torch.int32, device=old.device)
    act = torch.empty(rgn * 32, dtype=torch.uint8, device=old.device)
    _check(lib().pa_msc_resample_native(_ptr(old), L, R_old, _ptr(src), R_new, _ptr(new), _ptr(act), _stream()))
    return new, act
