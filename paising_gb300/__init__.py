"""GB300-native population annealing for the 2D Ising ferromagnet.

Python mirror of the C ABI in include/paising.h (loaded with ctypes from the
in-tree build paising_gb300/_lib/libpaising.so).  There is no CPU fallback:
if the library is missing, importing the bindings raises.

The reference (LevBarash/PAising) is driven from its command line; the same
parameters appear here as keyword arguments with the reference defaults
(PAisingSSC.cu:27,35-50):

    >>> from paising_gb300 import Engine
    >>> with Engine(L=64, R=20000, sweeps=100, dbeta=0.005, beta_final=1.0,
    ...             coding="msc", seed=100) as eng:
    ...     eng.run()
    ...     rows = eng.rows()      # columns of PA_results_run_0.dat
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

__all__ = [
    "Engine", "PaisingError", "anneal", "load_library", "lib", "COLUMNS", "SSC", "MSC",
    "RNG_NATIVE", "RNG_REFERENCE", "schedule", "ref_word", "WEIGHTS_FP32", "WEIGHTS_FP64", "library_path",
]

_HERE = os.path.dirname(os.path.abspath(__file__))
library_path = os.path.join(_HERE, "_lib", "libpaising.so")

SSC, MSC = 0, 1
RNG_NATIVE, RNG_REFERENCE = 0, 1
WEIGHTS_FP32, WEIGHTS_FP64 = 0, 1
# columns of PA_results_run_<r>.dat (PAisingSSC.cu:679-690)
COLUMNS = ("beta", "E/N", "C/N", "|M|/N", "M2/N^2", "M4/N^4", "betaF/N", "S/N", "R", "lnQ")

_STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "capacity exceeded", 4: "population extinct",
           5: "call out of order", 6: "too many temperature steps"}


class PaisingError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        super().__init__(f"paising status {status} ({_STATUS.get(status, '?')}): {msg}")
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [("L", ctypes.c_int), ("R", ctypes.c_int), ("sweeps", ctypes.c_int), ("dbeta", ctypes.c_double),
                ("beta_final", ctypes.c_double), ("runs", ctypes.c_int), ("seed", ctypes.c_uint64),
                ("coding", ctypes.c_int), ("rng_mode", ctypes.c_int), ("weights", ctypes.c_int),
                ("graph", ctypes.c_int), ("device", ctypes.c_int), ("capacity", ctypes.c_double),
                ("sweep_variant", ctypes.c_int), ("tile_groups", ctypes.c_int), ("adaptive", ctypes.c_int),
                ("min_overlap", ctypes.c_double), ("max_overlap", ctypes.c_double), ("mhr", ctypes.c_int),
                ("store_energies", ctypes.c_int), ("family", ctypes.c_int)]


class Row(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("beta", "e", "c", "m", "m2", "m4", "bf", "s", "r", "lnq")]


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 24), ("launches", ctypes.c_int), ("total_ms", ctypes.c_double)]


class SweepForm(ctypes.Structure):
    _fields_ = [("spins_per_word", ctypes.c_int), ("replicas_per_word", ctypes.c_int), ("tile", ctypes.c_int),
                ("cluster_ctas", ctypes.c_int)]


_vp, _i, _u64, _d = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_double
_SIGS = {
    "pa_abi_version": ([], _i),
    "pa_config_init": ([ctypes.POINTER(Config)], _i),
    "pa_create": ([ctypes.POINTER(Config), ctypes.POINTER(_vp)], _i),
    "pa_run": ([_vp], _i),
    "pa_autotune": ([_vp, _vp, _i], _i),
    "pa_sweep_form": ([_vp, _i, ctypes.POINTER(SweepForm)], _i),
    "pa_get_mhr_rows": ([_vp, _i, _vp, _i, ctypes.POINTER(_i)], _i),
    "pa_get_energies": ([_vp, _i, _i, _vp, _i, ctypes.POINTER(_i)], _i),
    "pa_get_family_rows": ([_vp, _i, _vp, _i, ctypes.POINTER(_i)], _i),
    "pa_set_lattice_dump": ([_vp, ctypes.c_char_p, _i], _i),
    "pa_run_begin": ([_vp], _i),
    "pa_run_steps": ([_vp, _i, ctypes.POINTER(_i)], _i),
    "pa_run_end": ([_vp], _i),
    "pa_checkpoint": ([_vp, ctypes.c_char_p], _i),
    "pa_restore": ([_vp, ctypes.c_char_p], _i),
    "pa_checkpoint_verify": ([ctypes.c_char_p], _i),
    "pa_num_rows": ([_vp, ctypes.POINTER(_i)], _i),
    "pa_get_rows": ([_vp, _i, _vp, _i, ctypes.POINTER(_i)], _i),
    "pa_get_timing": ([_vp, ctypes.POINTER(_d), ctypes.POINTER(_d)], _i),
    "pa_write_results": ([_vp, ctypes.c_char_p, _i], _i),
    "pa_destroy": ([_vp], _i),
    "pa_status_string": ([_i], ctypes.c_char_p),
    "pa_last_error": ([_vp], ctypes.c_char_p),
    "pa_schedule": ([_d, _d, _vp, _i, ctypes.POINTER(_i)], _i),
    "pa_ref_word": ([_u64, _u64, _u64], ctypes.c_uint32),
    "pa_create_batch": ([ctypes.POINTER(Config), _i, ctypes.POINTER(_vp)], _i),
    "pa_num_sets": ([_vp, ctypes.POINTER(_i)], _i),
    "pa_set_population": ([_vp, _vp], _i),
    "pa_get_population": ([_vp, _i, _vp, ctypes.c_size_t, ctypes.POINTER(_i)], _i),
    "pa_profile_run": ([_vp, _vp, _i, ctypes.POINTER(_i)], _i),
    "pa_ssc_init": ([_vp, _i, _i, _u64, _u64, _vp], _i),
    "pa_ssc_sweep": ([_vp, _i, _i, _i, _d, _i, _u64, _u64, _i, _vp, _vp, _vp], _i),
    "pa_ssc_sweep_bits": ([_vp, _i, _i, _i, _d, _u64, _i, _vp, _vp, _vp], _i),
    "pa_msc_init": ([_vp, _vp, _i, _i, _u64, _u64, _vp], _i),
    "pa_msc_sweep": ([_vp, _vp, _i, _i, _i, _d, _i, _u64, _u64, _i, _vp, _vp, _vp], _i),
    "pa_resample_plan": ([_vp, _vp, _i, _i, _i, _i, _d, _d, _d, _i, _u64, _u64, _vp, _vp, _vp, _vp, _vp], _i),
    "pa_resample_plan_noalloc": ([_vp, _vp, _i, _i, _i, _i, _d, _d, _d, _i, _u64, _u64, _vp, _vp, _vp, _vp, _vp], _i),
    "pa_ssc_resample": ([_vp, _i, _vp, _i, _vp, _vp], _i),
    "pa_msc_resample": ([_vp, _i, _vp, _i, _vp, _vp, _vp], _i),
    "pa_msc_resample_native": ([_vp, _i, _i, _vp, _i, _vp, _vp, _vp], _i),
}

_lib: ctypes.CDLL | None = None


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Load libpaising.so and declare every C ABI signature.  Raises if the
    library has not been built (python -m paising_gb300.build)."""
    p = path or library_path
    if not os.path.exists(p):
        raise ImportError(f"paising CUDA library not built: {p} (run python -m paising_gb300.build)")
    L = ctypes.CDLL(p)
    for name, (args, res) in _SIGS.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    return L


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        _lib = load_library()
    return _lib


def _check(status: int, handle=None) -> None:
    if status != 0:
        msg = lib().pa_last_error(handle)
        raise PaisingError(status, msg.decode() if msg else "")


_CODING = {"ssc": SSC, "msc": MSC, SSC: SSC, MSC: MSC}
_RNG = {"native": RNG_NATIVE, "reference": RNG_REFERENCE, RNG_NATIVE: RNG_NATIVE, RNG_REFERENCE: RNG_REFERENCE}
_W = {"fp32": WEIGHTS_FP32, "fp64": WEIGHTS_FP64, WEIGHTS_FP32: WEIGHTS_FP32, WEIGHTS_FP64: WEIGHTS_FP64}


def make_config(L=64, R=20000, sweeps=100, dbeta=0.005, beta_final=1.0, runs=1, seed=1, coding="ssc",
                rng="native", weights="fp32", graph=True, device=0, capacity=1.25, sweep_variant=0,
                tile_groups=0, adaptive=False, min_overlap=0.0, max_overlap=0.0, mhr=False,
                store_energies=False, family=False) -> Config:
    """sweep_variant: CTAs per MSC group in the sweep kernel (0 automatic,
    1 one CTA, 2 or 4 a thread-block cluster); tile_groups: MSC groups per
    work unit of the one-CTA sweep (0 automatic, 1, 2, 4 or 8); adaptive:
    the reference's adaptive temperature step with histogram overlap in
    [min_overlap, max_overlap) (0 selects the reference's 0.85 / 0.87); mhr:
    multi-histogram reweighting after every run; store_energies: keep every
    temperature's energies; family: family statistics every temperature."""
    c = Config()
    _check(lib().pa_config_init(ctypes.byref(c)))
    c.L, c.R, c.sweeps, c.dbeta, c.beta_final, c.runs = int(L), int(R), int(sweeps), float(dbeta), float(beta_final), int(runs)
    c.seed, c.coding, c.rng_mode, c.weights = int(seed), _CODING[coding], _RNG[rng], _W[weights]
    c.graph, c.device, c.capacity = int(bool(graph)), int(device), float(capacity)
    c.sweep_variant, c.tile_groups = int(sweep_variant), int(tile_groups)
    c.adaptive, c.min_overlap, c.max_overlap = int(bool(adaptive)), float(min_overlap), float(max_overlap)
    c.mhr, c.store_energies, c.family = int(bool(mhr)), int(bool(store_energies)), int(bool(family))
    return c


class Engine:
    """One population configuration on one GPU (pa_create / pa_run / pa_get_rows)."""

    def __init__(self, **kw):
        self.config = make_config(**kw)
        self.configs = [self.config]
        h = ctypes.c_void_p()
        _check(lib().pa_create(ctypes.byref(self.config), ctypes.byref(h)))
        self._h = h

    @classmethod
    def batch(cls, populations: list[dict], **common) -> "Engine":
        """Independent populations of uneven size annealed together
        (pa_create_batch); result set k belongs to populations[k]."""
        e = cls.__new__(cls)
        e.configs = [make_config(**{**common, **p}) for p in populations]
        e.config = e.configs[0]
        arr = (Config * len(e.configs))(*e.configs)
        h = ctypes.c_void_p()
        _check(lib().pa_create_batch(arr, len(e.configs), ctypes.byref(h)))
        e._h = h
        return e

    def num_sets(self) -> int:
        n = ctypes.c_int()
        _check(lib().pa_num_sets(self._h, ctypes.byref(n)), self._h)
        return n.value

    def run(self) -> None:
        _check(lib().pa_run(self._h), self._h)

    def mhr_rows(self, set_index: int = 0) -> np.ndarray:
        """Multi-histogram reweighting of a result set: rows of (beta, E/N,
        C/N, betaF/N)."""
        n = ctypes.c_int()
        _check(lib().pa_get_mhr_rows(self._h, set_index, None, 0, ctypes.byref(n)), self._h)
        out = np.zeros((n.value, 4))
        _check(lib().pa_get_mhr_rows(self._h, set_index, out.ctypes.data, n.value, ctypes.byref(n)), self._h)
        return out

    def run_begin(self) -> None:
        """Start a host-stepped run (initial population, temperature 0)."""
        _check(lib().pa_run_begin(self._h), self._h)

    def run_steps(self, n: int) -> bool:
        """Advance up to n temperatures; True once the schedule is complete."""
        d = ctypes.c_int()
        _check(lib().pa_run_steps(self._h, int(n), ctypes.byref(d)), self._h)
        return bool(d.value)

    def run_end(self) -> None:
        """Collect the rows of a stepped run (as run())."""
        _check(lib().pa_run_end(self._h), self._h)

    def checkpoint(self, path: str) -> None:
        """Complete state of a stepped run to a file (between steps)."""
        _check(lib().pa_checkpoint(self._h, path.encode()), self._h)

    def restore(self, path: str) -> None:
        """Continue a checkpointed run in this handle (same configuration)."""
        _check(lib().pa_restore(self._h, path.encode()), self._h)

    @staticmethod
    def verify_checkpoint(path: str) -> None:
        """File-level checks of a checkpoint (host only): raises PaisingError
        for a file pa_restore would refuse whatever the handle."""
        _check(lib().pa_checkpoint_verify(path.encode()))

    def set_lattice_dump(self, directory: str | None, precision: int = 11) -> None:
        """Per-temperature population text files of the first run
        (PA_lattice_<i>.dat); None switches them off."""
        d = None if directory is None else directory.encode()
        _check(lib().pa_set_lattice_dump(self._h, d, int(precision)), self._h)

    def family_rows(self, set_index: int = 0) -> np.ndarray:
        """Family statistics of a result set: rows of (families, rho_t, S_f)."""
        n = ctypes.c_int()
        _check(lib().pa_get_family_rows(self._h, set_index, None, 0, ctypes.byref(n)), self._h)
        out = np.zeros((n.value, 3))
        _check(lib().pa_get_family_rows(self._h, set_index, out.ctypes.data, n.value, ctypes.byref(n)), self._h)
        return out

    def energies(self, set_index: int = 0, step: int = 0) -> np.ndarray:
        """Energies of a result set's population at one temperature."""
        n = ctypes.c_int()
        _check(lib().pa_get_energies(self._h, set_index, step, None, 0, ctypes.byref(n)), self._h)
        out = np.zeros(n.value, dtype=np.int32)
        _check(lib().pa_get_energies(self._h, set_index, step, out.ctypes.data, n.value, ctypes.byref(n)), self._h)
        return out

    def autotune(self) -> list[int]:
        """Time the sweep forms and keep the fastest (pa_autotune): MSC groups
        per work unit, SSC int8 or bit-plane sweep.  Returns each population's
        work-unit size (sweep_form() gives the whole form)."""
        n = len(self.configs)
        arr = (ctypes.c_int * n)()
        _check(lib().pa_autotune(self._h, arr, n), self._h)
        return list(arr)

    def sweep_form(self, index: int = 0) -> dict:
        """{spins_per_word, replicas_per_word, tile, cluster_ctas} of population
        `index` (pa_sweep_form)."""
        f = SweepForm()
        _check(lib().pa_sweep_form(self._h, index, ctypes.byref(f)), self._h)
        return {k: getattr(f, k) for k, _ in SweepForm._fields_}

    def num_rows(self) -> int:
        n = ctypes.c_int()
        _check(lib().pa_num_rows(self._h, ctypes.byref(n)), self._h)
        return n.value

    def rows(self, set: int = 0) -> np.ndarray:
        """Rows of result set `set` (a population, or a sequential run)."""
        n = self.num_rows()
        out = np.zeros((n, 10), dtype=np.float64)
        got = ctypes.c_int()
        _check(lib().pa_get_rows(self._h, set, out.ctypes.data, n, ctypes.byref(got)), self._h)
        return out[: got.value]

    def timing(self) -> tuple[float, float]:
        """(device milliseconds of the last run() over all runs, spin-flip attempts)."""
        ms, att = ctypes.c_double(), ctypes.c_double()
        _check(lib().pa_get_timing(self._h, ctypes.byref(ms), ctypes.byref(att)), self._h)
        return ms.value, att.value

    def set_population(self, host_ptr) -> None:
        """Initial population from host memory (pointer or numpy array in the
        coding's layout); None restores the random initialisation."""
        p = host_ptr.ctypes.data if isinstance(host_ptr, np.ndarray) else host_ptr
        _check(lib().pa_set_population(self._h, p), self._h)

    def population(self, pop: int = 0) -> np.ndarray:
        """Final population of population `pop` (SSC int8 [R, N]; MSC uint32 [rg, N])."""
        c = self.configs[pop] if len(self.configs) > 1 else self.config
        N = c.L * c.L
        cap = int(c.R * c.capacity) + 512
        rg = (cap + 31) // 32
        buf = np.zeros(rg * N if c.coding == MSC else cap * N, dtype=np.uint32 if c.coding == MSC else np.int8)
        R = ctypes.c_int()
        _check(lib().pa_get_population(self._h, pop, buf.ctypes.data, buf.nbytes, ctypes.byref(R)), self._h)
        if c.coding == MSC:
            return buf[: ((R.value + 31) // 32) * N].reshape(-1, N)
        return buf[: R.value * N].reshape(R.value, N)

    def profile(self) -> dict:
        """{kernel: (launches, total ms)} of one run timed launch by launch."""
        arr = (KernelTime * 32)()
        n = ctypes.c_int()
        _check(lib().pa_profile_run(self._h, arr, 32, ctypes.byref(n)), self._h)
        return {arr[i].name.decode(): (arr[i].launches, arr[i].total_ms) for i in range(min(n.value, 32))}

    def write_results(self, directory: str, precision: int = 11) -> None:
        os.makedirs(directory, exist_ok=True)
        _check(lib().pa_write_results(self._h, directory.encode(), int(precision)), self._h)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().pa_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def schedule(dbeta: float = 0.005, beta_final: float = 1.0) -> np.ndarray:
    """The reference's inverse-temperature schedule (pa_schedule)."""
    n = ctypes.c_int()
    lib().pa_schedule(dbeta, beta_final, None, 0, ctypes.byref(n))
    out = np.zeros(n.value)
    _check(lib().pa_schedule(dbeta, beta_final, out.ctypes.data, n.value, ctypes.byref(n)))
    return out


def ref_word(seed: int, subseq: int, ctr: int) -> int:
    return int(lib().pa_ref_word(seed, subseq, ctr))


def anneal(**kw) -> np.ndarray:
    """Run a full anneal and return the rows of run 0 (or all runs stacked
    when runs > 1)."""
    with Engine(**kw) as e:
        e.run()
        n = e.num_sets()
        return e.rows(0) if n == 1 else np.stack([e.rows(r) for r in range(n)])
