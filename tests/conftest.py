import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine through libpaising.so")
    config.addinivalue_line("markers", "slow: full-size anneals (seconds each)")


def load_dat(name: str) -> np.ndarray:
    """A PA_results_run_<r>.dat fixture (10 columns)."""
    return np.loadtxt(os.path.join(GOLDEN, name))


@pytest.fixture(scope="session")
def oracle():
    from oracle import pa_oracle
    pa_oracle.lib()
    return pa_oracle


@pytest.fixture(scope="session")
def engine_lib():
    import paising_gb300
    return paising_gb300.lib()


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def st(cuda):
    """The stage-level entry points (paising_gb300.stages)."""
    from paising_gb300 import stages
    return stages


def compare_rows(got: np.ndarray, ref: np.ndarray, rtol: float = 1e-9, exact_R: bool = True):
    """Rows of a results file: the population size column exactly, the rest to
    rtol (relative, with an absolute floor for values that are ~0)."""
    assert got.shape == ref.shape, (got.shape, ref.shape)
    if exact_R:
        bad = np.nonzero(got[:, 8] != ref[:, 8])[0]
        assert bad.size == 0, f"R differs first at row {bad[0] if bad.size else -1}: {got[bad[:3], 8]} vs {ref[bad[:3], 8]}"
    scale = np.maximum(np.abs(ref), 1e-12)
    rel = np.abs(got - ref) / scale
    worst = np.unravel_index(np.argmax(rel), rel.shape)
    assert rel.max() <= rtol, f"max rel diff {rel.max():.3e} at row {worst[0]} col {worst[1]}: {got[worst]} vs {ref[worst]}"
