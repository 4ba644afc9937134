"""The C ABI library loads and exports every entry point include/paising.h
declares; argument checking and host-side helpers work without a GPU."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "paising.h")).read()
    return sorted(set(re.findall(r"PA_API\s+[\w\s\*]+?\b(pa_\w+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("pa_create", "pa_run", "pa_get_rows", "pa_destroy", "pa_ssc_sweep", "pa_msc_sweep", "pa_resample_plan"):
        assert s in syms


def test_library_exports_every_declared_symbol(engine_lib):
    import paising_gb300
    missing = [s for s in declared_symbols() if not hasattr(engine_lib, s)]
    assert not missing, missing
    # and the binding table covers them all
    assert set(declared_symbols()) <= set(paising_gb300._SIGS)


def test_no_oracle_in_product():
    """The product never links or imports the oracle."""
    for dp, _, fs in os.walk(os.path.join(ROOT, "paising_gb300")):
        for f in fs:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                txt = open(os.path.join(dp, f), errors="ignore").read()
                assert "oracle" not in re.sub(r"(//|#).*", "", txt).lower() or f == "__init__.py", f


def test_status_strings_and_defaults(engine_lib):
    import paising_gb300 as pa
    assert engine_lib.pa_abi_version() == 1
    assert engine_lib.pa_status_string(0) == b"ok"
    assert b"capacity" in engine_lib.pa_status_string(3)
    c = pa.Config()
    assert engine_lib.pa_config_init(ctypes.byref(c)) == 0
    assert (c.L, c.R, c.sweeps, c.dbeta, c.beta_final, c.runs) == (64, 20000, 100, 0.005, 1.0, 1)


@pytest.mark.parametrize("kw", [dict(L=12, coding="ssc"), dict(L=7, coding="msc"), dict(R=0), dict(sweeps=-1),
                                dict(dbeta=0.0), dict(capacity=0.5), dict(L=264, coding="msc"),
                                dict(L=256, coding="msc", sweep_variant=1), dict(L=64, coding="ssc", sweep_variant=2),
                                dict(R=2_000_000_000), dict(R=1_000_000_000, capacity=2.5),
                                dict(L=64, coding="msc", sweep_variant=3), dict(L=10, coding="msc", sweep_variant=2)])
def test_create_rejects_bad_arguments(engine_lib, kw):
    import paising_gb300 as pa
    with pytest.raises(pa.PaisingError) as ei:
        pa.Engine(**kw)
    assert ei.value.status == 1


def test_too_many_steps(engine_lib):
    import paising_gb300 as pa
    with pytest.raises(pa.PaisingError) as ei:
        pa.Engine(dbeta=1e-5, beta_final=1.0)
    assert ei.value.status == 6


def test_stage_argument_checks(engine_lib):
    # invalid sizes are rejected before any device work
    assert engine_lib.pa_ssc_sweep(None, 64, 10, 1, 0.4, 0, 1, 0, 1, None, None, None) == 1
    assert engine_lib.pa_msc_sweep(None, None, 64, 1, 1, 0.4, 0, 1, 0, 1, None, None, None) == 1
    assert engine_lib.pa_resample_plan(None, None, 0, 10, 10, 10, 0, 0.1, 0, 0, 1, 0, None, None, None, None, None) == 1
    assert engine_lib.pa_sweep_form(None, 0, None) == 1
    assert engine_lib.pa_autotune(None, None, 0) == 1


def test_cli_argument_errors():
    """The command-line driver rejects unknown options (usage, exit 1) and
    non-option arguments (exit 1) like PAisingSSC.cu:399-404."""
    import subprocess
    exe = os.path.join(ROOT, "paising_gb300", "_lib", "paising")
    if not os.path.exists(exe):
        pytest.skip("CLI not built")
    r = subprocess.run([exe, "-x"], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage" in r.stdout
    r = subprocess.run([exe, "extra"], capture_output=True, text=True)
    assert r.returncode == 1 and "Non-option argument extra" in r.stderr
    r = subprocess.run([exe, "-c", "ssc", "-L", "12", "-o", "/tmp/pa_cli_bad_L"], capture_output=True, text=True)
    assert r.returncode == 1 and "L % 8" in r.stderr
