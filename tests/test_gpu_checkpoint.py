"""Host-stepped runs and checkpoints (no counterpart in the reference): a run
advanced temperature by temperature, saved to a file part-way, and continued
in a fresh handle must give exactly the rows of the uninterrupted run."""
import numpy as np
import pytest

import paising_gb300 as pa
from conftest import compare_rows, load_dat

pytestmark = pytest.mark.gpu


def stepped(kw, cut, path):
    """Rows of a run stepped to temperature `cut`, checkpointed, and finished
    in a second handle; plus that handle (still open) for more results."""
    with pa.Engine(**kw) as a:
        a.run_begin()
        assert not a.run_steps(cut)
        a.checkpoint(str(path))
    b = pa.Engine(**kw)
    b.restore(str(path))
    while not b.run_steps(7):
        pass
    b.run_end()
    return b


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_checkpoint_reference_stream(cuda, tmp_path, coding):
    kw = dict(L=16, R=1000, sweeps=10, seed=100, coding=coding, rng="reference", weights="fp64")
    b = stepped(kw, 83, tmp_path / "c.bin")
    compare_rows(b.rows(0), load_dat(f"ref/inj_{coding.upper()}_L16_R1000_t10_d0.005_s100.dat"), rtol=2e-10)
    b.close()


def test_checkpoint_native_batch_with_statistics(cuda, tmp_path):
    """Native stream, an uneven batch with MHR, family statistics and one
    adaptive population: stepped + checkpointed rows equal pa_run's."""
    pops = [dict(L=16, R=2000, sweeps=5, dbeta=0.02, seed=1, mhr=True, family=True),
            dict(L=32, R=1500, sweeps=4, dbeta=0.01, seed=2, adaptive=True, family=True),
            dict(L=64, R=700, sweeps=3, dbeta=0.05, seed=3)]
    with pa.Engine.batch(pops, coding="msc") as e:
        e.run()
        ref = [e.rows(k) for k in range(3)]
        ref_f = [e.family_rows(k) for k in range(2)]
        ref_m = e.mhr_rows(0)
    path = str(tmp_path / "b.bin")
    with pa.Engine.batch(pops, coding="msc") as a:
        a.run_begin()
        a.run_steps(11)
        a.checkpoint(path)
    with pa.Engine.batch(pops, coding="msc") as b:
        b.restore(path)
        while not b.run_steps(5):
            pass
        b.run_end()
        for k in range(3):
            assert np.array_equal(b.rows(k), ref[k])
        for k in range(2):
            assert np.array_equal(b.family_rows(k), ref_f[k])
        assert np.array_equal(b.mhr_rows(0), ref_m)


def test_checkpoint_rejects_other_configuration(cuda, tmp_path):
    path = str(tmp_path / "c.bin")
    with pa.Engine(L=16, R=500, sweeps=3, dbeta=0.1, coding="msc") as a:
        a.run_begin()
        a.run_steps(2)
        a.checkpoint(path)
    with pa.Engine(L=16, R=600, sweeps=3, dbeta=0.1, coding="msc") as b:
        with pytest.raises(pa.PaisingError):
            b.restore(path)
    with pa.Engine(L=16, R=500, sweeps=3, dbeta=0.1, coding="msc") as c:
        with pytest.raises(pa.PaisingError) as ei:
            c.checkpoint(path)  # no stepped run in progress
        assert ei.value.status == 5


@pytest.mark.parametrize("coding", ["ssc", "msc"])
def test_restore_refuses_tampered_files_and_keeps_the_handle(cuda, tmp_path, coding):
    """A checkpoint whose population size or buffer parity was altered is
    refused before any device write (PA_ERR_ARG); the same handle then
    restores the intact file and finishes with the uninterrupted run's rows."""
    kw = dict(L=16, R=500, sweeps=3, dbeta=0.1, seed=5, coding=coding)
    with pa.Engine(**kw) as e:
        e.run()
        ref = e.rows(0)
    good = tmp_path / "good.bin"
    with pa.Engine(**kw) as a:
        a.run_begin()
        a.run_steps(4)
        a.checkpoint(str(good))
    data = good.read_bytes()
    # header 8 + 5 int32, shape 9 int32, then the scalars: nsteps, step, R_prev, R_cur, parity, ...
    off = 8 + 20 + 36
    import struct
    with pa.Engine(**kw) as b:
        for name, pos, val in (("R_cur", off + 12, 10 ** 7), ("parity", off + 16, 2), ("step", off + 4, 999)):
            bad = bytearray(data)
            bad[pos:pos + 4] = struct.pack("<i", val)
            p = tmp_path / f"bad_{name}.bin"
            p.write_bytes(bytes(bad))
            with pytest.raises(pa.PaisingError) as ei:
                b.restore(str(p))
            assert ei.value.status == 1, name
            with pytest.raises(pa.PaisingError):
                pa.Engine.verify_checkpoint(str(p))
        pa.Engine.verify_checkpoint(str(good))
        b.restore(str(good))
        while not b.run_steps(3):
            pass
        b.run_end()
        assert np.array_equal(b.rows(0), ref)


def test_checkpoint_of_a_cluster_swept_population(cuda, tmp_path):
    """A small L=64 population, swept by clusters of CTAs by default, stepped,
    checkpointed and finished in a second handle gives pa_run's rows."""
    kw = dict(L=64, R=3000, sweeps=4, dbeta=0.05, seed=17, coding="msc")
    with pa.Engine(**kw) as e:
        assert e.sweep_form(0)["cluster_ctas"] > 1
        e.run()
        ref = e.rows(0)
    b = stepped(kw, 7, tmp_path / "c.bin")
    assert np.array_equal(b.rows(0), ref)
    b.close()
