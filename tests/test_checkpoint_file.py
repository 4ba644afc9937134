"""Checkpoint files are checked on the host before anything reaches a device
(pa_checkpoint_verify; pa_restore makes the same checks first).  The files
here are written by hand in the documented format: a consistent one passes,
and each field that would index outside the handle's buffers -- a population
size beyond the capacity, a buffer parity other than 0 or 1, a temperature
index beyond the schedule, a buffer of the wrong size -- is refused with
PA_ERR_ARG and a message naming it.  No GPU is needed."""
import struct

import pytest

import paising_gb300 as pa

MSB = 32


def ckpt_bytes(coding=1, L=8, R=40, cap=6, R_cur=40, R_prev=40, parity=0, step=3, nsteps=5, rec=0, family=0,
               buffer_R=None, trailing=b"", truncate=0):
    """A checkpoint of one population (version 2): header, shape, scalars and
    the stateful buffers (zeros) sized for buffer_R replicas (default R_cur)."""
    Rcap = int(1.25 * R) + 256
    rgcap = (Rcap + MSB - 1) // MSB
    N = L * L
    head = b"PAGB300C" + struct.pack("<5i", 2, 1, coding, step - 1, 0)
    shape = struct.pack("<9i", L, R, Rcap, rgcap, cap, 1, coding, rec, family)
    sc = struct.pack("<12i3Q4q5d", nsteps, step, R_prev, R_cur, parity, 0, -2 * N, 0, 0, -1, -1, 0,
                     12345, 0, 0, 0, 0, 0, 0, 0.0, 0.0, 0.0, 0.0, 0.05)
    assert len(shape) == 36 and len(sc) == 144
    nR = R_cur if buffer_R is None else buffer_R
    units = rgcap * MSB if coding == 1 else Rcap
    sizes = [((nR + MSB - 1) // MSB) * N * 4 if coding == 1 else nR * N]
    if coding == 1:
        sizes.append(units)
    sizes += [4 * units, 4 * units, cap * 10 * 8, cap * 8, cap * 12 * 4]
    if rec & 1:
        sizes.append((N + 1) * 8)
    if family:
        sizes += [4 * units, cap * 3 * 8]
    body = b"".join(struct.pack("<Q", n) + bytes(n) for n in sizes)
    out = head + shape + sc + body + trailing
    return out[: len(out) - truncate] if truncate else out


def verify(tmp_path, data: bytes):
    p = tmp_path / "c.bin"
    p.write_bytes(data)
    st = pa.lib().pa_checkpoint_verify(str(p).encode())
    return st, (pa.lib().pa_last_error(None) or b"").decode()


@pytest.mark.parametrize("coding", [0, 1])
@pytest.mark.parametrize("rec,family", [(0, 0), (1, 1)])
def test_consistent_file_passes(tmp_path, coding, rec, family):
    st, msg = verify(tmp_path, ckpt_bytes(coding=coding, rec=rec, family=family))
    assert st == 0, msg


@pytest.mark.parametrize("coding", [0, 1])
@pytest.mark.parametrize("field,kw,words", [
    ("R_cur", dict(R_cur=10 ** 6, buffer_R=40), "capacity"),
    ("R_cur", dict(R_cur=-1, buffer_R=40), "capacity"),
    ("R_prev", dict(R_prev=10 ** 6), "capacity"),
    ("parity", dict(parity=2), "parity"),
    ("parity", dict(parity=-1), "parity"),
    ("step", dict(step=7, nsteps=5), "schedule"),
    ("nsteps", dict(nsteps=6, cap=6), "schedule"),
    ("buffer", dict(R_cur=40, buffer_R=80), "buffer size"),
    ("truncated", dict(truncate=3), "truncated"),
    ("trailing", dict(trailing=b"x"), "trailing"),
])
def test_inconsistent_file_is_refused(tmp_path, coding, field, kw, words):
    st, msg = verify(tmp_path, ckpt_bytes(coding=coding, **kw))
    assert st == 1, (field, msg)
    assert words in msg, (field, msg)


def test_huge_claimed_shape_is_refused_without_allocating(tmp_path):
    """A shape claiming a population far larger than the file (here ~2^31
    replicas at L=4096, terabytes of buffers) is refused as truncated before
    any buffer is allocated."""
    big = ckpt_bytes(coding=0, L=8)
    head, rest = big[:28], big[28:]
    shape = struct.pack("<9i", 4096, 2 ** 30, 2 ** 31 - 1, (2 ** 31 - 1 + 31) // 32, 6, 1, 0, 0, 0)
    st, msg = verify(tmp_path, head + shape + rest[36:])
    assert st == 1 and ("truncated" in msg or "size" in msg), msg


def test_not_a_checkpoint(tmp_path):
    st, msg = verify(tmp_path, b"PAGB300X" + bytes(64))
    assert st == 1 and "not a checkpoint" in msg
    st, msg = verify(tmp_path, ckpt_bytes()[:8] + struct.pack("<5i", 1, 1, 1, 0, 0))
    assert st == 1 and "version" in msg
