"""``.dtmf`` / ``.dtms`` files: reading files the reference wrote
(``tests/golden/io_*``, from ``make_golden.py``) and writing byte-identical
files from the same arrays; version-1 stacks and bad magic numbers."""
import io
import os

import numpy as np
import pytest

from dtmm_gb300 import io as dio

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def _expected():
    rng = np.random.Generator(np.random.PCG64(5))
    field = (rng.normal(size=(2, 3, 4, 6, 5)) + 1j * rng.normal(size=(2, 3, 4, 6, 5))).astype(np.complex128)
    d = np.asarray([1.0, 2.0, 0.5])
    epsa = rng.uniform(-1, 1, size=(3, 6, 5, 3))
    return field, d, epsa


def test_field_file_round_trip_matches_reference_bytes(tmp_path):
    field, _, _ = _expected()
    f, wl, ps = dio.load_field(os.path.join(GOLD, "io_field.dtmf"))
    assert np.array_equal(f, field) and np.array_equal(wl, [450.0, 550.0, 650.0]) and ps == 80.0
    out = str(tmp_path / "again")
    dio.save_field(out, (f, wl, ps))
    assert open(out + ".dtmf", "rb").read() == open(os.path.join(GOLD, "io_field.dtmf"), "rb").read()


def test_stack_file_round_trip_matches_reference_bytes(tmp_path):
    _, d, epsa = _expected()
    blocks = dio.load_stack(os.path.join(GOLD, "io_stack.dtms"))
    assert len(blocks) == 2
    assert np.array_equal(blocks[0][0], d) and np.array_equal(blocks[0][2], epsa)
    assert blocks[0][1].shape == (3, 6, 5, 3) and np.all(blocks[0][1][..., 2] == 2.89)
    assert blocks[1][1].dtype == np.complex128
    out = str(tmp_path / "again")
    dio.save_stack(out, blocks)
    assert open(out + ".dtms", "rb").read() == open(os.path.join(GOLD, "io_stack.dtms"), "rb").read()


def test_version_1_stack_and_bad_magic():
    buf = io.BytesIO()
    buf.write(b"dtms\x01")
    np.save(buf, np.ones(2))
    np.save(buf, np.full((2, 1, 1, 3), 2.0))
    buf.seek(0)
    d, epsv, epsa = dio.load_stack(buf)
    assert epsa is None and epsv.shape == (2, 1, 1, 3)
    with pytest.raises(OSError):
        dio.load_field(io.BytesIO(b"nope\x00"))
    with pytest.raises(OSError):
        dio.load_stack(io.BytesIO(b"dtms\x07"))
