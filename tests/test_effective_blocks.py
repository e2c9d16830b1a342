"""eff_data at the boundary: the engine's blocks and their effective-medium
symmetries, as the reference resolves them (dtmm/transfer.py:978-1005,
dtmm/data.py:1344-1419)."""
import numpy as np
import pytest

from dtmm_gb300 import samples
from dtmm_gb300.transfer import effective_blocks


def _blocks():
    a = samples.twisted_nematic((6, 6), 3, seed=1)
    b = samples.twisted_nematic((6, 6), 2, seed=2)
    return [a, b]


def test_isotropic_keeps_the_blocks():
    bl = _blocks()
    for e in (0, "isotropic", [0, "isotropic"]):
        out, sym = effective_blocks(bl, e)
        assert out is bl and sym is None


def test_one_symmetry_for_every_block_or_one_per_block():
    bl = _blocks()
    assert effective_blocks(bl, 1)[1] == [1, 1]
    assert effective_blocks(bl, "biaxial")[1] == [2, 2]
    assert effective_blocks(bl, [1, "isotropic"])[1] == [1, 0]
    assert effective_blocks(bl, [-1, 0])[1] == [2, 0]  # -1 keeps the eigenvalues: biaxial
    with pytest.raises(ValueError, match="Number of elements"):
        effective_blocks(bl, [1, 2, 0])
    with pytest.raises(ValueError, match="Invalid symmetry"):
        effective_blocks(bl, "nematic")
    with pytest.raises(ValueError, match="Invalid symmetry"):
        effective_blocks(bl, [3, 0])


def test_per_layer_symmetry_splits_its_block():
    bl = _blocks()
    out, sym = effective_blocks(bl, [[1, 0, 2], 1])
    assert sym == [1, 0, 2, 1]
    assert [len(b[0]) for b in out] == [1, 1, 1, 2]
    np.testing.assert_array_equal(out[1][2], bl[0][2][1:2])
    out, sym = effective_blocks(bl, [[0, 0, 0], 0])  # per-layer isotropic means
    assert sym == [0, 0, 0, 0] and len(out) == 4
    with pytest.raises(ValueError, match="incompatible with block size"):
        effective_blocks(bl, [[1, 0], 1])


def test_explicit_effective_blocks_are_outside_the_engine():
    bl = _blocks()
    eff = (np.ones(3), np.ones((3, 1, 1, 3)) * 2.3, np.zeros((3, 1, 1, 3)))
    with pytest.raises(NotImplementedError):
        effective_blocks(bl[:1], [eff])
