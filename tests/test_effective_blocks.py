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
        out, sym, given = effective_blocks(bl, e)
        assert out is bl and sym is None and given is None


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
    out, sym, given = effective_blocks(bl, [[1, 0, 2], 1])
    assert sym == [1, 0, 2, 1]
    assert [len(b[0]) for b in out] == [1, 1, 1, 2]
    np.testing.assert_array_equal(out[1][2], bl[0][2][1:2])
    out, sym, _ = effective_blocks(bl, [[0, 0, 0], 0])  # per-layer isotropic means
    assert sym == [0, 0, 0, 0] and len(out) == 4
    with pytest.raises(ValueError, match="incompatible with block size"):
        effective_blocks(bl, [[1, 0], 1])


def test_given_effective_blocks():
    """An effective block given as (thickness, epsv, epsa): one engine block
    per layer with its medium (symmetry 3), the other blocks as they are."""
    bl = _blocks()
    ev = np.array([[2.3, 2.3, 2.7], [2.4, 2.4, 2.4], [2.2, 2.3 + 0.01j, 2.6]])
    ea = np.array([[0.0, 0.5, 0.1], [0.0, 0.0, 0.0], [0.2, 0.3, 0.4]])
    out, sym, given = effective_blocks(bl, [(np.ones(3), ev, ea), "uniaxial"])
    assert sym == [3, 3, 3, 1] and len(out) == 4 and given.shape == (4, 9)
    np.testing.assert_array_equal(given[2], [2.2, 0.0, 2.3, 0.01, 2.6, 0.0, 0.2, 0.3, 0.4])
    np.testing.assert_array_equal(given[3], np.zeros(9))
    # the given layers' thicknesses must be the optical block's
    with pytest.raises(NotImplementedError):
        effective_blocks(bl[:1], [(2 * np.ones(3), ev, ea)])
    # a per-layer symmetry list is no optical block
    assert effective_blocks(bl[:1], [[1, 2, 0]])[1] == [1, 2, 0]
