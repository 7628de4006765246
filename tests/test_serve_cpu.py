"""Host logic of the relight server that needs no GPU: the dirty-probe list a request runs
(lumrad_dirty_probes, both its enumeration and its dilation path) against a numpy restatement."""
import numpy as np
import pytest

from lum_gb300 import worldgen


def _lib_dirty(dims, edits, radius):
    import lum_gb300
    return lum_gb300.dirty_probes(dims, edits, radius)


@pytest.mark.parametrize("dims,frac,radius", [
    ((8, 8, 8), 0.002, 2),        # a single edit: enumeration path
    ((16, 12, 9), 0.01, 2),       # enumeration
    ((16, 12, 9), 0.05, 2),       # dilation path (many edits)
    ((33, 17, 5), 0.03, 1),
    ((20, 20, 20), 0.001, 0),     # radius 0: exactly the edited blocks
    ((7, 5, 3), 0.5, 3),          # radius past the world's size on z
    ((64, 64, 32), 0.05, 2),      # the largest serving world
])
def test_dirty_probes_match_numpy(dims, frac, radius):
    edits = worldgen.edit_request(dims, frac, seed=3, stream=int(100 * frac) + radius)
    got = _lib_dirty(dims, edits, radius)
    ref = worldgen.dirty_probes(dims, edits, radius)
    assert got.dtype == np.int16 and got.shape == ref.shape
    assert np.array_equal(got, ref)


def test_dirty_probes_edges():
    import lum_gb300
    assert _lib_dirty((4, 4, 4), np.zeros((0, 4), np.int16), 2).shape == (0, 4)
    corner = np.array([[3, 3, 3, 1]], dtype=np.int16)
    got = _lib_dirty((4, 4, 4), corner, 2)
    assert got.shape == (27, 4) and got[:, :3].min() == 1 and got[:, :3].max() == 3
    with pytest.raises(lum_gb300.LumRadError):
        _lib_dirty((4, 4, 4), np.array([[4, 0, 0, 1]], dtype=np.int16), 2)
    with pytest.raises(lum_gb300.LumRadError):
        _lib_dirty((4, 4, 4), np.array([[-1, 0, 0, 1]], dtype=np.int16), 2)
    with pytest.raises(lum_gb300.LumRadError):
        _lib_dirty((4, 4, 4), corner, 16)


def test_edit_request_is_seeded():
    a = worldgen.edit_request((32, 32, 16), 0.03, seed=5, stream=7)
    b = worldgen.edit_request((32, 32, 16), 0.03, seed=5, stream=7)
    c = worldgen.edit_request((32, 32, 16), 0.03, seed=5, stream=8)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.shape == (round(0.03 * 32 * 32 * 16), 4)
    assert a[:, 3].min() >= 0 and a[:, 3].max() <= 32
