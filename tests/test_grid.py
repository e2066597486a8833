"""The Grid container (FiniteDifference/Grid.py's interface): initial grids
on 1-D and 2-D meshes, scalar initializers, spacing, monotonic meshes,
copy and reset."""
import numpy as np
import pytest

from fd_adi_gb300 import Grid


def test_initial_grids_and_spacing():
    S = np.array([0.0, 50.0, 100.0, 200.0])
    v = np.array([0.0, 0.5, 1.0])
    g = Grid([S, v], initializer=lambda s, var: np.maximum(s - 100.0, 0.0) + var)
    assert g.shape == (4, 3) and g.ndim == 2 and g.size == 12
    np.testing.assert_array_equal(g.domain[-1], np.maximum(S - 100.0, 0.0)[:, None] + v[None, :])
    np.testing.assert_array_equal(g.dx[0], [np.nan, 50.0, 50.0, 100.0])
    g1 = Grid([S], initializer=lambda s: s * 2)
    assert g1.shape == (4,)
    np.testing.assert_array_equal(g1.domain[-1], 2 * S)
    gs = Grid([S, v], initializer=lambda s, var: 1.5)
    np.testing.assert_array_equal(gs.domain[-1], np.full((4, 3), 1.5))
    assert gs.domain[-1].dtype == np.float64


def test_meshes_must_be_monotonic():
    with pytest.raises(AssertionError):
        Grid([np.array([0.0, 2.0, 1.0])], initializer=lambda s: s)
    Grid([np.array([3.0, 2.0, 1.0])], initializer=lambda s: s)   # decreasing is monotonic


def test_copy_and_reset():
    S = np.linspace(0.0, 1.0, 5)
    g = Grid([S], initializer=lambda s: s)
    g.domain.append(g.domain[-1] + 1.0)
    c = g.copy()
    assert len(c.domain) == 2
    c.domain[-1][0] = 99.0
    assert g.domain[-1][0] == 1.0          # the copy owns its grids
    g.reset()
    assert len(g.domain) == 1
    np.testing.assert_array_equal(g.domain[-1], S)
