"""CPU checks of the grid-KDE oracle's definitions (minima rule, interval
labels, wrap-around conformer, flat DOFs)."""
import numpy as np

from oracle import gridkde as GK


def test_linear_minima_and_labels():
    d = np.array([5.0, 3.0, 1.0, 2.0, 2.0, 0.5, 0.5, 4.0])
    g = np.arange(8, dtype=np.float64)
    m = GK.minima(1, d, g, False)
    # strict drop on the left, non-strict rise on the right: 2 and 5 (the
    # first of the flat bottom 5, 6), not 6
    np.testing.assert_array_equal(m, [2.0, 5.0])
    x = np.array([0.0, 1.99, 2.0, 4.9, 5.0, 7.0], np.float32)
    np.testing.assert_array_equal(GK.bins(1, x, m), [0, 0, 1, 1, 2, 2])


def test_circular_minima_wrap():
    G = 12
    g = 2 * np.pi * np.arange(G) / G
    d = 2.0 + np.cos(2 * g)          # minima at pi/2 and 3pi/2
    m = GK.minima(3, d, g, False)
    np.testing.assert_allclose(m, [np.pi / 2, 3 * np.pi / 2])
    a = np.array([0.1, 1.6, 3.0, 4.8, 6.2], np.float32)
    # [m0, m1) -> 0, [m1, 2pi) and [0, m0) -> M - 1 = 1
    np.testing.assert_array_equal(GK.bins(3, a, m), [1, 0, 0, 1, 1])


def test_constant_density_and_flat_dof():
    d = np.ones(10)
    assert GK.minima(3, d, np.arange(10.0), False).size == 0
    assert np.all(GK.bins(3, np.ones(5, np.float32), np.zeros(0)) == 0)
    b, mins, dens, nb = GK.gridkde(2, np.full((1, 50), 1.9, np.float32), 20)
    assert np.all(b == 0) and mins[0].size == 0 and nb[0] == 1


def test_two_gaussian_modes_found():
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.normal(1.0, 0.05, 3000), rng.normal(2.0, 0.05, 3000)])
    b, mins, dens, nb = GK.gridkde(1, x[None, :].astype(np.float32), 50)
    assert mins[0].size >= 1 and 1.2 < mins[0][0] < 1.8
    assert set(np.unique(b[0][x < 1.2])) == {0}
    assert not GK.near_tie(1, dens[0][:-1][dens[0][:-1] > 0])
