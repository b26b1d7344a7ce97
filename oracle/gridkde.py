"""CPU oracle of the grid-KDE conformer binning -- TEST INFRASTRUCTURE ONLY.

Parity unpinned: the reference (shaileshp51/centre) has no such mode.  Its
only KDE is the torsion von Mises KDE of Real2Int::getMinimaPositions
(src/Real2Int.cpp:481-657: a 361-point grid, a bandwidth derived from kappa,
minima refined by steepest descent).  This module restates, in FP64 numpy, the
grid-KDE variant the library implements for every DOF type, from the same
definitions, so that the GPU kernels have a checker; nothing here comes from
the reference's code.

* torsions: d_j = sum_i exp(kappa (cos g_j cos a_i + sin g_j sin a_i - 1)),
  g_j = 2 pi j / G;
* bonds/angles: d_j = sum_i exp(-((g_j - x_i) / h)^2 / 2), h = 1.06 sigma
  N^(-1/5) (population sigma), g_j = lo + (j + 1/2)(hi - lo) / G;
* minima: d_j < d_{j-1} and d_j <= d_{j+1} (cyclic for torsions, j = 1..G-2
  otherwise); bins: linear #{m <= x}, torsions (#{m <= a} + M - 1) mod M.

Only ``tests/`` import it.
"""
from __future__ import annotations

import numpy as np

TWO_PI = 6.283185307179586


def densities(bat_type: int, x, ngrid: int, kappa: float = 50.0, chunk: int = 4096):
    """Grid densities of one DOF (float32 frames) -> (d [G], grid [G], flat)."""
    x = np.asarray(x, np.float32).astype(np.float64)
    n = x.size
    j = np.arange(ngrid, dtype=np.float64)
    d = np.zeros(ngrid)
    if bat_type == 3:
        g = TWO_PI * j / ngrid
        cg, sg = np.cos(g), np.sin(g)
        for s in range(0, n, chunk):
            a = x[s:s + chunk]
            ca, sa = np.cos(a), np.sin(a)
            d += np.exp(kappa * (np.outer(ca, cg) + np.outer(sa, sg) - 1.0)).sum(axis=0)
        return d, g, False
    lo, hi = float(x.min()), float(x.max())
    mean = x.sum() / n
    sigma = np.sqrt(((x - mean) ** 2).sum() / n)
    h = 1.06 * sigma * n ** -0.2
    step = (hi - lo) / ngrid
    g = lo + (j + 0.5) * step
    if not (step > 0.0 and h > 0.0):
        return d, g, True
    for s in range(0, n, chunk):
        z = (g[None, :] - x[s:s + chunk, None]) / h
        d += np.exp(-0.5 * z * z).sum(axis=0)
    return d, g, False


def minima(bat_type: int, d, g, flat: bool):
    """Grid minima positions (sorted) of one DOF's densities."""
    if flat:
        return np.zeros(0)
    G = d.size
    if bat_type == 3:
        idx = [k for k in range(G) if d[k] < d[(k - 1) % G] and d[k] <= d[(k + 1) % G]]
    else:
        idx = [k for k in range(1, G - 1) if d[k] < d[k - 1] and d[k] <= d[k + 1]]
    return g[idx]


def bins(bat_type: int, x, m):
    """Conformer index of every frame for minima m (sorted)."""
    x = np.asarray(x, np.float32).astype(np.float64)
    c = np.searchsorted(m, x, side="right")       # #{m <= x}
    if bat_type == 3:
        M = m.size
        return ((c + M - 1) % M).astype(np.uint8) if M else np.zeros(x.size, np.uint8)
    return c.astype(np.uint8)


def gridkde(bat_type: int, data, ngrid: int, kappa: float = 50.0):
    """All DOFs of a block [ndof][nframes] -> (bins [ndof][nframes], list of
    minima arrays, densities [ndof][G], nbins [ndof])."""
    data = np.asarray(data, np.float32)
    out = np.empty(data.shape, np.uint8)
    mins, dens, nb = [], [], []
    for k in range(data.shape[0]):
        d, g, flat = densities(bat_type, data[k], ngrid, kappa)
        m = minima(bat_type, d, g, flat)
        out[k] = bins(bat_type, data[k], m)
        mins.append(m)
        dens.append(d)
        nb.append(max(m.size, 1) if bat_type == 3 else m.size + 1)
    return out, mins, np.array(dens), np.array(nb, np.uint8)


def near_tie(bat_type: int, d, rel: float = 1e-9) -> bool:
    """True when two neighbouring grid densities agree to `rel`: their order
    (and so the minima) may depend on rounding."""
    G = d.size
    r = range(G) if bat_type == 3 else range(G - 1)
    for k in r:
        a, b = d[k], d[(k + 1) % G]
        if abs(a - b) <= rel * max(abs(a), abs(b)):
            return True
    return False
