"""GPU parity of the grid-KDE conformer binning (a KDE variant for every DOF
type with no reference counterpart) against its CPU restatement in
oracle/gridkde.py.  Bins, minima and bin counts must be identical; DOFs whose
neighbouring grid densities agree to 1e-9 (rounding could reorder them) are
excluded and must be rare."""
import numpy as np
import pytest

from centre_gb300.api import CentreError
from centre_gb300.synth import chain_trajectory
from oracle import gridkde as GK

pytestmark = pytest.mark.gpu


def _check_block(gpu, typ, blk, ngrid, kappa=50.0):
    bins, mins, nmin, nbins = gpu.discretize_gridkde(typ, blk, ngrid, kappa)
    ob, om, od, onb = GK.gridkde(typ, blk, ngrid, kappa)
    skipped = 0
    for k in range(blk.shape[0]):
        if GK.near_tie(typ, od[k]):
            skipped += 1
            continue
        assert int(nmin[k]) == om[k].size, (typ, k)
        np.testing.assert_array_equal(mins[k, :nmin[k]], om[k])
        assert np.all(mins[k, nmin[k]:] == 0.0)
        assert int(nbins[k]) == int(onb[k])
        np.testing.assert_array_equal(bins[k, 0], ob[k])
        assert int(bins[k, 0].max()) < int(nbins[k])
    assert skipped <= max(1, blk.shape[0] // 10), skipped
    return bins, nmin, nbins


@pytest.mark.parametrize("nframes", [20_000, 4_099])
def test_gridkde_chain_vs_oracle(gpu, nframes):
    tr = chain_trajectory(12, nframes, seed=3, coupling="block8")
    seen = {}
    for typ, blk in tr.blocks():
        ngrid = 72 if typ == 3 else 50
        _, nmin, nbins = _check_block(gpu, typ, blk, ngrid)
        seen[typ] = int(nbins.max())
    # the torsions' three modes show up as several conformers
    assert seen[3] >= 2


@pytest.mark.parametrize("ngrid", [3, 37, 128])
def test_gridkde_grid_sizes(gpu, ngrid):
    tr = chain_trajectory(8, 6_000, seed=5, coupling="block8")
    for typ, blk in tr.blocks():
        _check_block(gpu, typ, blk, ngrid, kappa=20.0)


def test_gridkde_wraps_through_zero(gpu):
    # two modes, one straddling 0 / 2 pi: its frames on both sides share the
    # wrap-around conformer M - 1
    rng = np.random.default_rng(7)
    a = np.concatenate([rng.vonmises(0.0, 40.0, 5000), rng.vonmises(np.pi, 40.0, 5000)])
    a = np.mod(a, 2 * np.pi).astype(np.float32)[None, :]
    a = np.minimum(a, np.float32(6.2831850))
    bins, mins, nmin, nbins = gpu.discretize_gridkde(3, a, 72, 50.0)
    ob, om, od, onb = GK.gridkde(3, a, 72, 50.0)
    np.testing.assert_array_equal(bins[:, 0], ob)
    m = int(nmin[0])
    assert m == 2 and nbins[0] == 2
    near0 = (a[0] < 0.3) | (a[0] > 2 * np.pi - 0.3)
    assert np.all(bins[0, 0][near0] == m - 1)
    assert np.all(bins[0, 0][np.abs(a[0] - np.pi) < 0.3] == 0)


def test_gridkde_flat_and_errors(gpu):
    flat = np.full((2, 1000), 1.5, np.float32)
    bins, mins, nmin, nbins = gpu.discretize_gridkde(1, flat, 50)
    assert np.all(bins == 0) and np.all(nmin == 0) and np.all(nbins == 1)
    bad = np.ones((1, 100), np.float32)
    bad[0, 17] = np.nan
    with pytest.raises(CentreError):
        gpu.discretize_gridkde(2, bad, 50)
    with pytest.raises(CentreError):
        gpu.discretize_gridkde(1, flat, 2)
    with pytest.raises(CentreError):
        gpu.discretize_gridkde(1, flat, 129)
    with pytest.raises(CentreError):
        gpu.discretize_gridkde(3, flat, 72, kappa=0.0)
    b, m, nm, nb = gpu.discretize_gridkde(3, np.zeros((0, 10), np.float32), 72)
    assert b.size == 0


def test_gridkde_dev_matches_host(gpu):
    torch = pytest.importorskip("torch")
    tr = chain_trajectory(10, 3_000, seed=9)
    for typ, blk in tr.blocks():
        hb, hm, hn, hnb = gpu.discretize_gridkde(typ, blk, 64, 30.0)
        d = torch.from_numpy(np.ascontiguousarray(blk)).cuda()
        nd, n = blk.shape
        b = torch.empty((nd, n), dtype=torch.uint8, device="cuda")
        m = torch.empty((nd, 64), dtype=torch.float64, device="cuda")
        nm = torch.empty(nd, dtype=torch.uint8, device="cuda")
        nb = torch.empty(nd, dtype=torch.uint8, device="cuda")
        gpu.discretize_gridkde_dev(typ, d, 64, 30.0, b, m, nm, nb)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(b.cpu().numpy(), hb[:, 0])
        np.testing.assert_array_equal(m.cpu().numpy(), hm)
        np.testing.assert_array_equal(nm.cpu().numpy(), hn)
        np.testing.assert_array_equal(nb.cpu().numpy(), hnb)


def test_df_exp_error_bound(gpu):
    """The double-float e^y of the torsion sums (Tang's table-driven method on
    FP32 pairs) against FP64 on [-70, 0] (where the low word is a normal
    float): relative error below 5e-14 plus |y| * 4e-15 (y itself carries
    ~48 bits as a double-float); FP32-level down to -87, exact 0 below."""
    rng = np.random.default_rng(11)
    y = np.concatenate([-70.0 * rng.random(200_000), -rng.random(50_000) * 1e-3,
                        np.array([0.0, -1e-30, -0.5, -np.log(2) / 128]),
                        -np.arange(0, 70, 0.25)])
    got = gpu.df_exp_eval(y)
    want = np.exp(y)
    rel = np.abs(got - want) / want
    bound = 5e-14 + 4e-15 * np.abs(y)
    assert np.all(rel < bound), (rel.max(), y[np.argmax(rel / bound)])
    # near the end of the FP32 range the low word turns subnormal: FP32-level
    # accuracy there (such terms are summed again in FP64 when they dominate)
    y2 = -70.0 - 17.0 * rng.random(10_000)
    assert np.max(np.abs(gpu.df_exp_eval(y2) - np.exp(y2)) / np.exp(y2)) < 1e-6
    assert np.all(gpu.df_exp_eval(np.array([-87.5, -100.0, -1e3])) == 0.0)
