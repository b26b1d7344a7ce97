"""Batched scoring of several trajectories of uneven length (one captured
graph, one persistent count kernel) against the oracle directly and against
the single-trajectory entries.  1-D entropies agree exactly; joint entropies
within 1e-12 relative of the single-trajectory path (the batch rounds its
fixed-point c ln c terms at the scale of its longest trajectory) and within
the parity tolerance of the oracle; MIE / MIST sums within 1e-9 relative
(their summation order differs between the paths)."""
import numpy as np
import pytest

from centre_gb300.api import make_params
from centre_gb300.synth import chain_trajectory

pytestmark = pytest.mark.gpu


def _stack(tr, gpu, schemes):
    bins, ext, types = [], [], []
    for typ, blk in tr.blocks():
        b, e = gpu.discretize(typ, blk, schemes, bins_ref=schemes[0], optimize=True)
        bins.append(b)
        ext.append(e)
        types += [typ] * len(b)
    return np.concatenate(bins), np.concatenate(ext), np.array(types, np.uint8)


def _systems(torch, gpu, specs, schemes, nsteps, nest):
    dev = torch.device("cuda", 0)
    host, dsys = [], []
    G = nest * len(schemes) * nsteps
    for natoms, nframes, seed in specs:
        tr = chain_trajectory(natoms, nframes, seed=seed)
        bins, ext, types = _stack(tr, gpu, schemes)
        ndof = len(types)
        host.append((bins, ext, types))
        dsys.append({
            "types": torch.from_numpy(types).to(dev),
            "bins": torch.from_numpy(bins).to(dev),
            "ext": torch.from_numpy(ext).to(dev),
            "s1": torch.zeros((ndof, G), dtype=torch.float64, device=dev),
            "s2": torch.zeros((ndof * (ndof - 1) // 2, G), dtype=torch.float64, device=dev),
            "mi": torch.zeros((ndof * (ndof - 1) // 2, G), dtype=torch.float64, device=dev),
        })
    return host, dsys


def _check_oracle(orc, p, bins, ext, types, d, r):
    """The batch's S1, S2 and MIST totals against the oracle (the C
    restatement of binData1D/2D, entropy1D/2D and boruvkaMST)."""
    sch = list(p.bin_schemes[: p.nschemes])
    ests = list(p.estimators[: p.nestimators])
    ndof = len(types)
    iu = np.triu_indices(ndof, 1)
    pairs = np.stack(iu, 1).astype(np.uint32)
    o1 = orc.entropy1d(types, bins, ext, p.nsteps, sch, ests, bool(p.jacobian))
    o2 = orc.entropy2d(pairs, types, bins, ext, p.nsteps, sch, ests, bool(p.jacobian))
    g1 = d["s1"].cpu().numpy().reshape(o1.shape)
    g2 = d["s2"].cpu().numpy().reshape(o2.shape)
    np.testing.assert_allclose(g1, o1, rtol=1e-9, atol=1e-13)
    np.testing.assert_allclose(g2, o2, rtol=1e-9, atol=1e-13)
    s1f, s2f = o1.reshape(ndof, -1), o2.reshape(len(pairs), -1)
    for g in range(s1f.shape[1]):
        mi = s1f[iu[0], g] + s1f[iu[1], g] - s2f[:, g]
        tree = orc.mst(ndof, pairs[:, 0], pairs[:, 1], mi)
        want = s1f[:, g].sum() - mi[tree].sum()
        np.testing.assert_allclose(r["mist"][g, 16], want, rtol=1e-9, atol=1e-10)


def _check(gpu, p, host, dsys, res, orc=None):
    for (bins, ext, types), d, r in zip(host, dsys, res):
        if orc is not None:
            _check_oracle(orc, p, bins, ext, types, d, r)
        pk = make_params(bins.shape[2], p.nsteps, list(p.bin_schemes[: p.nschemes]),
                         list(p.estimators[: p.nestimators]), bool(p.jacobian))
        s1 = gpu.entropy1d(pk, types, bins, ext)
        s2 = gpu.entropy2d(pk, types, bins, ext)
        assert np.array_equal(d["s1"].cpu().numpy().reshape(s1.shape), s1)
        np.testing.assert_allclose(d["s2"].cpu().numpy().reshape(s2.shape), s2, rtol=1e-12,
                                   atol=1e-13)
        out = gpu.score(pk, types, s1, s2)
        np.testing.assert_allclose(r["mie"], out["mie"].reshape(r["mie"].shape), rtol=1e-9,
                                   atol=1e-12)
        np.testing.assert_allclose(r["mist"], out["mist"].reshape(r["mist"].shape), rtol=1e-9,
                                   atol=1e-12)
        mi = d["mi"].cpu().numpy()
        s1f = s1.reshape(len(types), -1)
        s2f = s2.reshape(mi.shape)
        iu = np.triu_indices(len(types), 1)
        np.testing.assert_allclose(mi, s1f[iu[0]] + s1f[iu[1]] - s2f, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("schemes,ests", [([50], [0]), ([50, 7], [0, 1])])
def test_batch_matches_oracle_and_single_trajectory(gpu, orc, schemes, ests):
    import torch
    specs = [(6, 5003, 1), (11, 12000, 2), (4, 997, 3), (9, 20011, 4)]
    nsteps = 10
    host, dsys = _systems(torch, gpu, specs, schemes, nsteps, len(ests))
    p = make_params(0, nsteps, schemes, ests, True)
    res = gpu.entropy_batch_dev(p, dsys)
    _check(gpu, p, host, dsys, res, orc)


def test_batch_graph_replay_sees_new_data(gpu):
    """The cached graph reads the trajectories' buffers when it runs: new
    contents in the same buffers give the new trajectories' results."""
    import torch
    specs = [(7, 4001, 5), (10, 8000, 6)]
    host, dsys = _systems(torch, gpu, specs, [30], 5, 1)
    p = make_params(0, 5, [30], [0], True)
    gpu.entropy_batch_dev(p, dsys)
    launches0 = gpu.launches
    specs2 = [(7, 4001, 15), (10, 8000, 16)]
    host2, dsys2 = _systems(torch, gpu, specs2, [30], 5, 1)
    for d, d2 in zip(dsys, dsys2):
        d["bins"].copy_(d2["bins"])
        d["ext"].copy_(d2["ext"])
    res = gpu.entropy_batch_dev(p, dsys)
    assert gpu.launches > launches0
    _check(gpu, p, host2, dsys, res)


def test_batch_rejects_bad_input(gpu):
    import torch
    from centre_gb300.api import CentreError
    host, dsys = _systems(torch, gpu, [(5, 2000, 7)], [20], 4, 1)
    p = make_params(0, 4, [20], [2], True)   # Chao-Shen is not batched
    with pytest.raises(CentreError):
        gpu.entropy_batch_dev(p, dsys)
    p = make_params(0, 4, [10], [0], True)   # bins above the bin count
    dsys[0]["bins"][3, 0, 17] = 12
    with pytest.raises(CentreError):
        gpu.entropy_batch_dev(p, dsys)
