"""The learned pair screen on the GPU: its training kernels' gradients
against the CPU oracle of the network, the shape of what it selects, and
what it gains over the exact all-pairs method (the fallback and the yardstick):
far fewer exact pairs at a total MIST entropy within 0.5 %."""
import numpy as np
import pytest

from centre_gb300.api import make_params, make_screen_params
from centre_gb300.synth import chain_trajectory
from oracle import screen_mlp as M

pytestmark = pytest.mark.gpu


def test_mlp_gradients_match_oracle(gpu):
    rng = np.random.default_rng(3)
    w = rng.normal(0, 0.25, M.NPARAMS).astype(np.float32)
    x = np.abs(rng.normal(0, 1, (512, M.NFEAT))).astype(np.float32)
    y = np.abs(rng.normal(0, 0.3, 512)).astype(np.float32)
    pred, grad, loss = gpu.screen_mlp_grad(w, x, y)
    opred, ograd, oloss = M.forward_backward(w, x, y, round_bf16=True)
    # FP32 sums on the GPU against float64 in the oracle, bf16 rounding at
    # the same points: a rounding step can flip for a value within FP32
    # error of a bf16 boundary, so compare at 1e-2 of each block's scale
    np.testing.assert_allclose(pred, opred, rtol=1e-3, atol=1e-3 * np.abs(opred).max())
    assert abs(loss - oloss) <= 1e-3 * oloss
    blocks = [(M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2),
              (M.OFF_B2, M.OFF_W3), (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.NPARAMS)]
    for a, b in blocks:
        scale = np.abs(ograd[a:b]).max() + 1e-12
        err = np.abs(grad[a:b] - ograd[a:b]).max() / scale
        assert err < 1e-2, (a, b, err)


def _chain_on_gpu(gpu, torch, natoms, nframes, nb, seed):
    tr = chain_trajectory(natoms, nframes, seed=seed, coupling="block8")
    dev = torch.device("cuda", 0)
    bins, ext, types = [], [], []
    for typ, blk in tr.blocks():
        b, e = gpu.discretize(typ, blk, [nb], bins_ref=nb, optimize=True)
        bins.append(b)
        ext.append(e)
        types += [typ] * len(b)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    return t(np.concatenate(bins)), t(np.concatenate(ext)), t(np.array(types, np.uint8))


def _mist_total(gpu, torch, p, types, bins, ext, pairs):
    ndof = bins.shape[0]
    G = p.nsteps
    s1 = torch.empty((ndof, G), dtype=torch.float64, device=bins.device)
    gpu.entropy1d_dev(p, types, bins, ext, s1)
    npairs = pairs.shape[0] if pairs is not None else ndof * (ndof - 1) // 2
    s2 = torch.empty((npairs, G), dtype=torch.float64, device=bins.device)
    gpu.entropy2d_dev(p, types, bins, ext, s2, pairs)
    out = gpu.score_dev(p, types, s1, s2, pairs, True)
    return out["mist"][:, 16]       # S2 column per step


def test_screen_selects_sorted_unique_pairs(gpu):
    import torch
    bins, ext, types = _chain_on_gpu(gpu, torch, 60, 20000, 30, 5)
    p = make_params(20000, 5, [30], [0], True)
    sp = make_screen_params(ntrain=8192, nprefilter=64, nneigh=8, epochs=4, batch=1024)
    pairs, w, losses = gpu.screen_dev(p, sp, types, bins, ext)
    pr = pairs.cpu().numpy().astype(np.int64)
    ndof = bins.shape[0]
    assert len(pr) <= ndof * 8 and len(pr) >= ndof * 8 // 2
    assert np.all(pr[:, 0] < pr[:, 1]) and pr.max() < ndof
    key = pr[:, 0] * ndof + pr[:, 1]
    assert np.all(np.diff(key) > 0)               # row-major, no duplicates
    assert np.all(np.isfinite(w)) and losses[-1] < losses[0]
    # the same weights, not retrained, select the same pairs
    sp2 = make_screen_params(ntrain=8192, nprefilter=64, nneigh=8, epochs=4, batch=1024,
                             train=False)
    pairs2, _, _ = gpu.screen_dev(p, sp2, types, bins, ext, weights=w)
    assert torch.equal(pairs, pairs2)


def test_screen_gain_over_all_pairs(gpu):
    """A-MIST over the screened pairs against MIST over all pairs on a
    200-atom chain: at most 0.5 % total-entropy difference at every step,
    with a small fraction of the exact pair work."""
    import torch
    nframes = 40000
    bins, ext, types = _chain_on_gpu(gpu, torch, 200, nframes, 50, 7)
    ndof = bins.shape[0]
    p = make_params(nframes, 10, [50], [0], True)
    full = _mist_total(gpu, torch, p, types, bins, ext, None)
    sp = make_screen_params(ntrain=50000, nprefilter=256, nneigh=64, epochs=8, batch=2048)
    pairs, w, losses = gpu.screen_dev(p, sp, types, bins, ext)
    screened = _mist_total(gpu, torch, p, types, bins, ext, pairs)
    rel = np.abs(screened - full) / np.abs(full)
    assert rel.max() <= 5e-3, rel
    assert pairs.shape[0] <= 0.25 * ndof * (ndof - 1) // 2
