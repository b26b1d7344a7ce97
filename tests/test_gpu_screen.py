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


def test_screen_short_prefix_gap_is_all_pairs_bias(gpu):
    """At short convergence prefixes the screened A-MIST total differs from
    the all-pairs MIST total by more than at the full trajectory (on the
    5000-atom chain 0.64 % at the 10 % prefix, 0.09 % at 100 %).  Both are
    plug-in estimates over few frames, biased by the same small-sample term,
    and the all-pairs tree, a maximum over every noisy pair MI, collects more
    of it.  On the 1000-atom chain (100,000 frames, 50 bins, 10 prefixes):
    at every prefix the screened total lies closer to the all-pairs value
    over the whole trajectory (ten times the frames of the first prefix, the
    least biased estimate available) than the all-pairs total at that prefix
    does, and its gap to the all-pairs total is smaller than the all-pairs
    total's own distance from that value (3.5 % of it at the 10 % prefix);
    at the full trajectory the screened total is within 0.5 % of it."""
    import torch
    from centre_gb300.synth import chain_blocks_torch
    dev = torch.device("cuda", 0)
    natoms, nframes, nb = 1000, 100_000, 50
    blocks = chain_blocks_torch(natoms, nframes, 4000, dev, coupling="block8")
    ndof = sum(x.shape[0] for _, x in blocks)
    bins = torch.empty((ndof, 1, nframes), dtype=torch.uint8, device=dev)
    ext = torch.empty((ndof, 4), dtype=torch.float64, device=dev)
    off = 0
    for typ, data in blocks:
        k = data.shape[0]
        gpu.discretize_dev(typ, data, [nb], bins[off:off + k], ext[off:off + k])
        off += k
    del blocks
    types = torch.tensor(sum([[t] * k for t, k in ((1, natoms - 1), (2, natoms - 2),
                                                  (3, natoms - 3))], []),
                         dtype=torch.uint8, device=dev)
    p = make_params(nframes, 10, [nb], [0], True)
    full = _mist_total(gpu, torch, p, types, bins, ext, None)
    sp = make_screen_params(feat_div=5, ntrain=200_000, nprefilter=256, nneigh=64, epochs=3,
                            batch=4096, lr=2e-3, seed=17)
    pairs, w, losses = gpu.screen_dev(p, sp, types, bins, ext)
    screened = _mist_total(gpu, torch, p, types, bins, ext, pairs)
    conv = full[-1]
    d_scr = np.abs(screened - conv)
    d_all = np.abs(full - conv)
    gap = np.abs(screened - full)
    print("prefix gap screened/all-pairs:", np.round(gap / np.abs(full), 5))
    print("distance to the full-trajectory value, screened:", np.round(d_scr / abs(conv), 5))
    print("distance to the full-trajectory value, all pairs:", np.round(d_all / abs(conv), 5))
    assert gap[-1] <= 5e-3 * abs(conv)
    assert np.all(d_scr[:-1] < d_all[:-1]), (d_scr, d_all)
    assert np.all(gap[:-1] < d_all[:-1]), (gap, d_all)
    assert gap[0] <= 0.1 * d_all[0], (gap[0], d_all[0])


@pytest.mark.parametrize("n,K", [(300, 1000), (517, 64), (1024, 4096), (130, 20001)])
def test_correlation_gemm_vs_torch_fp32(gpu, n, K):
    """The screen's tensor-core GEMM R = X X^T (bf16 operands, fp32
    accumulation) against torch's fp32 product of the same bf16 values;
    shapes cut tiles, K chunks and the row padding at every edge."""
    import torch
    dev = torch.device("cuda", 0)
    g = torch.Generator(device="cpu").manual_seed(n + K)
    ldx = (K + 7) // 8 * 8
    ldr = (n + 3) // 4 * 4
    X = torch.zeros((n, ldx), dtype=torch.bfloat16)
    X[:, :K] = (torch.randn((n, K), generator=g) / K ** 0.5).to(torch.bfloat16)
    X[:, K:] = float("nan")   # the padding is never read
    Xd = X.to(dev)
    R = torch.full((n, ldr), float("nan"), dtype=torch.float32, device=dev)
    gpu.corr_gemm_dev(Xd, n, K, ldx, R, ldr)
    Xf = X[:, :K].to(torch.float64)
    want = (Xf @ Xf.T).to(torch.float32)
    got = R[:, :n].cpu()
    # fp32 sums of K bf16 products in another order: |err| ~ K * 2^-24 * sum|x y|
    tol = 4 * K * 2.0 ** -24 * (Xf.abs() @ Xf.abs().T).to(torch.float32) + 1e-6
    assert torch.all((got - want).abs() <= tol), float((got - want).abs().max())
