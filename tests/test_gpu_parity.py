"""GPU parity: the CUDA library through its C ABI against the CPU oracle and
the reference's golden fixtures.  Bins and counts must be bit-identical;
entropies agree within 1e-9 relative, with an absolute floor of 1e-13 for
entropies within rounding of zero (different summation orders of the
reference's own per-cell sum already differ at ~1e-15 absolute)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from centre_gb300.api import CentreError, make_params
from centre_gb300.synth import chain_trajectory

pytestmark = pytest.mark.gpu

RTOL = 1e-9


def all_pairs(n):
    return np.array([(i, j) for i in range(n) for j in range(i + 1, n)], np.uint32).reshape(-1, 2)


def stack_blocks(tr, gpu, schemes, optimize=True):
    bins, ext, types = [], [], []
    for typ, blk in tr.blocks():
        b, e = gpu.discretize(typ, blk, schemes, bins_ref=schemes[0], optimize=optimize)
        bins.append(b)
        ext.append(e)
        types += [typ] * len(b)
    return np.concatenate(bins), np.concatenate(ext), np.array(types, np.uint8)


# ------------------------------------------------------------ discretise --
def test_discretize_golden_fixture(gpu, golden):
    g = golden("discretize_ref.npz")
    for sch_name, sch in (("s30", [30]), ("s2", [50, 7])):
        for typ, name in ((1, "bonds"), (2, "angles"), (3, "torsions")):
            for opt in ((1, 0) if typ == 3 else (1,)):
                bins, ext = gpu.discretize(typ, g[name], sch, bins_ref=sch[0], optimize=bool(opt))
                key = f"{name}_{sch_name}_o{opt}"
                assert np.array_equal(bins, g[key + "_bins"]), key
                want = g[key + "_ext"]
                assert np.array_equal(ext[:, [0, 1, 3]], want[:, [0, 1, 3]]), key
                np.testing.assert_allclose(ext[:, 2], want[:, 2], rtol=1e-12, err_msg=key)


@pytest.mark.parametrize("nframes", [50_000, 20_001, 1_003, 37, 150_000, 300_001])
def test_discretize_synthetic_vs_oracle(gpu, orc, nframes):
    tr = chain_trajectory(9, nframes, seed=nframes)
    for typ, blk in tr.blocks():
        for sch in ([30], [50, 7, 255]):
            for opt in ((True, False) if typ == 3 else (True,)):
                gb, ge = gpu.discretize(typ, blk, sch, bins_ref=sch[0], optimize=opt)
                ob, oe = orc.discretize(typ, blk, sch, bins_ref=sch[0], optimize=opt)
                assert np.array_equal(gb, ob), (typ, sch, opt)
                assert np.array_equal(ge[:, [0, 1, 3]], oe[:, [0, 1, 3]])
                np.testing.assert_allclose(ge[:, 2], oe[:, 2], rtol=1e-12)


def test_discretize_chunked_transfers_vs_oracle(gpu, orc):
    """Blocks of 256 DOFs and more go through the host entry in four chunks
    whose transfers overlap the binning: bins and extremes equal the
    oracle's, and a value out of domain in the last chunk fails the call."""
    tr = chain_trajectory(300, 20_001, seed=77)
    for typ, blk in tr.blocks():
        gb, ge = gpu.discretize(typ, blk, [50, 7], bins_ref=50, optimize=True)
        ob, oe = orc.discretize(typ, blk, [50, 7], bins_ref=50, optimize=True)
        assert blk.shape[0] >= 256
        assert np.array_equal(gb, ob), typ
        assert np.array_equal(ge[:, [0, 1, 3]], oe[:, [0, 1, 3]])
        np.testing.assert_allclose(ge[:, 2], oe[:, 2], rtol=1e-12)
    bad = np.array(tr.blocks()[2][1])
    bad[290, 17] = 7.0   # torsion >= 2pi
    with pytest.raises(CentreError) as e:
        gpu.discretize(3, bad, [50], bins_ref=50, optimize=True)
    assert e.value.status == -1


def test_discretize_edge_values_vs_oracle(gpu, orc):
    """Signed zeros, exact zeros, constant DOFs, wide uniform ranges and
    values on a single float: the binning table's edge cases."""
    rng = np.random.default_rng(11)
    n = 40_000
    rows = {
        1: [np.abs(rng.normal(0, 1e-3, n)), rng.uniform(0.0, 9.0, n), np.full(n, 1.5),
            np.where(rng.random(n) < 0.5, 0.0, 1.25)],
        2: [rng.uniform(0.0, np.pi, n), np.full(n, 2.0), np.where(rng.random(n) < 0.3, 0.0, 1.0)],
        3: [rng.uniform(0.0, 2 * np.pi, n), np.where(rng.random(n) < 0.5, 0.0, 3.0),
            np.mod(rng.vonmises(0.0, 2.0, n), 2 * np.pi)],
    }
    for typ, rs in rows.items():
        x = np.stack(rs).astype(np.float32)
        x[:, ::97] = np.float32(-0.0)
        for sch in ([30], [255, 16]):
            for opt in ((True, False) if typ == 3 else (True,)):
                gb, ge = gpu.discretize(typ, x, sch, bins_ref=sch[0], optimize=opt)
                ob, oe = orc.discretize(typ, x, sch, bins_ref=sch[0], optimize=opt)
                assert np.array_equal(gb, ob), (typ, sch, opt)
                assert np.array_equal(ge[:, [0, 1, 3]], oe[:, [0, 1, 3]])


def test_discretize_rejects_out_of_domain(gpu):
    x = np.full((2, 64), 1.0, np.float32)
    x[1, 5] = 7.0   # torsion >= 2pi
    with pytest.raises(CentreError) as e:
        gpu.discretize(3, x, [10])
    assert e.value.status == -1
    x = np.full((1, 64), 1.5, np.float32)
    x[0, 3] = -0.1  # negative bond
    with pytest.raises(CentreError):
        gpu.discretize(1, x, [10])
    x = np.full((1, 64), 1.5, np.float32)
    x[0, 3] = np.nan
    with pytest.raises(CentreError):
        gpu.discretize(2, x, [10])


# ----------------------------------------------------------------- 1-D ----
def test_entropy1d_golden_fixture(gpu, golden):
    g = golden("entropy_ref.npz")
    sch = g["schemes"].tolist()
    for jac in (0, 1):
        p = make_params(g["bins"].shape[2], int(g["nsteps"]), sch, g["ests"].tolist(), bool(jac))
        s1 = gpu.entropy1d(p, g["types"], g["bins"], g["ext"])
        np.testing.assert_allclose(s1, g[f"s1_j{jac}"], rtol=RTOL, atol=1e-13)
    p = make_params(4000, int(g["nsteps"]), [3], g["ests"].tolist(), True, kde=True)
    s1 = gpu.entropy1d(p, np.full(4, 3, np.uint8), g["kde_bins"], np.full((4, 4), 1000.0))
    np.testing.assert_allclose(s1, g["kde_s1"], rtol=RTOL, atol=1e-13)


def test_entropy1d_counts_exact(gpu, orc):
    tr = chain_trajectory(8, 30_011, seed=5)
    bins, ext, types = stack_blocks(tr, gpu, [30, 11])
    p = make_params(bins.shape[2], 7, [30, 11], [0, 1, 2, 3], True)
    s1, freq = gpu.entropy1d(p, types, bins, ext, want_freq=True)
    for d in range(len(bins)):
        want = orc.bin1d(bins[d], 7, [30, 11])
        assert np.array_equal(freq[d].reshape(-1), want)
    o = orc.entropy1d(types, bins, ext, 7, [30, 11], [0, 1, 2, 3], True)
    np.testing.assert_allclose(s1, o, rtol=RTOL, atol=1e-13)


# ----------------------------------------------------------------- 2-D ----
@pytest.mark.parametrize("nframes,nsteps", [(20_000, 4), (10_007, 3), (4_096, 1)])
def test_counts2d_exact(gpu, orc, nframes, nsteps):
    tr = chain_trajectory(6, nframes, seed=nframes + nsteps)
    bins, ext, types = stack_blocks(tr, gpu, [30, 7])
    pairs = all_pairs(len(bins))
    p = make_params(nframes, nsteps, [30, 7])
    freq = gpu.counts2d(p, bins, pairs)
    for q, (i, j) in enumerate(pairs):
        want = orc.bin2d(bins[i], bins[j], nsteps, [30, 7])
        assert np.array_equal(freq[q].reshape(-1), want), (i, j)


def test_entropy2d_golden_fixture(gpu, golden):
    g = golden("entropy_ref.npz")
    sch = g["schemes"].tolist()
    for jac in (0, 1):
        p = make_params(g["bins"].shape[2], int(g["nsteps"]), sch, g["ests"].tolist(), bool(jac),
                        counts_form=1)
        s2 = gpu.entropy2d(p, g["types"], g["bins"], g["ext"], g["pairs"])
        np.testing.assert_allclose(s2, g[f"s2_j{jac}"], rtol=RTOL, atol=1e-13)
    kp = all_pairs(4)
    p = make_params(4000, int(g["nsteps"]), [3], g["ests"].tolist(), True, kde=True, counts_form=1)
    s2 = gpu.entropy2d(p, np.full(4, 3, np.uint8), g["kde_bins"], np.full((4, 4), 1000.0), kp)
    np.testing.assert_allclose(s2, g["kde_s2"], rtol=RTOL, atol=1e-13)


@pytest.mark.parametrize("ests", [[0], [0, 1], [1]])
def test_entropy2d_moments_all_pairs_vs_oracle(gpu, orc, ests):
    tr = chain_trajectory(12, 40_000, seed=len(ests))
    bins, ext, types = stack_blocks(tr, gpu, [50])
    p = make_params(40_000, 10, [50], ests, True, counts_form=1)
    s2 = gpu.entropy2d(p, types, bins, ext)       # all pairs, implicit
    pairs = all_pairs(len(bins))
    o = orc.entropy2d(pairs, types, bins, ext, 10, [50], ests, True)
    np.testing.assert_allclose(s2, o, rtol=RTOL, atol=1e-13)
    s2b = gpu.entropy2d(p, types, bins, ext, pairs)  # explicit list
    assert np.array_equal(s2, s2b)


def test_entropy2d_explicit_pair_list_orientation(gpu, orc):
    tr = chain_trajectory(10, 12_000, seed=3)
    bins, ext, types = stack_blocks(tr, gpu, [20])
    rng = np.random.default_rng(0)
    pairs = rng.integers(0, len(bins), size=(60, 2)).astype(np.uint32)
    pairs = pairs[pairs[:, 0] != pairs[:, 1]]
    for ests in ([0, 1], [2, 3], [0, 1, 2, 3]):
        p = make_params(12_000, 4, [20], ests, True, counts_form=1)
        s2 = gpu.entropy2d(p, types, bins, ext, pairs)
        o = orc.entropy2d(pairs, types, bins, ext, 4, [20], ests, True)
        np.testing.assert_allclose(s2, o, rtol=RTOL, atol=1e-13)


@pytest.mark.parametrize("ndof,nframes,nsteps,nb", [
    (2, 17, 4, 2),        # fewest DOFs, frames not divisible by steps
    (3, 1003, 10, 255),   # largest bin count
    (5, 4096, 1, 1),      # a single bin: every entropy from one cell
    (7, 999, 7, 13),
])
def test_entropy_edge_sizes_vs_oracle(gpu, orc, ndof, nframes, nsteps, nb):
    """Edge shapes of the count and entropy kernels against the oracle, all
    four estimators, including a constant DOF (one occupied bin)."""
    rng = np.random.default_rng(nframes + nb)
    bins = rng.integers(0, nb, size=(ndof, 1, nframes), dtype=np.uint8)
    bins[0, 0, :] = 0                                   # constant DOF
    types = np.array([(1 + k % 3) for k in range(ndof)], np.uint8)
    types.sort()
    ext = np.tile(np.array([[0.5, 2.5, 1.5, 0.0]]), (ndof, 1))
    ext[types == 3, 1] = 2 * np.pi
    ext[types == 2, 1] = np.pi
    ests = [0, 1, 2, 3]
    p = make_params(nframes, nsteps, [nb], ests, True)
    s1 = gpu.entropy1d(p, types, bins, ext)
    o1 = orc.entropy1d(types, bins, ext, nsteps, [nb], ests, True)
    np.testing.assert_allclose(s1, o1, rtol=RTOL, atol=1e-13)
    s2 = gpu.entropy2d(p, types, bins, ext)
    o2 = orc.entropy2d(all_pairs(ndof), types, bins, ext, nsteps, [nb], ests, True)
    np.testing.assert_allclose(s2, o2, rtol=RTOL, atol=1e-13)


def test_entropy2d_large_bins_explicit_pairs_vs_oracle(gpu, orc):
    """More than 214 bins with an explicit pair list (ML, MM): histograms that
    do not fit shared memory are counted in global memory."""
    rng = np.random.default_rng(240)
    ndof, nframes, nb = 6, 3001, 240
    bins = (rng.integers(0, 40, size=(ndof, 1, nframes)) * 6 % nb).astype(np.uint8)
    types = np.array([1, 1, 2, 2, 3, 3], np.uint8)
    ext = np.tile(np.array([[0.5, 2.5, 1.5, 0.0]]), (ndof, 1))
    ext[types == 3, 1] = 2 * np.pi
    ext[types == 2, 1] = np.pi
    pairs = np.array([(0, 5), (4, 1), (2, 3), (3, 2), (1, 2)], np.uint32)
    p = make_params(nframes, 3, [nb], [0, 1], True)
    s2 = gpu.entropy2d(p, types, bins, ext, pairs=pairs)
    o2 = orc.entropy2d(pairs, types, bins, ext, 3, [nb], [0, 1], True)
    np.testing.assert_allclose(s2, o2, rtol=RTOL, atol=1e-13)


def test_entropy2d_rejects_bad_bins(gpu):
    bins = np.zeros((3, 1, 1000), np.uint8)
    bins[1, 0, 10] = 40
    ext = np.tile(np.array([0.0, 1.0, 0.5, 0.0]), (3, 1))
    p = make_params(1000, 2, [30], [0], True, counts_form=1)
    with pytest.raises(CentreError) as e:
        gpu.entropy2d(p, np.array([1, 1, 1], np.uint8), bins, ext)
    assert e.value.status == -4


def test_pair_counts_report_bad_bin_of_any_thread(gpu):
    """A bin out of range read by any thread of the count kernel (here the
    one that takes frames 1000-1003, not thread 0) fails the call."""
    rng = np.random.default_rng(5)
    bins = rng.integers(0, 30, (6, 1, 4000), dtype=np.uint8)
    bins[4, 0, 1001] = 30
    p = make_params(4000, 2, [30], [0, 1], True, counts_form=1)
    with pytest.raises(CentreError) as e:
        gpu.pair_moments(p, bins)
    assert e.value.status == -4


@pytest.mark.parametrize("nframes,nsteps", [(100_000, 16), (100_000, 1), (70_001, 25)])
def test_pair_counts_of_concentrated_cells(gpu, orc, nframes, nsteps):
    """Histogram-form moments on cells far past the shared c ln c table and
    past 2^16 counts (three DOFs nearly constant, one exactly constant), with
    one step of 100,000 frames and with many short steps, and on a frame count
    that is not a multiple of 4 (rows off word boundaries, read through the
    funnel-shifted 32-bit loads): equal to the oracle's."""
    rng = np.random.default_rng(nframes + nsteps)
    nb = 50
    bins = rng.integers(0, nb, (7, 1, nframes), dtype=np.uint8)
    bins[0, 0] = 7
    for d, keep in ((1, 0.9), (2, 0.97), (3, 0.6)):
        bins[d, 0, rng.random(nframes) < keep] = 11 + d
    p = make_params(nframes, nsteps, [nb], [0, 1], True, counts_form=1)
    ca, za, sa = gpu.pair_moments(p, bins)
    xo, zo = oracle_moments(orc, bins[:, 0], nsteps, nb)
    assert np.array_equal(za, zo)
    np.testing.assert_allclose(ca.astype(np.float64) * 2.0 ** -sa, xo, rtol=1e-12,
                               atol=nb * nb * 2.0 ** -(sa + 1))


# --------------------------------------------------------------- score ----
def reference_edge_order(types):
    """Pairs in the reference's edge-list order: B/B, B/A, B/D, A/A, A/D, D/D
    blocks, row-major within each (src/EntropyScorer.cpp:675-741)."""
    idx = {t: np.nonzero(types == t)[0] for t in (1, 2, 3)}
    out = []
    for a, b in ((1, 1), (1, 2), (1, 3), (2, 2), (2, 3), (3, 3)):
        for x in idx[a]:
            for y in idx[b]:
                if a != b or x < y:
                    out.append((x, y))
    return np.array(out, np.uint32)


def test_score_sums_and_tree_vs_oracle(gpu, orc):
    tr = chain_trajectory(14, 30_000, seed=9)
    bins, ext, types = stack_blocks(tr, gpu, [30])
    p = make_params(30_000, 5, [30], [0, 1], True, counts_form=1)
    s1 = gpu.entropy1d(p, types, bins, ext)
    pairs = reference_edge_order(types)
    s2 = gpu.entropy2d(p, types, bins, ext, pairs)
    out = gpu.score(p, types, s1, s2, pairs)
    G = 2 * 1 * 5
    mi = out["mi"].reshape(len(pairs), G)
    s1g = s1.reshape(len(types), G)
    np.testing.assert_allclose(mi, s1g[pairs[:, 0]] + s1g[pairs[:, 1]] - s2.reshape(len(pairs), G),
                               rtol=0, atol=1e-13)
    mie = out["mie"].reshape(G, 17)
    blocks = {(1, 1): 3, (2, 2): 5, (3, 3): 7, (1, 2): 9, (1, 3): 11, (2, 3): 13}
    tp = np.sort(types[pairs], axis=1)
    for g in range(G):
        for t in (1, 2, 3):
            np.testing.assert_allclose(mie[g, t - 1], s1g[types == t, g].sum(), rtol=1e-12)
        for (a, b), col in blocks.items():
            m = (tp[:, 0] == a) & (tp[:, 1] == b)
            np.testing.assert_allclose(mie[g, col], s2.reshape(len(pairs), G)[m, g].sum(), rtol=1e-12)
            np.testing.assert_allclose(mie[g, col + 1], mi[m, g].sum(), rtol=1e-9, atol=1e-9)
        # tree: the reference's Boruvka on the same edge order
        t_or = orc.mst(len(types), pairs[:, 0], pairs[:, 1], mi[:, g])
        assert sorted(out["tree"][g].tolist()) == sorted(t_or.tolist())
        mist = out["mist"].reshape(G, 17)[g]
        np.testing.assert_allclose(mist[16], mie[g, 15] - mi[t_or, g].sum(), rtol=1e-9, atol=1e-9)
    # implicit all-pairs mode ranks edges in the same reference order
    s2u = gpu.entropy2d(p, types, bins, ext)
    outu = gpu.score(p, types, s1, s2u)
    ap = all_pairs(len(types))
    for g in range(G):
        got = {tuple(ap[q]) for q in outu["tree"][g]}
        want = {tuple(pairs[q]) for q in out["tree"][g]}
        assert got == want


def test_score_tree_ties_follow_reference_order(gpu, orc, golden):
    g = golden("mst_ref.npz")
    for k in range(12):
        nv = int(g[f"g{k}_nv"])
        src, dst, w = g[f"g{k}_src"], g[f"g{k}_dst"], g[f"g{k}_w"]
        # feed MI through the scorer: s1 = 0, s2 = -w  =>  MI = w
        p = make_params(4, 1, [2], [0], False)
        types = np.full(nv, 3, np.uint8)
        s1 = np.zeros((nv, 1, 1, 1))
        s2 = (-w).reshape(-1, 1, 1, 1)
        pairs = np.stack([src, dst], 1)
        out = gpu.score(p, types, s1, s2, pairs)
        got = sorted((int(src[q]), int(dst[q])) for q in out["tree"][0])
        want = sorted(zip(g[f"g{k}_tsrc"].tolist(), g[f"g{k}_tdst"].tolist()))
        assert got == want, k


# ----------------------------------------------------------- example-1 ----
def test_example1_on_gpu(gpu):
    d = np.load(os.path.join(GOLDEN, "example1.npz"))
    with open(os.path.join(GOLDEN, "example1.json")) as f:
        meta = json.load(f)
    names = {"B": "bonds", "A": "angles", "T": "torsions"}
    tcode = {"B": 1, "A": 2, "T": 3}
    coord = np.concatenate([d[f"{names[k]}_coord"] for k in "BAT"])
    ext = np.concatenate([d[f"{names[k]}_ext"] for k in "BAT"])
    types = np.concatenate([np.full(len(d[f"{names[k]}_coord"]), tcode[k], np.uint8) for k in "BAT"])
    off = {"B": 0, "A": len(d["bonds_coord"]), "T": len(d["bonds_coord"]) + len(d["angles_coord"])}
    p = make_params(coord.shape[2], 4, [30], [0], True)
    s1 = gpu.entropy1d(p, types, coord, ext)
    col = meta["mie_columns"].index("DIHED-S1")
    for step in range(4):
        assert abs(s1[types == 3, 0, 0, step].sum() - meta["mie_rows"][step][col]) <= 0.5e-4 + 1e-9
    s2 = gpu.entropy2d(p, types, coord, ext)
    ap = all_pairs(len(types))
    lut = {tuple(x): q for q, x in enumerate(ap.tolist())}
    for step in range(4):
        for a, b, i, j, want in meta["trees"][str(step)]:
            x, y = off[a] + i, off[b] + j
            q = lut[(min(x, y), max(x, y))]
            mi = s1[x, 0, 0, step] + s1[y, 0, 0, step] - s2[q, 0, 0, step]
            assert abs(mi - want) <= 0.5e-6 + 1e-9


def test_entropies_from_unaligned_bins_view(gpu):
    """A bins pointer that is not 4-byte aligned (an offset view into a
    larger device buffer) takes the byte-load path and gives the same 1-D and
    2-D entropies as an aligned copy."""
    import torch
    tr = chain_trajectory(10, 8_000, seed=3)
    bins, ext, types = stack_blocks(tr, gpu, [30])
    p = make_params(8_000, 4, [30], [0, 1], True)
    want1 = gpu.entropy1d(p, types, bins, ext)
    want2 = gpu.entropy2d(p, types, bins, ext)
    dev = torch.device("cuda", 0)
    raw = torch.zeros(bins.size + 3, dtype=torch.uint8, device=dev)
    d_types = torch.from_numpy(types).to(dev)
    d_ext = torch.from_numpy(ext).to(dev)
    ndof = len(types)
    for off in (1, 2, 3):
        view = raw[off:off + bins.size].view(bins.shape)
        view.copy_(torch.from_numpy(bins))
        assert view.data_ptr() % 4 == off % 4
        s1 = torch.empty((ndof, 2, 1, 4), dtype=torch.float64, device=dev)
        s2 = torch.empty((ndof * (ndof - 1) // 2, 2, 1, 4), dtype=torch.float64, device=dev)
        gpu.entropy1d_dev(p, d_types, view, d_ext, s1)
        gpu.entropy2d_dev(p, d_types, view, d_ext, s2)
        torch.cuda.synchronize()
        assert np.array_equal(s1.cpu().numpy(), want1), off
        assert np.array_equal(s2.cpu().numpy(), want2), off


# ------------------------------------------------- size-independent checks --
def test_full_size_properties(gpu):
    """At the 1000-atom shape: counts cover every frame of every step,
    plug-in MI is non-negative, results are run-to-run identical."""
    import torch
    tr = chain_trajectory(60, 100_000, seed=1, coupling="block8")
    bins, ext, types = stack_blocks(tr, gpu, [50])
    p = make_params(100_000, 10, [50], [0, 1], True, counts_form=1)
    s1, freq = gpu.entropy1d(p, types, bins, ext, want_freq=True)
    assert np.all(freq.sum(axis=2) == (np.arange(1, 11) * 10_000)[None, :])
    s2 = gpu.entropy2d(p, types, bins, ext)
    s2b = gpu.entropy2d(p, types, bins, ext)
    assert np.array_equal(s2, s2b)
    out = gpu.score(p, types, s1, s2, build_tree=False)
    assert out["mi"][:, 0].min() > -1e-10   # ML plug-in MI >= 0
    del torch


# ------------------------------------------------- tensor-core counts ----
def oracle_moments(orc, bins, nsteps, nb):
    """sum c ln c and non-empty cells per pair/step from the oracle's counts."""
    n = len(bins)
    out_x, out_z = [], []
    for i in range(n):
        for j in range(i + 1, n):
            f = orc.bin2d(bins[i], bins[j], nsteps, [nb]).reshape(nsteps, -1).astype(np.float64)
            x = np.where(f > 1, f * np.log(np.where(f > 0, f, 1)), 0).sum(axis=1)
            out_x.append(x)
            out_z.append((f > 0).sum(axis=1))
    return np.array(out_x), np.array(out_z)


@pytest.mark.parametrize("natoms,nframes,nsteps,nb", [
    (4, 4_096, 1, 50), (8, 20_000, 4, 50), (12, 10_007, 3, 30), (30, 30_000, 10, 16),
    (10, 12_000, 2, 100), (6, 8_000, 2, 255), (9, 6_000, 3, 32), (7, 5_001, 2, 64),
    (6, 4_000, 2, 128), (5, 3_000, 2, 136), (7, 1_000, 10, 24), (6, 997, 7, 17)])
def test_tc_counts_identical_to_atomic(gpu, orc, natoms, nframes, nsteps, nb):
    """Moments of the tensor-core form against the oracle's counts and the
    histogram form.  The cases cover the three one-hot encodings (bins below
    64, below 128, up to 255), bin counts whose 8-row groups stay inside one
    DOF (multiples of 8) and ones that straddle two, frame counts that are not
    multiples of 16 (the bins are re-pitched for TMA), and convergence steps
    shorter than a 128-frame block (several step ends inside one block)."""
    tr = chain_trajectory(natoms, nframes, seed=natoms * 7 + nb)
    bins, ext, types = stack_blocks(tr, gpu, [nb])
    pa = make_params(nframes, nsteps, [nb], [0, 1], True, counts_form=1)
    pt = make_params(nframes, nsteps, [nb], [0, 1], True, counts_form=2)
    if nb * nb * 4 <= 200 * 1024:
        ca, za, sa = gpu.pair_moments(pa, bins)
    ct, zt, st = gpu.pair_moments(pt, bins)
    xo, zo = oracle_moments(orc, bins[:, 0], nsteps, nb)
    assert np.array_equal(zt, zo)
    # sum of c ln c in units of 2^-scale: each cell rounded by at most half a unit
    xt = ct.astype(np.float64) * 2.0 ** -st
    np.testing.assert_allclose(xt, xo, rtol=1e-12, atol=nb * nb * 2.0 ** -(st + 1))
    if nb * nb * 4 <= 200 * 1024:
        assert sa == st and np.array_equal(ct, ca) and np.array_equal(zt, za)
        s_at = gpu.entropy2d(pa, types, bins, ext)
        s_tc = gpu.entropy2d(pt, types, bins, ext)
        assert np.array_equal(s_at, s_tc)


def test_tc_second_scheme(gpu):
    """Two bin schemes: the tensor-core form reads the second scheme's rows
    (an offset of nframes into each DOF's bins) and matches the histogram
    form bit for bit on both."""
    tr = chain_trajectory(9, 8_000, seed=91)
    bins, ext, types = stack_blocks(tr, gpu, [16, 40])
    pa = make_params(8_000, 4, [16, 40], [0, 1], True, counts_form=1)
    pt = make_params(8_000, 4, [16, 40], [0, 1], True, counts_form=2)
    for sch in (0, 1):
        ca, za, sa = gpu.pair_moments(pa, bins, scheme=sch)
        ct, zt, st = gpu.pair_moments(pt, bins, scheme=sch)
        assert sa == st and np.array_equal(ca, ct) and np.array_equal(za, zt)
    assert np.array_equal(gpu.entropy2d(pa, types, bins, ext), gpu.entropy2d(pt, types, bins, ext))


def test_tc_rejects_bins_out_of_range(gpu):
    from centre_gb300.api import CentreError
    tr = chain_trajectory(5, 4_000, seed=3)
    bins, ext, types = stack_blocks(tr, gpu, [20])
    bins[2, 0, 1234] = 20
    pt = make_params(4_000, 2, [20], [0], True, counts_form=2)
    with pytest.raises(CentreError):
        gpu.pair_moments(pt, bins)


@pytest.mark.parametrize("natoms,nframes,nsteps,nb", [
    (200, 20_000, 4, 50), (200, 12_000, 3, 16), (120, 10_000, 2, 30)])
def test_tc_counts_many_tiles_per_cta(gpu, orc, natoms, nframes, nsteps, nb):
    """Thousands of 256 x 256 tiles for 76 persistent CTA pairs: every pair
    walks many tiles, and its producer warps move their stages from tile to
    tile (the 594-DOF chain at 50 bins gives about 6,900 tiles).  The moments
    must equal the shared-memory histogram's bit for bit on every run, and a
    sample of pairs must equal the oracle's counts."""
    tr = chain_trajectory(natoms, nframes, seed=natoms + nb, coupling="block8")
    bins, ext, types = stack_blocks(tr, gpu, [nb])
    pa = make_params(nframes, nsteps, [nb], [0, 1], True, counts_form=1)
    pt = make_params(nframes, nsteps, [nb], [0, 1], True, counts_form=2)
    ca, za, sa = gpu.pair_moments(pa, bins)
    for run in range(3):
        ct, zt, st = gpu.pair_moments(pt, bins)
        assert st == sa
        bad = np.nonzero(np.any(ct != ca, axis=1) | np.any(zt != za, axis=1))[0]
        assert len(bad) == 0, f"run {run}: {len(bad)} pairs differ, first {bad[:5]}"
    ndof = len(bins)
    rng = np.random.default_rng(nb)
    for _ in range(12):
        i, j = sorted(rng.choice(ndof, 2, replace=False))
        q = i * ndof - i * (i + 1) // 2 + (j - i - 1)
        f = orc.bin2d(bins[i, 0], bins[j, 0], nsteps, [nb]).reshape(nsteps, -1).astype(np.float64)
        x = np.where(f > 1, f * np.log(np.where(f > 0, f, 1)), 0).sum(axis=1)
        assert np.array_equal(zt[q], (f > 0).sum(axis=1)), (i, j)
        xt = ct[q].astype(np.float64) * 2.0 ** -st
        np.testing.assert_allclose(xt, x, rtol=1e-12, atol=nb * nb * 2.0 ** -(st + 1))
    s_at = gpu.entropy2d(pa, types, bins, ext)
    s_tc = gpu.entropy2d(pt, types, bins, ext)
    assert np.array_equal(s_at, s_tc)


# ----------------------------------------------------- von Mises KDE ----
# Frames per torsion whose conformer may differ from the oracle's: only a
# frame within rounding (1e-9 rad) of a minimum can fall on either side, and
# a float32 torsion lies that close to a given double minimum with
# probability ~1e-2 per float value it takes, so more than one such frame in
# a torsion means the minima or the assignment disagree.
KDE_MAX_DIFF_FRAMES = 1


def _kde_compare(gb, gm, gf, ob, omins, of, x):
    """Bins equal except frames within rounding of a minimum (at most
    KDE_MAX_DIFF_FRAMES per torsion); minima agree.  Returns the number of
    differing frames."""
    assert gf == of
    np.testing.assert_allclose(gm[:gf], omins, rtol=0, atol=1e-9)
    diff = np.nonzero(gb != ob)[0]
    for k in diff:
        assert np.min(np.abs(np.float64(x[k]) - omins)) < 1e-9, (k, x[k])
    assert len(diff) <= KDE_MAX_DIFF_FRAMES, len(diff)
    return len(diff)


def test_vmkde_golden_fixture(gpu, golden):
    g = golden("vmkde_ref.npz")
    t = g["torsions"]
    ndiff = 0
    for kappa in (1.0, 8.0):
        bins, mins, nf = gpu.discretize_vmkde(t, 5, kappa, 5, 1e-4, 1000)
        for d in range(len(t)):
            want_b = g[f"k{kappa:g}_d{d}_bins"]
            want_m = g[f"k{kappa:g}_d{d}_minima"]
            ndiff += _kde_compare(bins[d, 0], mins[d], int(nf[d]), want_b, want_m, len(want_m),
                                  t[d])
    print(f"KDE frames differing from the reference fixture: {ndiff} of "
          f"{2 * t.shape[0] * t.shape[1]}")


@pytest.mark.parametrize("nframes,kappa,nconf", [(20_000, 1.0, 5), (10_007, 8.0, 3), (4_000, 50.0, 9)])
def test_vmkde_vs_oracle(gpu, orc, nframes, kappa, nconf):
    tr = chain_trajectory(12, nframes, seed=int(kappa) + nframes)
    t = tr.torsions
    bins, mins, nf = gpu.discretize_vmkde(t, nconf, kappa, 5, 1e-4, 1000)
    ndiff = 0
    for d in range(len(t)):
        ob, om, of = orc.vmkde(t[d], nconf, kappa, 5, 1e-4, 1000)
        ndiff += _kde_compare(bins[d, 0], mins[d], int(nf[d]), ob, om, of, t[d])
    print(f"KDE frames differing from the oracle: {ndiff} of {t.size}")
