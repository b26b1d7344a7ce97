"""Pin the CPU oracle against golden outputs of the reference.

The fixtures in tests/golden/ were produced by the reference's own code
(tests/golden/make_golden.py) and by the reference's shipped example-1 run.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def test_discretize_matches_reference_fixture(orc, golden):
    g = golden("discretize_ref.npz")
    for sch_name, sch in (("s30", [30]), ("s2", [50, 7])):
        for typ, name in ((1, "bonds"), (2, "angles"), (3, "torsions")):
            for opt in ((1, 0) if typ == 3 else (1,)):
                bins, ext = orc.discretize(typ, g[name], sch, bins_ref=sch[0], optimize=bool(opt))
                key = f"{name}_{sch_name}_o{opt}"
                assert np.array_equal(bins, g[key + "_bins"]), key
                assert np.array_equal(ext, g[key + "_ext"]), key


def test_entropy_matches_reference_fixture(orc, golden):
    g = golden("entropy_ref.npz")
    sch = g["schemes"].tolist()
    nsteps = int(g["nsteps"])
    ests = g["ests"].tolist()
    for jac in (0, 1):
        s1 = orc.entropy1d(g["types"], g["bins"], g["ext"], nsteps, sch, ests, bool(jac))
        np.testing.assert_allclose(s1, g[f"s1_j{jac}"], rtol=1e-12, atol=0)
        s2 = orc.entropy2d(g["pairs"], g["types"], g["bins"], g["ext"], nsteps, sch, ests,
                           bool(jac))
        np.testing.assert_allclose(s2, g[f"s2_j{jac}"], rtol=1e-12, atol=0)
    kext = np.full((4, 4), 1000.0)
    t3 = np.full(4, 3, np.uint8)
    s1 = orc.entropy1d(t3, g["kde_bins"], kext, nsteps, [3], ests, True, True)
    np.testing.assert_allclose(s1, g["kde_s1"], rtol=1e-12)
    kp = np.array([(i, j) for i in range(4) for j in range(i + 1, 4)], np.uint32)
    s2 = orc.entropy2d(kp, t3, g["kde_bins"], kext, nsteps, [3], ests, True, True)
    np.testing.assert_allclose(s2, g["kde_s2"], rtol=1e-12)


def test_mst_matches_reference_fixture(orc, golden):
    g = golden("mst_ref.npz")
    for k in range(12):
        nv = int(g[f"g{k}_nv"])
        src, dst, w = g[f"g{k}_src"], g[f"g{k}_dst"], g[f"g{k}_w"]
        t = orc.mst(nv, src, dst, w)
        assert np.array_equal(src[t], g[f"g{k}_tsrc"])
        assert np.array_equal(dst[t], g[f"g{k}_tdst"])
        assert np.array_equal(w[t], g[f"g{k}_tw"])


def test_vmkde_matches_reference_fixture(orc, golden):
    g = golden("vmkde_ref.npz")
    t = g["torsions"]
    for kappa in (1.0, 8.0):
        for d in range(len(t)):
            bins, mins, _ = orc.vmkde(t[d], 5, kappa, 5, 1e-4, 1000)
            assert np.array_equal(bins, g[f"k{kappa:g}_d{d}_bins"])
            np.testing.assert_array_equal(mins, g[f"k{kappa:g}_d{d}_minima"])


@pytest.fixture(scope="module")
def ex1():
    d = np.load(os.path.join(GOLDEN, "example1.npz"))
    with open(os.path.join(GOLDEN, "example1.json")) as f:
        meta = json.load(f)
    return d, meta


def test_example1_torsion_entropy_sum(orc, ex1):
    """DIHED-S1 of MIE-ML_convergence_b-30.csv (all 30 torsions are in the
    example's subset) at each of the 4 steps, to the CSV's 4 decimals."""
    d, meta = ex1
    coord, ext = d["torsions_coord"], d["torsions_ext"]
    s1 = orc.entropy1d(np.full(len(coord), 3, np.uint8), coord, ext, 4, [30], [0], True)
    col = meta["mie_columns"].index("DIHED-S1")
    for step in range(4):
        want = meta["mie_rows"][step][col]
        assert abs(s1[:, 0, 0, step].sum() - want) <= 0.5e-4 + 1e-9


def test_example1_tree_edge_mi(orc, ex1):
    """Every edge MI of the shipped Tree-MIST-ML_b-30_s-{0..3}.csv, to 6 dp."""
    d, meta = ex1
    names = {"B": "bonds", "A": "angles", "T": "torsions"}
    tcode = {"B": 1, "A": 2, "T": 3}
    coord = np.concatenate([d[f"{names[k]}_coord"] for k in "BAT"])
    ext = np.concatenate([d[f"{names[k]}_ext"] for k in "BAT"])
    types = np.concatenate([np.full(len(d[f"{names[k]}_coord"]), tcode[k], np.uint8) for k in "BAT"])
    off = {"B": 0, "A": len(d["bonds_coord"]), "T": len(d["bonds_coord"]) + len(d["angles_coord"])}
    s1 = orc.entropy1d(types, coord, ext, 4, [30], [0], True)
    for step in range(4):
        edges = meta["trees"][str(step)]
        pairs = np.array([(off[a] + i, off[b] + j) for a, b, i, j, _ in edges], np.uint32)
        s2 = orc.entropy2d(pairs, types, coord, ext, 4, [30], [0], True)
        mi = s1[pairs[:, 0], 0, 0, step] + s1[pairs[:, 1], 0, 0, step] - s2[:, 0, 0, step]
        want = np.array([e[4] for e in edges])
        assert np.max(np.abs(mi - want)) <= 0.5e-6 + 1e-9


# ---- the reference's own entropy-contribution files of example 1 ---------
BLOCKS2D = (("bnd_2d", "B", "B"), ("ba_2d", "B", "A"), ("bd_2d", "B", "T"),
            ("ang_2d", "A", "A"), ("ad_2d", "A", "T"), ("tor_2d", "T", "T"))


@pytest.fixture(scope="module")
def ex1ent():
    return np.load(os.path.join(GOLDEN, "example1_entcontri.npz"))


def _ex1_arrays(d):
    names = {"B": "bonds", "A": "angles", "T": "torsions"}
    tcode = {"B": 1, "A": 2, "T": 3}
    coord = np.concatenate([d[f"{names[k]}_coord"] for k in "BAT"])
    ext = np.concatenate([d[f"{names[k]}_ext"] for k in "BAT"])
    types = np.concatenate([np.full(len(d[f"{names[k]}_coord"]), tcode[k], np.uint8) for k in "BAT"])
    off = {"B": 0, "A": len(d["bonds_coord"]), "T": len(d["bonds_coord"]) + len(d["angles_coord"])}
    return coord, ext, types, off


def test_example1_entcontri_matches_oracle(orc, ex1, ex1ent):
    """The oracle's 1-D and 2-D entropies of the example's subset DOFs and
    neighbour pairs against the values the reference wrote to its
    entcontri_*.nc files (ML, 30 bins, 4 steps, Jacobian on)."""
    d, _ = ex1
    coord, ext, types, off = _ex1_arrays(d)
    s1 = orc.entropy1d(types, coord, ext, 4, [30], [0], True)
    for f, k in (("bnd_1d", "B"), ("ang_1d", "A"), ("tor_1d", "T")):
        ids = ex1ent[f + "_ids"][:, 0].astype(np.int64)
        np.testing.assert_allclose(s1[off[k] + ids], ex1ent[f + "_contri"], rtol=1e-9, atol=1e-13)
    for f, a, b in BLOCKS2D:
        ids = ex1ent[f + "_ids"].astype(np.int64)
        pairs = np.stack([off[a] + ids[:, 0], off[b] + ids[:, 1]], 1).astype(np.uint32)
        s2 = orc.entropy2d(pairs, types, coord, ext, 4, [30], [0], True)
        np.testing.assert_allclose(s2, ex1ent[f + "_contri"], rtol=1e-9, atol=1e-13)


def test_example1_sums_and_tree_from_reference_entropies(orc, ex1, ex1ent):
    """MIE and MIST rows of the shipped CSVs, and every shipped tree, rebuilt
    from the reference's own entropies: the block sums, MI and the spanning
    tree over the neighbour pairs in the reference's edge order (B/B, B/A,
    B/D, A/A, A/D, D/D)."""
    _, meta = ex1
    s1 = {k: ex1ent[f + "_contri"][:, 0, 0, :] for f, k in (("bnd_1d", "B"), ("ang_1d", "A"),
                                                            ("tor_1d", "T"))}
    id2idx = {k: {int(i): n for n, i in enumerate(ex1ent[f + "_ids"][:, 0])}
              for f, k in (("bnd_1d", "B"), ("ang_1d", "A"), ("tor_1d", "T"))}
    base = {"B": 0, "A": len(s1["B"]), "T": len(s1["B"]) + len(s1["A"])}
    cols = meta["mie_columns"]
    for step in range(4):
        mie = meta["mie_rows"][step]
        mist = meta["mist_rows"][step]
        for k, c in (("B", "BOND-S1"), ("A", "ANGLE-S1"), ("T", "DIHED-S1")):
            assert abs(s1[k][:, step].sum() - mie[cols.index(c)]) <= 0.5e-4 + 1e-9
        src, dst, w, tag = [], [], [], []
        for f, a, b in BLOCKS2D:
            ids = ex1ent[f + "_ids"]
            s2 = ex1ent[f + "_contri"][:, 0, 0, step]
            ia = np.array([id2idx[a][int(x)] for x in ids[:, 0]])
            ib = np.array([id2idx[b][int(x)] for x in ids[:, 1]])
            mi = s1[a][ia, step] + s1[b][ib, step] - s2
            name = {"B": "B", "A": "A", "T": "D"}
            c = f"{name[a]}/{name[b]}"
            assert abs(s2.sum() - mie[cols.index(c + "-S2")]) <= 0.5e-4 + 1e-9
            assert abs(mi.sum() - mie[cols.index(c + "-I2")]) <= 0.5e-4 + 1e-9
            src += list(base[a] + ia)
            dst += list(base[b] + ib)
            w += list(mi)
            tag += [c] * len(mi)
        tree = orc.mst(base["T"] + len(s1["T"]), src, dst, w)
        tot = {c: 0.0 for c in set(tag)}
        for e in tree:
            tot[tag[e]] += w[e]
        for c, v in tot.items():
            assert abs(v - mist[cols.index(c + "-I2")]) <= 0.5e-4 + 1e-9, (step, c)
        inv = {v: (k, i) for k in "BAT" for i, v in ((i, base[k] + n) for i, n in id2idx[k].items())}
        got = sorted((inv[src[e]][0], inv[dst[e]][0], inv[src[e]][1], inv[dst[e]][1]) for e in tree)
        want = sorted((a, b, i, j) for a, b, i, j, _ in meta["trees"][str(step)])
        assert got == want, step


# ------------------------------------------------ histogram dump (ex-2) --
def hist_mids(mn, mx, schemes):
    """binData1D's bin mids (src/Estimators.cpp:67-77): a running offset
    from the minimum, half a bin width added.  The C++ driver writes the same
    expression into hist_*.nc (host/stages.cpp, append_mids)."""
    out = []
    for nb in schemes:
        w = (mx - mn) / nb
        half = w / 2.0
        off = mn
        for _ in range(nb):
            out.append(off + half)
            off += w
    return np.array(out)


def test_hist_dump_golden_mids_and_counts():
    g = np.load(os.path.join(GOLDEN, "hist_tor1d_ref.npz"))
    hdr = json.load(open(os.path.join(GOLDEN, "hist_tor1d_ref.json")))
    atts = {a[0]: a for a in hdr["atts"]}
    schemes = atts["binSchemes"][2]
    nsteps, first, stride = atts["nsteps"][2][0], atts["firstStep"][2][0], atts["stepStride"][2][0]
    assert (first, stride) == (nsteps - 1, 1)       # the default: the last step only
    for r in range(g["id"].shape[0]):
        mn, mx = g["extrema"][r, 0, 0], g["extrema"][r, 0, 1]
        np.testing.assert_array_equal(g["mid"][r], hist_mids(mn, mx, schemes))
    # cumulative counts of the last step: every record counts the same frames
    tot = g["freq"].sum(axis=2)
    assert np.all(tot == tot[0, 0]) and tot[0, 0] > 0
