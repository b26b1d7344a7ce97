"""The C++ driver end to end (centre_gpu -i input.cfg): BAT file in, bin
files, entropy-contribution files and convergence / tree CSVs out, as the
reference's Discretizer, EntropyCalculator and EntropyScorer write them.
Every number is checked against the library's own entry points on the same
data (which the parity tests pin to the oracle and the reference): bins and
entropies exactly, CSV sums to their printed digits."""
import os
import subprocess

import numpy as np
import pytest

from centre_gb300 import cdf5
from centre_gb300.api import make_params
from centre_gb300.synth import chain_trajectory

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOOL = os.path.join(ROOT, "centre_gb300", "centre_gpu")
NAMES = {1: "bonds", 2: "angles", 3: "torsions"}
CONTENT = {1: "B", 2: "A", 3: "T"}


def case(tmp_path, tr, body):
    (tmp_path / "out").mkdir(exist_ok=True)
    cdf5.write_bat(str(tmp_path / "traj_bat.nc"), tr.bonds, tr.angles, tr.torsions)
    cfg = tmp_path / "in.cfg"
    cfg.write_text(f"[control]\n    infilepath = {tmp_path}/\n    outfilepath = {tmp_path}/out/\n"
                   + body)
    r = subprocess.run([TOOL, "-i", str(cfg), "-O"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return tmp_path / "out"


def read_csv(path):
    lines = open(path).read().splitlines()
    head = [h.strip() for h in lines[0].split(",")]
    rows = [[c.strip() for c in ln.split(",")] for ln in lines[1:]]
    return head, rows


BODY = """    nsteps = 4
[discretization]
    fname = traj_bat.nc
    optimizedih = true
[histogram]
    referencenbins = 30
    nbins = 30, 20
[entropy]
    workset = 2D
    estimator = ML, MM
    scoringmethod = MIST
"""


def test_pipeline_all_pairs(gpu, tmp_path):
    tr = chain_trajectory(12, 6001, seed=21)
    out = case(tmp_path, tr, BODY)
    sch = [30, 20]
    # --- bin files: the library's bins, written with the reference's layout
    bins_all, ext_all, types = [], [], []
    for typ, blk in tr.blocks():
        b, e = gpu.discretize(typ, blk, sch, bins_ref=30, optimize=True)
        dimid, ext, coord, schemes = cdf5.read_bins(str(out / f"bin_{NAMES[typ]}.nc"))
        assert np.array_equal(coord, b) and np.array_equal(ext, e)
        assert dimid.tolist() == list(range(len(b))) and schemes.tolist() == sch
        ref = tmp_path / f"py_{typ}.nc"
        cdf5.write_bins(str(ref), CONTENT[typ], dimid, e, b, sch)
        assert open(ref, "rb").read() == open(out / f"bin_{NAMES[typ]}.nc", "rb").read()
        bins_all.append(b)
        ext_all.append(e)
        types += [typ] * len(b)
    bins_all, ext_all = np.concatenate(bins_all), np.concatenate(ext_all)
    types = np.array(types, np.uint8)
    n = tr.nframes
    p = make_params(n, 4, sch, [0, 1], True)
    s1 = gpu.entropy1d(p, types, bins_all, ext_all)
    s2 = gpu.entropy2d(p, types, bins_all, ext_all)
    # --- 1-D contributions
    off = {1: 0, 2: int((types == 1).sum()), 3: int((types <= 2).sum())}
    for typ, f in ((1, "bnd"), (2, "ang"), (3, "tor")):
        ids, c = cdf5.read_entcontri(str(out / f"entcontri_{f}-1d.nc"))
        k = int((types == typ).sum())
        assert ids.ravel().tolist() == list(range(k))
        assert np.array_equal(c, s1[off[typ]:off[typ] + k])
    # --- 2-D contributions, record order key-then-partner
    ndof = len(types)
    iu = {(i, j): q for q, (i, j) in enumerate(zip(*np.triu_indices(ndof, 1)))}
    blocks = {}
    for f, tx, ty in (("bnd", 1, 1), ("ang", 2, 2), ("tor", 3, 3), ("ba", 1, 2), ("bd", 1, 3),
                      ("ad", 2, 3)):
        ids, c = cdf5.read_entcontri(str(out / f"entcontri_{f}-2d.nc"))
        gi = [(off[tx] + a, off[ty] + b) for a, b in ids]
        if tx == ty:
            want = [(a, b) for a in range(off[tx], off[tx] + int((types == tx).sum()))
                    for b in range(a + 1, off[tx] + int((types == tx).sum()))]
        else:
            want = [(a, b) for a in range(off[tx], off[tx] + int((types == tx).sum()))
                    for b in range(off[ty], off[ty] + int((types == ty).sum()))]
        assert gi == want
        assert np.array_equal(c, s2[[iu[x] for x in gi]])
        blocks[f] = gi
    # --- scores: pairs in the reference's edge order B/B B/A B/D A/A A/D D/D
    order = blocks["bnd"] + blocks["ba"] + blocks["bd"] + blocks["ang"] + blocks["ad"] + blocks["tor"]
    pairs = np.array(order, np.uint32)
    res = gpu.score(p, types, s1, s2[[iu[x] for x in order]], pairs=pairs)
    step = n // 4
    for e, est in enumerate(("ML", "MM")):
        for s, nb in enumerate(sch):
            for kind in ("MIE", "MIST"):
                head, rows = read_csv(out / f"{kind}-{est}_convergence_b-{nb}.csv")
                assert head[0] == "TIME" and head[-1] == "S2" and len(head) == 18
                sums = res["mie" if kind == "MIE" else "mist"][e, s]
                for t, row in enumerate(rows):
                    assert int(row[0]) == step * (t + 1)
                    assert row[1:] == [f"{v:.4f}" for v in sums[t]], (kind, est, nb, t)
            for t in range(4):
                g = (e * 2 + s) * 4 + t
                head, rows = read_csv(out / f"Tree-MIST-{est}_b-{nb}_s-{t}.csv")
                assert head == ["TD1", "TD2", "IndexDim1", "IndexDim2", "MI"]
                tree = res["tree"][g]
                assert len(rows) == len(tree) == ndof - 1
                tc = "-BAT"
                for row, q in zip(rows, tree):
                    a, b = order[q]
                    assert row[0] == tc[types[a]] and row[1] == tc[types[b]]
                    assert int(row[2]) == a - off[types[a]] and int(row[3]) == b - off[types[b]]
                    assert row[4] == f"{res['mi'][q].reshape(-1)[g]:.6f}"


def test_pipeline_multiple_bat_files(gpu, tmp_path):
    """Several BAT files listed in discretization.fname are read in order and
    their frames concatenated (src/Inputs.cpp:555-625): a trajectory split
    into two files gives the same bin files, entropy contributions and CSVs,
    byte for byte, as the whole trajectory in one file."""
    tr = chain_trajectory(10, 6001, seed=31)
    body = BODY.replace("fname = traj_bat.nc", "fname = part1_bat.nc, part2_bat.nc")
    single = tmp_path / "single"
    single.mkdir()
    out1 = case(single, tr, BODY)
    split = tmp_path / "split"
    split.mkdir()
    (split / "out").mkdir()
    cut = 2500
    cdf5.write_bat(str(split / "part1_bat.nc"), tr.bonds[:, :cut], tr.angles[:, :cut],
                   tr.torsions[:, :cut])
    cdf5.write_bat(str(split / "part2_bat.nc"), tr.bonds[:, cut:], tr.angles[:, cut:],
                   tr.torsions[:, cut:])
    cfg = split / "in.cfg"
    cfg.write_text(f"[control]\n    infilepath = {split}/\n    outfilepath = {split}/out/\n" + body)
    r = subprocess.run([TOOL, "-i", str(cfg), "-O"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out2 = split / "out"
    names = sorted(f for f in os.listdir(out1) if f.endswith((".nc", ".csv")))
    assert any(f.startswith("bin_") for f in names) and any(f.startswith("entcontri_") for f in names)
    assert any(f.startswith("MIST-") for f in names)
    assert names == sorted(f for f in os.listdir(out2) if f.endswith((".nc", ".csv")))
    for f in names:
        assert open(out1 / f, "rb").read() == open(out2 / f, "rb").read(), f


def test_pipeline_subset_neighbours_and_frames(gpu, tmp_path):
    tr = chain_trajectory(11, 5003, seed=22)
    (tmp_path / "sub.txt").write_text("bond 10 3 0 2 5;\nangle 9 2 1 4;\ntorsion 8 4 0 1 2 6;\n")
    (tmp_path / "neigh.txt").write_text("bond 5 1 0;\nbond 0 2 2 5;\ntorsion 6 2 0 1;\n"
                                        "bacross 0 1 4;\nadcross 4 2 6 0;\nbdcross 2 1 1;\n")
    body = """    nsteps = 3
[discretization]
    fname = traj_bat.nc
[histogram]
    nbins = 24
[entropy]
    workset = 2D
    estimator = ML
    usesubset = true
    useneighbor = true
    subsetfile = sub.txt
    neighborfile = neigh.txt
    startframe = 7
    strideframe = 2
    nframe = 4800
    scoringmethod = MIE
"""
    out = case(tmp_path, tr, body)
    n_eff = (4800 - 7 + 2 - 1) // 2
    full = {}
    for typ, blk in tr.blocks():
        b, e = gpu.discretize(typ, blk, [24], bins_ref=24, optimize=True)
        full[typ] = (b[:, :, 7::2][:, :, :n_eff], e)
    # array order: subset ids, then other ids a pair list names
    order = {1: [0, 2, 5], 2: [1, 4], 3: [0, 1, 2, 6]}
    types = np.array(sum([[t] * len(order[t]) for t in (1, 2, 3)], []), np.uint8)
    bins = np.concatenate([full[t][0][order[t]] for t in (1, 2, 3)])
    ext = np.concatenate([full[t][1][order[t]] for t in (1, 2, 3)])
    index = {}
    for t in (1, 2, 3):
        for k, i in enumerate(order[t]):
            index[(t, i)] = len(index)
    p = make_params(n_eff, 3, [24], [0], True)
    s1 = gpu.entropy1d(p, types, np.ascontiguousarray(bins), ext)
    for typ, f in ((1, "bnd"), (2, "ang"), (3, "tor")):
        ids, c = cdf5.read_entcontri(str(out / f"entcontri_{f}-1d.nc"))
        assert ids.ravel().tolist() == order[typ]
        assert np.array_equal(c, s1[[index[(typ, i)] for i in order[typ]]])
    want = {"bnd": [(0, 2), (0, 5), (5, 0)], "tor": [(6, 0), (6, 1)], "ba": [(0, 4)],
            "bd": [(2, 1)], "ad": [(4, 6), (4, 0)], "ang": []}
    tys = {"bnd": (1, 1), "tor": (3, 3), "ba": (1, 2), "bd": (1, 3), "ad": (2, 3), "ang": (2, 2)}
    for f, recs in want.items():
        ids, c = cdf5.read_entcontri(str(out / f"entcontri_{f}-2d.nc"))
        assert [tuple(r) for r in ids] == recs, f
        if not recs:
            continue
        tx, ty = tys[f]
        pr = np.array([(index[(tx, a)], index[(ty, b)]) for a, b in recs], np.uint32)
        s2 = gpu.entropy2d(p, types, np.ascontiguousarray(bins), ext, pairs=pr)
        assert np.array_equal(c, s2), f
    head, rows = read_csv(out / "MIE-ML_convergence_b-24.csv")
    assert [int(r[0]) for r in rows] == [n_eff // 3 * (k + 1) for k in range(3)]
    assert not os.path.exists(out / "MIST-ML_convergence_b-24.csv")


def test_pipeline_vonmises_kde(gpu, tmp_path):
    tr = chain_trajectory(9, 4000, seed=23)
    body = """    nsteps = 2
[discretization]
    fname = traj_bat.nc
    pdfmethod = vonMisesKDE
[vonmiseskde]
    nmaxconf = 3
    kappa = 1.0
    sdosteps = 5
    sdoiterations = 1000
    sdoconvlimit = 0.0001
[entropy]
    workset = D1D, DD2D
    estimator = ML
    scoringmethod = MIST
"""
    out = case(tmp_path, tr, body)
    b, minima, nfound = gpu.discretize_vmkde(tr.torsions, 3, 1.0, 5, 1e-4, 1000)
    dimid, ext, coord, sch = cdf5.read_bins(str(out / "bin_torsions.nc"))
    assert np.array_equal(coord, b) and sch.tolist() == [3]
    assert np.all(ext == 1000.0)
    assert not os.path.exists(out / "bin_bonds.nc")
    lines = open(out / "vmkde_torsions_minimas.out").read().splitlines()
    assert len(lines) == tr.torsions.shape[0]
    for d, ln in enumerate(lines):
        f = ln.rstrip(";").split()
        assert f[0] == "torsion" and int(f[1]) == d and int(f[2]) == nfound[d]
        assert [float(x) for x in f[3:]] == pytest.approx(minima[d, : nfound[d]], abs=1e-8)
    assert os.path.exists(out / "Tree-MIST-ML_b-3_s-1.csv")


def test_pipeline_learned_neighbours(gpu, tmp_path):
    """--learned-neighbours K: the pair screen replaces the neighbour file;
    its lists are written in the reference's neighbour-file grammar, the
    entropy files hold exactly those pairs, and A-MIST stays close to the
    all-pairs MIST of the same trajectory."""
    tr = chain_trajectory(40, 20000, seed=31, coupling="block8")
    body = """    nsteps = 4
[discretization]
    fname = traj_bat.nc
[histogram]
    nbins = 30
[entropy]
    workset = 2D
    estimator = ML
    scoringmethod = MIST
"""
    (tmp_path / "full").mkdir()
    full_dir = case(tmp_path / "full", tr, body)
    learned = tmp_path / "learned"
    learned.mkdir()
    (learned / "out").mkdir()
    cdf5.write_bat(str(learned / "traj_bat.nc"), tr.bonds, tr.angles, tr.torsions)
    cfg = learned / "in.cfg"
    cfg.write_text(f"[control]\n    infilepath = {learned}/\n    outfilepath = {learned}/out/\n"
                   + body)
    r = subprocess.run([TOOL, "-i", str(cfg), "-O", "--learned-neighbours", "12"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = learned / "out"
    # neighbour file grammar: "<kind> <key> <n> ids...;"
    lists = {}
    for chunk in open(out / "neigh_learned.txt").read().split(";"):
        f = chunk.split()
        if not f:
            continue
        kind, key, n = f[0], int(f[1]), int(f[2])
        assert len(f) == 3 + n
        lists.setdefault(kind, []).extend((key, int(v)) for v in f[3:])
    files = {"bond": "bnd", "angle": "ang", "torsion": "tor", "bacross": "ba", "bdcross": "bd",
             "adcross": "ad"}
    total = 0
    for kind, f in files.items():
        ids, _ = cdf5.read_entcontri(str(out / f"entcontri_{f}-2d.nc"))
        assert [tuple(x) for x in ids] == lists.get(kind, [])
        total += len(ids)
    ndof = 3 * 40 - 6
    assert 0 < total <= ndof * 12
    _, rows_full = read_csv(full_dir / "MIST-ML_convergence_b-30.csv")
    _, rows_learn = read_csv(out / "MIST-ML_convergence_b-30.csv")
    s_full, s_learn = float(rows_full[-1][-1]), float(rows_learn[-1][-1])
    assert abs(s_learn - s_full) <= 0.01 * abs(s_full)


def test_pipeline_histogram_dumps(gpu, tmp_path):
    """[histogram] writefreq: hist_*.nc with the reference's header layout
    (pinned by its own example-2 dump) and the counts of the written steps."""
    import json
    from conftest import GOLDEN
    tr = chain_trajectory(8, 4003, seed=31)
    body = BODY.replace("    nbins = 30, 20\n",
                        "    nbins = 30, 20\n    writefreq = true\n"
                        "    writeset = B1D, A1D, D1D, BB2D, AA2D, DD2D, BA2D, BD2D, AD2D\n"
                        "    writestepstart = 1\n    writestepstride = 2\n")
    out = case(tmp_path, tr, body)
    ref = json.load(open(os.path.join(GOLDEN, "hist_tor1d_ref.json")))
    sch = [30, 20]
    n = tr.nframes
    step = n // 4
    steps = [1, 3]                                   # first 1, stride 2 of 4 steps
    bins, ext = {}, {}
    for typ in (1, 2, 3):
        _, e, c, _ = cdf5.read_bins(str(out / f"bin_{NAMES[typ]}.nc"))
        bins[typ], ext[typ] = c, e

    def mids1(e, nb):
        # binData1D's running offset (src/Estimators.cpp:67-77)
        m = []
        w = (e[1] - e[0]) / nb
        half, off = w / 2.0, e[0]
        for _ in range(nb):
            m.append(off + half)
            off += w
        return m

    def mids(e):
        return np.array(sum((mids1(e, nb) for nb in sch), []))

    def check_header(ds, content, ndims, storage, dim_lens):
        # attribute names, order and types as the reference writes them
        got = [(k, "text" if isinstance(v, str) else v.dtype.newbyteorder("=").name)
               for k, v in ds.attrs.items()]
        assert got == [(a[0], a[1]) for a in ref["atts"]]
        for a in ref["atts"]:
            if a[0] in ("appication", "program", "programVersion", "convention",
                        "conventionVersion"):
                assert ds.attrs[a[0]] == a[2]
        assert ds.attrs["content"] == content
        assert ds.attrs["title"].tolist() == [1 if storage else 0]
        assert ds.attrs["order"].tolist() == [ndims] and ds.attrs["ndims"].tolist() == [ndims]
        assert ds.attrs["firstStep"].tolist() == [1] and ds.attrs["stepStride"].tolist() == [2]
        assert ds.attrs["nsteps"].tolist() == [4]
        assert ds.attrs["storagetype"].tolist() == [storage]
        assert ds.attrs["dimLengths"].tolist() == dim_lens
        assert ds.attrs["binSchemes"].tolist() == sch
        assert list(ds.dims) == [d[0] for d in ref["dims"]]
        assert [[v.name, list(v.dims), v.nctype] for v in ds.vars.values()] == ref["vars"]

    # --- 1-D
    for typ, f, content in ((1, "bnd", "B"), (2, "ang", "A"), (3, "tor", "D")):
        ds = cdf5.read(str(out / f"hist_{f}-1d.nc"))
        k = bins[typ].shape[0]
        check_header(ds, content, 1, 0, [k])
        assert ds.vars["id"].data.ravel().tolist() == list(range(k))
        np.testing.assert_array_equal(ds.vars["extrema"].data[:, 0], ext[typ])
        fr = ds.vars["freq"].data
        for r in range(k):
            np.testing.assert_array_equal(ds.vars["mid"].data[r], mids(ext[typ][r]))
            for si, t in enumerate(steps):
                want = np.concatenate([np.bincount(bins[typ][r, s, :(t + 1) * step], minlength=nb)
                                       for s, nb in enumerate(sch)])
                np.testing.assert_array_equal(fr[r, si], want)
    # --- 2-D
    for f, tx, ty, content in (("bnd", 1, 1, "B/B"), ("ang", 2, 2, "A/A"), ("tor", 3, 3, "D/D"),
                               ("ba", 1, 2, "B/A"), ("bd", 1, 3, "B/D"), ("ad", 2, 3, "A/D")):
        ds = cdf5.read(str(out / f"hist_{f}-2d.nc"))
        kx, ky = bins[tx].shape[0], bins[ty].shape[0]
        check_header(ds, content, 2, 0 if tx == ty else 3, [kx, ky])
        ids = ds.vars["id"].data
        eids, _ = cdf5.read_entcontri(str(out / f"entcontri_{f}-2d.nc"))
        assert np.array_equal(ids, eids)
        fr = ds.vars["freq"].data
        for r in range(0, ids.shape[0], max(1, ids.shape[0] // 7)):
            a, b = ids[r]
            np.testing.assert_array_equal(ds.vars["extrema"].data[r, 0], ext[tx][a])
            np.testing.assert_array_equal(ds.vars["extrema"].data[r, 1], ext[ty][b])
            # per scheme: the first DOF's mids, then the second's (binData2D)
            m = sum((mids1(ext[tx][a], nb) + mids1(ext[ty][b], nb) for nb in sch), [])
            np.testing.assert_array_equal(ds.vars["mid"].data[r], np.array(m))
            for si, t in enumerate(steps):
                want = []
                for s, nb in enumerate(sch):
                    x = bins[tx][a, s, :(t + 1) * step].astype(np.int64)
                    y = bins[ty][b, s, :(t + 1) * step].astype(np.int64)
                    want.append(np.bincount(x * nb + y, minlength=nb * nb))
                np.testing.assert_array_equal(fr[r, si], np.concatenate(want))
