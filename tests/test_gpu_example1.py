"""The reference's shipped example 1 (33-atom molecule, 10,000 frames, 30
bins, 4 steps, subset + neighbour lists, MIST, ML) end to end on the GPU:
the library's entropies against the reference's own entcontri_*.nc values,
its sums and trees against the shipped CSVs, and the C++ driver run on the
example's bin files against the same CSVs."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN
from centre_gb300 import cdf5
from centre_gb300.api import make_params

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOOL = os.path.join(ROOT, "centre_gb300", "centre_gpu")
BLOCKS2D = (("bnd_2d", "B", "B"), ("ba_2d", "B", "A"), ("bd_2d", "B", "T"),
            ("ang_2d", "A", "A"), ("ad_2d", "A", "T"), ("tor_2d", "T", "T"))
ONED = (("bnd_1d", "B"), ("ang_1d", "A"), ("tor_1d", "T"))
NAMES = {"B": "bonds", "A": "angles", "T": "torsions"}
CODE = {"B": 1, "A": 2, "T": 3}
SUMNAME = {"B": "B", "A": "A", "T": "D"}


@pytest.fixture(scope="module")
def ex():
    d = np.load(os.path.join(GOLDEN, "example1.npz"))
    e = np.load(os.path.join(GOLDEN, "example1_entcontri.npz"))
    with open(os.path.join(GOLDEN, "example1.json")) as f:
        meta = json.load(f)
    return d, e, meta


def subset_arrays(d, e):
    """The example's subset DOFs (bonds, angles, torsions), as the scorer
    orders them, with their bins and extremes."""
    bins, ext, types, index = [], [], [], {}
    for f, k in ONED:
        ids = e[f + "_ids"][:, 0].astype(int)
        for i in ids:
            index[(k, int(i))] = len(types)
            types.append(CODE[k])
        bins.append(d[NAMES[k] + "_coord"][ids])
        ext.append(d[NAMES[k] + "_ext"][ids])
    return (np.ascontiguousarray(np.concatenate(bins)), np.concatenate(ext),
            np.array(types, np.uint8), index)


def test_entropies_match_reference_files(gpu, ex):
    d, e, _ = ex
    bins, ext, types, index = subset_arrays(d, e)
    p = make_params(bins.shape[2], 4, [30], [0], True)
    s1 = gpu.entropy1d(p, types, bins, ext)
    off = 0
    for f, k in ONED:
        n = len(e[f + "_ids"])
        np.testing.assert_allclose(s1[off:off + n], e[f + "_contri"], rtol=1e-9, atol=1e-13)
        off += n
    for f, a, b in BLOCKS2D:
        pairs = np.array([(index[(a, int(i))], index[(b, int(j))]) for i, j in e[f + "_ids"]],
                         np.uint32)
        s2 = gpu.entropy2d(p, types, bins, ext, pairs=pairs)
        np.testing.assert_allclose(s2, e[f + "_contri"], rtol=1e-9, atol=1e-13)


def test_sums_and_trees_match_reference_csv(gpu, ex):
    d, e, meta = ex
    bins, ext, types, index = subset_arrays(d, e)
    p = make_params(bins.shape[2], 4, [30], [0], True)
    s1 = gpu.entropy1d(p, types, bins, ext)
    pairs = np.concatenate([np.array([(index[(a, int(i))], index[(b, int(j))])
                                      for i, j in e[f + "_ids"]], np.uint32)
                            for f, a, b in BLOCKS2D])
    s2 = gpu.entropy2d(p, types, bins, ext, pairs=pairs)
    out = gpu.score(p, types, s1, s2, pairs=pairs)
    cols = meta["mie_columns"][1:]
    inv = {v: k for k, v in index.items()}
    for step in range(4):
        np.testing.assert_allclose(out["mie"][0, 0, step], meta["mie_rows"][step][1:], rtol=0,
                                   atol=0.5e-4 + 1e-9, err_msg=f"MIE step {step} {cols}")
        np.testing.assert_allclose(out["mist"][0, 0, step], meta["mist_rows"][step][1:], rtol=0,
                                   atol=0.5e-4 + 1e-9, err_msg=f"MIST step {step}")
        got = sorted((inv[pairs[q, 0]][0], inv[pairs[q, 1]][0], inv[pairs[q, 0]][1],
                      inv[pairs[q, 1]][1]) for q in out["tree"][step])
        want = sorted((a, b, i, j) for a, b, i, j, _ in meta["trees"][str(step)])
        assert got == want, step


def test_driver_reproduces_reference_outputs(gpu, ex, tmp_path):
    """centre_gpu with the example's input file (subset, neighbours, MIST,
    ML, 30 bins, 4 steps), started from its bin files."""
    d, e, meta = ex
    out = tmp_path / "out"
    out.mkdir()
    for k, c in (("B", "B"), ("A", "A"), ("T", "T")):
        n = NAMES[k]
        cdf5.write_bins(str(out / f"bin_{n}.nc"), c, d[n + "_dimid"], d[n + "_ext"],
                        d[n + "_coord"], [30])
    totals = {"B": len(d["bonds_coord"]), "A": len(d["angles_coord"]), "T": len(d["torsions_coord"])}
    word = {"B": "bond", "A": "angle", "T": "torsion"}
    with open(tmp_path / "subset.txt", "w") as f:
        for fk, k in ONED:
            ids = e[fk + "_ids"][:, 0]
            f.write(f"{word[k]} {totals[k]} {len(ids)} " + " ".join(map(str, ids)) + ";\n")
    kind = {"bnd_2d": "bond", "ang_2d": "angle", "tor_2d": "torsion", "ba_2d": "bacross",
            "bd_2d": "bdcross", "ad_2d": "adcross"}
    with open(tmp_path / "neigh.txt", "w") as f:
        for fk, _, _ in BLOCKS2D:
            groups = {}
            for i, j in e[fk + "_ids"]:
                groups.setdefault(int(i), []).append(int(j))
            for key, part in groups.items():
                f.write(f"{kind[fk]} {key} {len(part)} " + " ".join(map(str, part)) + ";\n")
    cfg = tmp_path / "centre-histogram-inp.cfg"
    cfg.write_text(f"""[control]
    infilepath           = {tmp_path}/
    outfilepath          = {out}/
    infofile             = progress-1.info
    nsteps               = 4
    discretize           = false
    calcentropy          = true
    genconvgdata         = true
[discretization]
    fname                = 0O.lig-s500_dfs_11-8-7_bat.nc
    optimizedih          = true
    pdfmethod            = histogram
[histogram]
    referencenbins       = 30
    nbins                = 30
[entropy]
    workset              = 2D
    usesubset            = true
    useneighbor          = true
    jacobian             = true
    subsetfile           = subset.txt
    neighborfile         = neigh.txt
    scoringmethod        = MIST
    estimator            = ML
""")
    r = subprocess.run([TOOL, "-i", str(cfg)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    for kind_, rows in (("MIE", meta["mie_rows"]), ("MIST", meta["mist_rows"])):
        lines = open(out / f"{kind_}-ML_convergence_b-30.csv").read().splitlines()
        assert [h.strip() for h in lines[0].split(",")] == meta["mie_columns"]
        for step, ln in enumerate(lines[1:]):
            vals = [float(x) for x in ln.split(",")]
            np.testing.assert_allclose(vals, rows[step], rtol=0, atol=0.5e-4 + 1e-9,
                                       err_msg=f"{kind_} step {step}")
    for step in range(4):
        lines = open(out / f"Tree-MIST-ML_b-30_s-{step}.csv").read().splitlines()
        got = sorted((r[0].strip(), r[1].strip(), int(r[2]), int(r[3]))
                     for r in (ln.split(",") for ln in lines[1:]))
        want = sorted((a, b, i, j) for a, b, i, j, _ in meta["trees"][str(step)])
        assert got == want
        mi = sorted(float(r.split(",")[4]) for r in lines[1:])
        np.testing.assert_allclose(mi, sorted(x[4] for x in meta["trees"][str(step)]),
                                   atol=0.5e-6 + 1e-9)
    # the command-line tool's own entropy-contribution files hold the reference's values
    for f, _ in ONED:
        ids, c = cdf5.read_entcontri(str(out / f"entcontri_{f.replace('_', '-')}.nc"))
        assert np.array_equal(ids[:, 0], e[f + "_ids"][:, 0])
        np.testing.assert_allclose(c, e[f + "_contri"], rtol=1e-9, atol=1e-13)
    for f, _, _ in BLOCKS2D:
        ids, c = cdf5.read_entcontri(str(out / f"entcontri_{f.replace('_', '-')}.nc"))
        ref = {(int(i), int(j)): v for (i, j), v in zip(e[f + "_ids"], e[f + "_contri"])}
        assert len(ids) == len(ref)
        for (i, j), v in zip(ids, c):
            np.testing.assert_allclose(v, ref[(int(i), int(j))], rtol=1e-9, atol=1e-13)
