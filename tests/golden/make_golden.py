"""Generate the golden fixtures in this directory from the reference itself.

Run where the reference sources (shaileshp51/centre) are checked out, with
CENTRE_REFERENCE_ROOT naming that checkout:

    CENTRE_REFERENCE_ROOT=<checkout> python tests/golden/make_golden.py

It builds oracle/_ref/libcentre_ref.so from the reference's own numeric
sources (oracle/Makefile), runs the reference functions on seeded inputs, and
stores inputs and outputs:

  discretize_ref.npz  Real2Int::{bnd,ang,dih}Real2Int (src/Real2Int.cpp:27-479)
  entropy_ref.npz     binData1D/2D + entropy1D/2D, every estimator
                      (src/Estimators.cpp:56-651)
  mst_ref.npz         boruvkaMST on graphs with ties and disconnected parts
                      (src/Centre.cpp:5-143)
  vmkde_ref.npz       Real2Int::getMinimaPositions (src/Real2Int.cpp:481-716)
  example1.npz/.json  the bin files and expected CSV values shipped in the
                      reference's test_examples/example-1/outfiles-h-ref
  example1_entcontri.npz  the DOF/pair ids and contri_S entropies of that
                      example's entcontri_*.nc files (HDF5, read with
                      hdf5_min.py): the reference's own 1-D and 2-D entropies
                      of the subset DOFs and neighbour pairs

  hist_tor1d_ref.json/.npz  header and first records of the reference's
                      histogram dump test_examples/example-2/outfiles-h-ref/
                      hist_tor-1d.nc
  example1_binfiles.json  SHA-256 and size of example-1's bin_*.nc files, so
                      the bin-file writer is checked byte for byte without
                      the reference checkout

    python tests/golden/make_golden.py example1     # only the example-1 fixtures
    python tests/golden/make_golden.py binhash      # only the bin-file hashes
    python tests/golden/make_golden.py hist         # only the histogram-dump fixture
"""
from __future__ import annotations

import csv
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from centre_gb300 import cdf5  # noqa: E402

REF = os.environ.get("CENTRE_REFERENCE_ROOT", "")


def dof_inputs(seed=7, n=4000):
    """Small DOF blocks covering the discretiser's branches."""
    rng = np.random.default_rng(seed)
    two_pi = 2 * np.pi
    bonds = [rng.normal(1.5, 0.03, n), rng.normal(1.09, 0.01, n), rng.uniform(0.9, 2.1, n),
             np.full(n, 1.52) + rng.normal(0, 1e-7, n),      # range < 1e-4 (+0.05 branch)
             np.abs(rng.normal(0.0, 1e-9, n))]                # min - dx clamps to 0
    angles = [rng.normal(1.91, 0.08, n), rng.normal(2.0, 0.02, n), rng.uniform(0.01, 3.13, n),
              np.full(n, 1.8) + rng.normal(0, 1e-7, n),
              rng.uniform(3.0, np.pi - 1e-6, n)]              # max + dx clamps to pi
    tors = [np.mod(rng.vonmises(np.pi, 8, n), two_pi),       # centred at pi
            np.mod(rng.vonmises(0.0, 8, n), two_pi),         # straddles 0 / 2pi
            np.mod(rng.vonmises(0.05, 30, n), two_pi),       # narrow near 0
            np.mod(rng.vonmises(-0.05, 30, n), two_pi),      # narrow near 2pi
            rng.uniform(0, two_pi, n),                        # no empty coarse bin
            np.mod(np.where(rng.random(n) < 0.5, rng.vonmises(-np.pi / 3, 8, n),
                            rng.vonmises(np.pi / 3, 8, n)), two_pi),
            np.mod(rng.vonmises(2.0, 200, n), two_pi),        # very narrow
            np.mod(np.where(rng.random(n) < 0.4, rng.vonmises(-np.pi / 3, 8, n),
                            np.where(rng.random(n) < 0.5, rng.vonmises(np.pi / 3, 8, n),
                                     rng.vonmises(np.pi, 8, n))), two_pi)]
    f = lambda L: np.ascontiguousarray(np.array(L, dtype=np.float32))
    t = f(tors)
    t[t >= np.float32(two_pi)] = 0
    return f(bonds), f(angles), t


def make_discretize(R):
    b, a, t = dof_inputs()
    out = {"bonds": b, "angles": a, "torsions": t}
    for sch_name, sch in (("s30", [30]), ("s2", [50, 7])):
        for typ, name, data in ((1, "bonds", b), (2, "angles", a), (3, "torsions", t)):
            for opt in ((1, 0) if typ == 3 else (1,)):
                bins, ext = R.discretize(typ, data, sch, bins_ref=sch[0], optimize=bool(opt))
                out[f"{name}_{sch_name}_o{opt}_bins"] = bins
                out[f"{name}_{sch_name}_o{opt}_ext"] = ext
    np.savez_compressed(os.path.join(HERE, "discretize_ref.npz"), **out)
    return out


def make_entropy(R, disc):
    sch = [50, 7]
    bins = np.concatenate([disc["bonds_s2_o1_bins"], disc["angles_s2_o1_bins"],
                           disc["torsions_s2_o1_bins"]])
    ext = np.concatenate([disc["bonds_s2_o1_ext"], disc["angles_s2_o1_ext"],
                          disc["torsions_s2_o1_ext"]])
    types = np.array([1] * 5 + [2] * 5 + [3] * 8, np.uint8)
    nsteps = 4
    ests = [0, 1, 2, 3]
    out = {"bins": bins, "ext": ext, "types": types, "schemes": np.array(sch, np.uint8),
           "nsteps": np.array(nsteps), "ests": np.array(ests, np.uint8)}
    for jac in (0, 1):
        out[f"s1_j{jac}"] = np.stack([R.entropy1d(int(types[d]), bins[d], ext[d, 0], ext[d, 1],
                                                  nsteps, sch, ests, bool(jac))
                                      for d in range(len(bins))])
    pairs = np.array([(i, j) for i in range(len(bins)) for j in range(i + 1, len(bins))],
                     np.uint32)
    out["pairs"] = pairs
    for jac in (0, 1):
        out[f"s2_j{jac}"] = np.stack([R.entropy2d(int(types[i]), int(types[j]), bins[i], bins[j],
                                                  ext[i], ext[j], nsteps, sch, ests, bool(jac))
                                      for i, j in pairs])
    # KDE-mode entropies (width 1, no Jacobian effect) on 3-state bins
    rng = np.random.default_rng(3)
    kb = rng.integers(0, 3, size=(4, 1, 4000)).astype(np.uint8)
    kext = np.full((4, 4), 1000.0)
    out["kde_bins"] = kb
    out["kde_s1"] = np.stack([R.entropy1d(3, kb[d], 1000.0, 1000.0, nsteps, [3], ests, True, True)
                              for d in range(4)])
    kp = np.array([(i, j) for i in range(4) for j in range(i + 1, 4)], np.uint32)
    out["kde_s2"] = np.stack([R.entropy2d(3, 3, kb[i], kb[j], kext[i], kext[j], nsteps, [3], ests,
                                          True, True) for i, j in kp])
    np.savez_compressed(os.path.join(HERE, "entropy_ref.npz"), **out)


def make_mst(R):
    rng = np.random.default_rng(11)
    out = {}
    for g in range(12):
        nv = int(rng.integers(3, 40))
        dense = g % 3 != 2
        E = [(i, j) for i in range(nv) for j in range(i + 1, nv) if dense or rng.random() < 0.15]
        src = np.array([e[0] for e in E], np.uint32)
        dst = np.array([e[1] for e in E], np.uint32)
        if g % 2:
            w = rng.integers(0, 4, len(E)).astype(np.float64) * 0.25   # many ties
        else:
            w = rng.random(len(E))
        ts, td, tw = R.mst(nv, src, dst, w)
        out[f"g{g}_nv"] = np.array(nv)
        out[f"g{g}_src"], out[f"g{g}_dst"], out[f"g{g}_w"] = src, dst, w
        out[f"g{g}_tsrc"], out[f"g{g}_tdst"], out[f"g{g}_tw"] = ts, td, tw
    np.savez_compressed(os.path.join(HERE, "mst_ref.npz"), **out)


def make_vmkde(R):
    _, _, t = dof_inputs(seed=19, n=3000)
    out = {"torsions": t}
    for kappa in (1.0, 8.0):
        for d in range(len(t)):
            bins, mins, found = R.vmkde(t[d], 5, kappa, 5, 1e-4, 1000)
            out[f"k{kappa:g}_d{d}_bins"] = bins
            out[f"k{kappa:g}_d{d}_minima"] = mins
    np.savez_compressed(os.path.join(HERE, "vmkde_ref.npz"), **out)


def make_example1():
    base = os.path.join(REF, "test_examples", "example-1", "outfiles-h-ref")
    out, meta = {}, {}
    for t in ("bonds", "angles", "torsions"):
        dimid, ext, coord, sch = cdf5.read_bins(os.path.join(base, f"bin_{t}.nc"))
        out[f"{t}_dimid"], out[f"{t}_ext"], out[f"{t}_coord"] = dimid, ext, coord
        meta["schemes"] = sch.tolist()
    with open(os.path.join(base, "MIE-ML_convergence_b-30.csv")) as f:
        rows = list(csv.reader(f))
    head = [h.strip() for h in rows[0]]
    meta["mie_columns"] = head
    meta["mie_rows"] = [[float(x) for x in r] for r in rows[1:] if r]
    with open(os.path.join(base, "MIST-ML_convergence_b-30.csv")) as f:
        rows = list(csv.reader(f))
    meta["mist_rows"] = [[float(x) for x in r] for r in rows[1:] if r]
    trees = {}
    for s in range(4):
        with open(os.path.join(base, f"Tree-MIST-ML_b-30_s-{s}.csv")) as f:
            rr = list(csv.reader(f))
        trees[str(s)] = [[r[0].strip(), r[1].strip(), int(r[2]), int(r[3]), float(r[4])]
                         for r in rr[1:] if r]
    meta["trees"] = trees
    meta["nsteps"] = 4
    meta["source"] = "test_examples/example-1/outfiles-h-ref (shaileshp51/centre)"
    np.savez_compressed(os.path.join(HERE, "example1.npz"), **out)
    with open(os.path.join(HERE, "example1.json"), "w") as f:
        json.dump(meta, f, indent=1)
    sys.path.insert(0, HERE)
    import hdf5_min
    ent = {}
    for f in ("bnd-1d", "ang-1d", "tor-1d", "bnd-2d", "ang-2d", "tor-2d", "ba-2d", "bd-2d", "ad-2d"):
        ids, contri = hdf5_min.read_entcontri(os.path.join(base, f"entcontri_{f}.nc"))
        key = f.replace("-", "_")
        ent[f"{key}_ids"], ent[f"{key}_contri"] = ids, contri
    np.savez_compressed(os.path.join(HERE, "example1_entcontri.npz"), **ent)


def make_bin_hashes():
    import hashlib
    base = os.path.join(REF, "test_examples", "example-1", "outfiles-h-ref")
    out = {}
    for t in ("bonds", "angles", "torsions"):
        with open(os.path.join(base, f"bin_{t}.nc"), "rb") as f:
            raw = f.read()
        out[t] = {"sha256": hashlib.sha256(raw).hexdigest(), "bytes": len(raw)}
    out["source"] = "test_examples/example-1/outfiles-h-ref/bin_*.nc (shaileshp51/centre)"
    with open(os.path.join(HERE, "example1_binfiles.json"), "w") as f:
        json.dump(out, f, indent=1)


def make_hist():
    """Header and first records of the reference's histogram dump
    test_examples/example-2/outfiles-h-ref/hist_tor-1d.nc (CDF-5, written by
    Netcdf_HistUtil, src/Netcdf_HistUtils.cpp:804-1029): attribute names,
    types and values in file order, dimensions, variables, and the id,
    extrema, mid and freq of the first 16 records."""
    from centre_gb300 import cdf5
    path = os.path.join(REF, "test_examples", "example-2", "outfiles-h-ref", "hist_tor-1d.nc")
    ds = cdf5.read(path)
    atts = []
    for k, v in ds.attrs.items():
        if isinstance(v, str):
            atts.append([k, "text", v])
        else:
            atts.append([k, str(v.dtype.newbyteorder("=").name), [int(x) for x in v]])
    out = {"version": int(ds.version), "numrecs": int(ds.numrecs), "atts": atts,
           "dims": [[k, int(n)] for k, n in ds.dims.items()],
           "vars": [[v.name, list(v.dims), int(v.nctype)] for v in ds.vars.values()]}
    with open(os.path.join(HERE, "hist_tor1d_ref.json"), "w") as f:
        json.dump(out, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "hist_tor1d_ref.npz"),
                        id=ds.vars["id"].data[:16], extrema=ds.vars["extrema"].data[:16],
                        mid=ds.vars["mid"].data[:16], freq=ds.vars["freq"].data[:16])


if __name__ == "__main__":
    if not REF or not os.path.isdir(os.path.join(REF, "src")):
        sys.exit("set CENTRE_REFERENCE_ROOT to the reference checkout")
    if sys.argv[1:] == ["example1"]:
        make_example1()
        sys.exit(0)
    if sys.argv[1:] == ["hist"]:
        make_hist()
        sys.exit(0)
    if sys.argv[1:] == ["binhash"]:
        make_bin_hashes()
        sys.exit(0)
    oracle.build(with_ref=True)
    R = oracle.Reference()
    disc = make_discretize(R)
    make_entropy(R, disc)
    make_mst(R)
    make_vmkde(R)
    make_example1()
    make_bin_hashes()
    make_hist()
    print("fixtures written to", HERE)
