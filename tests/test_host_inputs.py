"""The C++ driver's input handling (centre_gpu --print-inputs), no GPU needed:
the reference's input-file tokenisation and defaults (src/Inputs.cpp:12-1060,
src/Utils.cpp:198-270), BAT headers, subset and neighbour files
(src/Centre.cpp:206-593), the frame selection and the overwrite guard."""
import os
import subprocess

import numpy as np
import pytest

from centre_gb300 import cdf5
from centre_gb300.synth import chain_trajectory

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOOL = os.path.join(ROOT, "centre_gb300", "centre_gpu")


@pytest.fixture(scope="module")
def tool():
    from centre_gb300 import build as B
    B.build()
    return TOOL


def run(tool, cfg, *extra):
    r = subprocess.run([tool, "-i", str(cfg), "--print-inputs", *extra], capture_output=True,
                       text=True)
    kv = {}
    for line in r.stdout.splitlines():
        if " = " in line:
            k, v = line.split(" = ", 1)
            kv[k] = v
    return r.returncode, kv, r.stderr


def setup_case(tmp_path, natoms=8, nframes=3000, body=""):
    tr = chain_trajectory(natoms, nframes, seed=1)
    (tmp_path / "out").mkdir(exist_ok=True)
    cdf5.write_bat(str(tmp_path / "traj_bat.nc"), tr.bonds, tr.angles, tr.torsions)
    cfg = tmp_path / "in.cfg"
    cfg.write_text(f"[control]\n    infilepath = {tmp_path}/\n    outfilepath = {tmp_path}/out/\n"
                   + body)
    return cfg


def test_defaults_and_tokenisation(tool, tmp_path):
    cfg = setup_case(tmp_path, body="""
# a comment line
[discretization]
    fname       = traj_bat.nc     # inline comment
    optimizedih = FALSE
[histogram]
    nbins       = 30, 20,7
[entropy]
    estimator   = ML, JS
    reportfileext = "dat"
""")
    rc, kv, err = run(tool, cfg)
    assert rc == 0, err
    assert kv["control.nsteps"] == "20"                   # reference default
    assert kv["discretization.optimizedih"] == "0"
    assert kv["discretization.nbond"] == "7" and kv["discretization.ndihed"] == "5"
    assert kv["discretization.nframe"] == "3000"
    # "20,7" is one token whose commas are trimmed only at its ends -> atoi("20,7") = 20
    assert kv["histogram.nbins"] == "30 20"
    assert kv["histogram.referencenbins"] == "30"
    assert kv["entropy.estimator"] == "ML JS"
    assert kv["entropy.reportfileext"] == "dat"
    assert kv["entropy.workset"] == "511"
    assert kv["entropy.scoringmethod"] == "MIST"
    # all pairs of 7 bonds, 6 angles, 5 torsions: BB AA DD BA BD AD
    assert kv["neighbours.pairs"] == "21 15 10 42 35 30"


def test_default_estimator_and_frame_selection(tool, tmp_path):
    cfg = setup_case(tmp_path, body="""
    nsteps = 5
[discretization]
    fname = traj_bat.nc
[histogram]
    nbins = 25
[entropy]
    workset = D1D, DD2D
    startframe = 100
    strideframe = 3
    nframe = 2000
""")
    rc, kv, err = run(tool, cfg)
    assert rc == 0, err
    assert kv["entropy.estimator"] == "MM"                # no estimator given
    assert kv["entropy.nframes_eff"] == str((2000 - 100 + 3 - 1) // 3)
    assert kv["entropy.workset"] == "36"
    assert kv["subset.sizes"] == "0 0 5"
    assert kv["neighbours.pairs"] == "0 0 10 0 0 0"


def test_vonmises_kde_adjustments(tool, tmp_path):
    cfg = setup_case(tmp_path, body="""
[discretization]
    fname = traj_bat.nc
    pdfmethod = vonMisesKDE
[vonmiseskde]
    nmaxconf = 3
    kappa = 1.5
[entropy]
    workset = 2D
""")
    rc, kv, err = run(tool, cfg)
    assert rc == 0, err
    assert kv["histogram.nbins"] == "3" and kv["histogram.referencenbins"] == "3"
    assert kv["entropy.workset"] == str(4 | 32)            # torsions only
    assert kv["vonmiseskde.kappa"] == "1.5"


def test_subset_and_neighbour_files(tool, tmp_path):
    cfg = setup_case(tmp_path, natoms=10, body="""
[discretization]
    fname = traj_bat.nc
[histogram]
    nbins = 30
[entropy]
    workset = 2D
    usesubset = true
    useneighbor = true
    subsetfile = sub.txt
    neighborfile = neigh.txt
""")
    (tmp_path / "sub.txt").write_text("#comment;\nbond 9 3 0 2 5;\nangle 8 2 1 4;\n"
                                      "torsion 7 4 0 1 2 6;\n")
    (tmp_path / "neigh.txt").write_text("bond 0 2 2 5;\nbond 2 1 5;\ntorsion 6 2 0 1;\n"
                                        "bacross 0 1 4;\nadcross 4 2 0 6;\nbdcross 5 0;\n")
    rc, kv, err = run(tool, cfg)
    assert rc == 0, err
    assert kv["subset.sizes"] == "3 2 4"
    assert kv["neighbours.pairs"] == "3 0 2 1 0 2"


def test_missing_inputs_fail_with_status(tool, tmp_path):
    cfg = setup_case(tmp_path, body="""
[discretization]
    fname = nothere_bat.nc
[histogram]
    nbins = 30
""")
    rc, kv, err = run(tool, cfg)
    assert rc != 0 and "nothere_bat.nc" in err
    cfg2 = setup_case(tmp_path, body="""
[discretization]
    fname = traj_bat.nc
[histogram]
    nbins = 30
[entropy]
    usesubset = true
    subsetfile = none.txt
""")
    rc, kv, err = run(tool, cfg2)
    assert rc != 0 and "none.txt" in err


def test_existing_outputs_need_overwrite_flag(tool, tmp_path):
    cfg = setup_case(tmp_path, body="""
[discretization]
    fname = traj_bat.nc
[histogram]
    nbins = 30
""")
    (tmp_path / "out" / "bin_bonds.nc").write_bytes(b"x")
    r = subprocess.run([tool, "-i", str(cfg)], capture_output=True, text=True)
    assert r.returncode == 3 and "already exists" in r.stderr
    assert (tmp_path / "out" / "bin_bonds.nc").read_bytes() == b"x"


def test_bat_file_roundtrip(tmp_path):
    tr = chain_trajectory(6, 500, seed=2)
    p = tmp_path / "t.nc"
    cdf5.write_bat(str(p), tr.bonds, tr.angles, tr.torsions)
    ds = cdf5.read(str(p))
    assert ds.attrs["convention"] == "CENTRE"
    assert np.array_equal(ds.vars["bond"].data.T, tr.bonds)
    assert np.array_equal(ds.vars["dihedral"].data.T, tr.torsions)
