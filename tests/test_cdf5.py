"""CDF5 (NetCDF classic) reader/writer against the reference's bin files."""
import os

import numpy as np
import pytest

from centre_gb300 import cdf5
from conftest import GOLDEN

# the reference checkout's example-1 output files (set CENTRE_REFERENCE_ROOT
# to run the byte-for-byte comparison; the fixtures cover the rest)
REFDIR = os.path.join(os.environ.get("CENTRE_REFERENCE_ROOT", ""), "test_examples",
                      "example-1", "outfiles-h-ref")


def test_roundtrip_bins(tmp_path):
    d = np.load(os.path.join(GOLDEN, "example1.npz"))
    p = tmp_path / "bin_torsions.nc"
    cdf5.write_bins(str(p), "T", d["torsions_dimid"], d["torsions_ext"], d["torsions_coord"], [30])
    dimid, ext, coord, sch = cdf5.read_bins(str(p))
    assert np.array_equal(dimid, d["torsions_dimid"])
    assert np.array_equal(ext, d["torsions_ext"])
    assert np.array_equal(coord, d["torsions_coord"])
    assert sch.tolist() == [30]


def test_bin_files_hash_like_the_reference(tmp_path):
    """The writer, fed example-1's bins, extremes and DOF ids, produces files
    whose SHA-256 and size are those of the reference's own bin_*.nc."""
    import hashlib
    import json
    d = np.load(os.path.join(GOLDEN, "example1.npz"))
    with open(os.path.join(GOLDEN, "example1.json")) as f:
        schemes = json.load(f)["schemes"]
    with open(os.path.join(GOLDEN, "example1_binfiles.json")) as f:
        want = json.load(f)
    for t, c in (("bonds", "B"), ("angles", "A"), ("torsions", "T")):
        out = tmp_path / f"bin_{t}.nc"
        cdf5.write_bins(str(out), c, d[f"{t}_dimid"], d[f"{t}_ext"], d[f"{t}_coord"], schemes)
        raw = out.read_bytes()
        assert len(raw) == want[t]["bytes"], t
        assert hashlib.sha256(raw).hexdigest() == want[t]["sha256"], t


@pytest.mark.skipif(not os.environ.get("CENTRE_REFERENCE_ROOT") or not os.path.isdir(REFDIR),
                    reason="CENTRE_REFERENCE_ROOT unset or its example files absent")
def test_reference_bin_file_is_reproduced_byte_for_byte(tmp_path):
    for t, c in (("bonds", "B"), ("angles", "A"), ("torsions", "T")):
        src = os.path.join(REFDIR, f"bin_{t}.nc")
        dimid, ext, coord, sch = cdf5.read_bins(src)
        out = tmp_path / f"bin_{t}.nc"
        cdf5.write_bins(str(out), c, dimid, ext, coord, sch)
        assert open(src, "rb").read() == open(out, "rb").read()


def test_truncated_and_corrupt_files_raise(tmp_path):
    d = np.load(os.path.join(GOLDEN, "example1.npz"))
    p = tmp_path / "b.nc"
    cdf5.write_bins(str(p), "B", d["bonds_dimid"], d["bonds_ext"], d["bonds_coord"], [30])
    raw = open(p, "rb").read()
    for cut in (3, 40, 200, len(raw) - 100):
        q = tmp_path / f"t{cut}.nc"
        q.write_bytes(raw[:cut])
        with pytest.raises(cdf5.CDFError):
            cdf5.read(str(q))
    q = tmp_path / "bad.nc"
    q.write_bytes(b"HDF5" + raw[4:])
    with pytest.raises(cdf5.CDFError):
        cdf5.read(str(q))


def test_generic_dataset_roundtrip(tmp_path):
    ds = cdf5.Dataset(version=5)
    ds.dims = {"records": 0, "ids": 2, "n": 3}
    ds.attrs = {"title": "x", "order": np.array([2], np.uint8), "vals": np.arange(3.0)}
    ds.vars = {
        "id": cdf5.Variable("id", ("records", "ids"), 9, {}, np.arange(10, dtype=np.uint32).reshape(5, 2)),
        "s": cdf5.Variable("s", ("records", "n"), 6, {}, np.random.default_rng(0).random((5, 3))),
        "fixed": cdf5.Variable("fixed", ("n",), 11, {}, np.array([1, 2, 3], np.uint64)),
    }
    p = tmp_path / "g.nc"
    cdf5.write(str(p), ds)
    r = cdf5.read(str(p))
    assert r.numrecs == 5
    for k in ds.vars:
        assert np.array_equal(r.vars[k].data, ds.vars[k].data)
    assert r.attrs["title"] == "x"
