"""Reader and writer for NetCDF classic files (CDF-1, CDF-2 and CDF-5).

The reference stores its intermediate bin files as CDF-5 ("64-bit data",
``NC_64BIT_DATA``, src/Netcdf_TrjInt.cpp:549) and reads BAT trajectories and
writes entropy contributions through libnetcdf.  libnetcdf is not part of
this project; this module implements the published classic-format layout
(big-endian header of dimensions, attributes and variables, then the data
section with record variables interleaved per record) so the reference's
files can be read and files it can read can be written.

    ds = read("bin_torsions.nc")
    ds.dims["frames"], ds.vars["coord"].data.shape, ds.attrs["binSchemes"]
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

NC_DIMENSION, NC_VARIABLE, NC_ATTRIBUTE = 0x0A, 0x0B, 0x0C

# nc_type -> numpy big-endian dtype
_TYPES = {
    1: np.dtype(">i1"), 2: np.dtype("S1"), 3: np.dtype(">i2"), 4: np.dtype(">i4"),
    5: np.dtype(">f4"), 6: np.dtype(">f8"), 7: np.dtype(">u1"), 8: np.dtype(">u2"),
    9: np.dtype(">u4"), 10: np.dtype(">i8"), 11: np.dtype(">u8"),
}
_CODES = {"i1": 1, "S1": 2, "i2": 3, "i4": 4, "f4": 5, "f8": 6, "u1": 7, "u2": 8,
          "u4": 9, "i8": 10, "u8": 11}


class CDFError(ValueError):
    pass


@dataclass
class Variable:
    name: str
    dims: tuple
    nctype: int
    attrs: dict = field(default_factory=dict)
    data: np.ndarray | None = None
    vsize: int = 0
    begin: int = 0


@dataclass
class Dataset:
    version: int = 5
    dims: dict = field(default_factory=dict)        # name -> length (0 = record)
    attrs: dict = field(default_factory=dict)
    vars: dict = field(default_factory=dict)
    numrecs: int = 0

    @property
    def record_dim(self):
        for k, v in self.dims.items():
            if v == 0:
                return k
        return None


def _pad4(n: int) -> int:
    return (4 - n % 4) % 4


class _Reader:
    def __init__(self, buf: bytes):
        self.b = buf
        self.o = 0
        if len(buf) < 4 or buf[:3] != b"CDF":
            raise CDFError("not a NetCDF classic file (magic)")
        self.ver = buf[3]
        if self.ver not in (1, 2, 5):
            raise CDFError(f"unsupported CDF version {self.ver}")
        self.o = 4

    def need(self, n):
        if self.o + n > len(self.b):
            raise CDFError("truncated NetCDF header")

    def u32(self):
        self.need(4)
        v = struct.unpack_from(">I", self.b, self.o)[0]
        self.o += 4
        return v

    def u64(self):
        self.need(8)
        v = struct.unpack_from(">Q", self.b, self.o)[0]
        self.o += 8
        return v

    def nonneg(self):
        return self.u64() if self.ver == 5 else self.u32()

    def offset(self):
        return self.u32() if self.ver == 1 else self.u64()

    def name(self):
        n = self.nonneg()
        self.need(n)
        s = self.b[self.o:self.o + n].decode("utf-8", "replace")
        self.o += n + _pad4(n)
        return s

    def values(self, nctype, n):
        if nctype not in _TYPES:
            raise CDFError(f"bad nc_type {nctype}")
        dt = _TYPES[nctype]
        nb = dt.itemsize * n
        self.need(nb)
        raw = self.b[self.o:self.o + nb]
        self.o += nb + _pad4(nb)
        if nctype == 2:
            return raw.decode("utf-8", "replace")
        return np.frombuffer(raw, dtype=dt).astype(dt.newbyteorder("="))

    def att_list(self):
        tag = self.u32()
        n = self.nonneg()
        if tag == 0 and n == 0:
            return {}
        if tag != NC_ATTRIBUTE:
            raise CDFError("bad attribute list tag")
        out = {}
        for _ in range(n):
            nm = self.name()
            t = self.u32()
            cnt = self.nonneg()
            out[nm] = self.values(t, cnt)
        return out


def read(path: str, load_data: bool = True) -> Dataset:
    with open(path, "rb") as f:
        buf = f.read()
    return parse(buf, load_data)


def parse(buf: bytes, load_data: bool = True) -> Dataset:
    r = _Reader(buf)
    ds = Dataset(version=r.ver)
    ds.numrecs = r.nonneg()
    tag = r.u32()
    n = r.nonneg()
    dimnames = []
    if not (tag == 0 and n == 0):
        if tag != NC_DIMENSION:
            raise CDFError("bad dimension list tag")
        for _ in range(n):
            nm = r.name()
            ln = r.nonneg()
            ds.dims[nm] = ln
            dimnames.append(nm)
    ds.attrs = r.att_list()
    tag = r.u32()
    n = r.nonneg()
    if not (tag == 0 and n == 0):
        if tag != NC_VARIABLE:
            raise CDFError("bad variable list tag")
        for _ in range(n):
            nm = r.name()
            nd = r.nonneg()
            ids = [r.nonneg() for _ in range(nd)]
            for i in ids:
                if i >= len(dimnames):
                    raise CDFError("variable refers to an unknown dimension")
            attrs = r.att_list()
            t = r.u32()
            vsize = r.nonneg()
            begin = r.offset()
            ds.vars[nm] = Variable(nm, tuple(dimnames[i] for i in ids), t, attrs, None, vsize, begin)
    if load_data:
        _load(ds, buf)
    return ds


def _is_record(ds: Dataset, v: Variable) -> bool:
    return bool(v.dims) and ds.dims[v.dims[0]] == 0


def _recsize(ds: Dataset) -> int:
    recvars = [v for v in ds.vars.values() if _is_record(ds, v)]
    if len(recvars) == 1:
        v = recvars[0]
        dt = _TYPES[v.nctype]
        return int(np.prod([ds.dims[d] for d in v.dims[1:]], dtype=np.int64)) * dt.itemsize
    return sum(v.vsize for v in recvars)


def _load(ds: Dataset, buf: bytes):
    recsize = _recsize(ds)
    for v in ds.vars.values():
        dt = _TYPES[v.nctype]
        if _is_record(ds, v):
            inner = [ds.dims[d] for d in v.dims[1:]]
            per = int(np.prod(inner, dtype=np.int64)) * dt.itemsize
            out = np.empty((ds.numrecs, per), np.uint8)
            for rec in range(ds.numrecs):
                o = v.begin + rec * recsize
                if o + per > len(buf):
                    raise CDFError(f"truncated data for {v.name}")
                out[rec] = np.frombuffer(buf, np.uint8, per, o)
            arr = out.view(dt).reshape([ds.numrecs] + inner)
        else:
            shape = [ds.dims[d] for d in v.dims]
            cnt = int(np.prod(shape, dtype=np.int64))
            if v.begin + cnt * dt.itemsize > len(buf):
                raise CDFError(f"truncated data for {v.name}")
            arr = np.frombuffer(buf, dt, cnt, v.begin).reshape(shape)
        if v.nctype == 2:
            v.data = arr
        else:
            v.data = arr.astype(dt.newbyteorder("="))


# ---------------------------------------------------------------- writing --
def _enc_name(ver, s: str) -> bytes:
    b = s.encode()
    n = struct.pack(">Q" if ver == 5 else ">I", len(b))
    return n + b + b"\0" * _pad4(len(b))


def _nonneg(ver, v):
    return struct.pack(">Q" if ver == 5 else ">I", v)


def _enc_att(ver, name, val) -> bytes:
    if isinstance(val, str):
        raw = val.encode()
        t, cnt = 2, len(raw)
    else:
        a = np.atleast_1d(np.asarray(val))
        code = _CODES.get(a.dtype.str[1:])
        if code is None:
            raise CDFError(f"cannot store attribute dtype {a.dtype}")
        raw = a.astype(_TYPES[code]).tobytes()
        t, cnt = code, a.size
    return _enc_name(ver, name) + struct.pack(">I", t) + _nonneg(ver, cnt) + raw + b"\0" * _pad4(len(raw))


def _enc_atts(ver, attrs) -> bytes:
    if not attrs:
        return struct.pack(">I", 0) + _nonneg(ver, 0)
    return (struct.pack(">I", NC_ATTRIBUTE) + _nonneg(ver, len(attrs)) +
            b"".join(_enc_att(ver, k, v) for k, v in attrs.items()))


def write(path: str, ds: Dataset) -> None:
    """Write ds (dims, attrs, vars with .data set) as a classic file."""
    ver = ds.version
    rec = ds.record_dim
    numrecs = 0
    for v in ds.vars.values():
        if v.dims and v.dims[0] == rec and rec is not None:
            numrecs = max(numrecs, int(v.data.shape[0]))
    dimnames = list(ds.dims)
    # sizes
    for v in ds.vars.values():
        dt = _TYPES[v.nctype]
        shape = [ds.dims[d] for d in v.dims]
        if rec is not None and v.dims and v.dims[0] == rec:
            shape = shape[1:]
        nbytes = int(np.prod(shape, dtype=np.int64)) * dt.itemsize
        v.vsize = nbytes + _pad4(nbytes)

    def header(begins):
        h = b"CDF" + bytes([ver]) + _nonneg(ver, numrecs)
        if ds.dims:
            h += struct.pack(">I", NC_DIMENSION) + _nonneg(ver, len(ds.dims))
            for k, ln in ds.dims.items():
                h += _enc_name(ver, k) + _nonneg(ver, ln)
        else:
            h += struct.pack(">I", 0) + _nonneg(ver, 0)
        h += _enc_atts(ver, ds.attrs)
        if ds.vars:
            h += struct.pack(">I", NC_VARIABLE) + _nonneg(ver, len(ds.vars))
            for (k, v), b in zip(ds.vars.items(), begins):
                h += _enc_name(ver, k) + _nonneg(ver, len(v.dims))
                for d in v.dims:
                    h += _nonneg(ver, dimnames.index(d))
                h += _enc_atts(ver, v.attrs) + struct.pack(">I", v.nctype)
                h += _nonneg(ver, v.vsize)
                h += struct.pack(">I" if ver == 1 else ">Q", b)
        else:
            h += struct.pack(">I", 0) + _nonneg(ver, 0)
        return h

    names = list(ds.vars)
    hlen = len(header([0] * len(names)))
    fixed = [k for k in names if not (rec and ds.vars[k].dims and ds.vars[k].dims[0] == rec)]
    recs = [k for k in names if k not in fixed]
    begins = {}
    o = hlen
    for k in fixed:
        begins[k] = o
        o += ds.vars[k].vsize
    recstart = o
    for k in recs:
        begins[k] = o
        o += ds.vars[k].vsize
    recsize = sum(ds.vars[k].vsize for k in recs)
    if len(recs) == 1:
        v = ds.vars[recs[0]]
        dt = _TYPES[v.nctype]
        recsize = int(np.prod([ds.dims[d] for d in v.dims[1:]], dtype=np.int64)) * dt.itemsize
    with open(path, "wb") as f:
        f.write(header([begins[k] for k in names]))
        for k in fixed:
            v = ds.vars[k]
            raw = np.ascontiguousarray(v.data, dtype=_TYPES[v.nctype]).tobytes()
            f.write(raw + b"\0" * (v.vsize - len(raw)))
        for r in range(numrecs):
            for k in recs:
                v = ds.vars[k]
                raw = np.ascontiguousarray(v.data[r], dtype=_TYPES[v.nctype]).tobytes()
                f.write(raw + (b"\0" * (v.vsize - len(raw)) if len(recs) > 1 else b""))
        del recstart


# ----------------------------------------------------- CENTRE bin files --
def read_bins(path: str):
    """bin_*.nc (src/Netcdf_TrjInt.cpp:542-755) -> (dimid, extremes, coord,
    bin_schemes): dimid [dims], extremes [dims][4], coord [dims][nschemes][frames]."""
    ds = read(path)
    dimid = ds.vars["dimid"].data.astype(np.uint32)
    ext = ds.vars["extreme"].data.astype(np.float64)
    coord = ds.vars["coord"].data.astype(np.uint8)
    schemes = np.atleast_1d(ds.attrs.get("binSchemes", np.array([coord.shape[1]]))).astype(np.uint8)
    return dimid, ext, coord, schemes


def write_bins(path: str, content: str, dimid, extremes, coord, bin_schemes):
    """Write a bin file with the reference's dims, variables and attributes."""
    coord = np.ascontiguousarray(coord, np.uint8)
    ndof, nsch, nfr = coord.shape
    ds = Dataset(version=5)
    ds.dims = {"dims": 0, "extremes": 4, "bin_scheme_count": nsch, "frames": nfr}
    ds.attrs = {
        "title": f"{content} Integer Vectors", "application": "CENTRE",
        "program": "Real2Int", "programVersion": "1.0.0", "convention": "CENTRE_Real",
        "conventionVersion": "1.0", "content": content,
        "ncoordims": np.array([ndof], np.uint32),
        "nbinSchemes": np.array([nsch], np.uint8),
        "binSchemes": np.asarray(bin_schemes, np.uint8),
    }
    ds.vars = {
        "dimid": Variable("dimid", ("dims",), 9, {}, np.asarray(dimid, np.uint32)),
        "extreme": Variable("extreme", ("dims", "extremes"), 6, {},
                             np.asarray(extremes, np.float64)),
        "coord": Variable("coord", ("dims", "bin_scheme_count", "frames"), 7, {}, coord),
    }
    write(path, ds)


# ------------------------------------------------------- BAT trajectories --
def write_bat(path: str, bonds, angles, torsions, time=None, version: int = 5):
    """A CENTRE BAT trajectory as Netcdf_BAT reads it (src/Netcdf_BAT.cpp:
    24-132, 236-330): global attribute convention = "CENTRE", record
    dimension "frame", variables time [frame], bond [frame][bond], angle
    [frame][angle], dihedral [frame][dihedral] (float32).  Inputs are
    DOF-major [ndof][nframes] arrays."""
    b = np.ascontiguousarray(np.asarray(bonds, np.float32).T)
    a = np.ascontiguousarray(np.asarray(angles, np.float32).T)
    d = np.ascontiguousarray(np.asarray(torsions, np.float32).T)
    nfr = b.shape[0]
    t = np.arange(nfr, dtype=np.float32) if time is None else np.asarray(time, np.float32)
    ds = Dataset(version=version)
    ds.dims = {"frame": 0, "bond": b.shape[1], "angle": a.shape[1], "dihedral": d.shape[1]}
    ds.attrs = {"title": "BAT trajectory", "application": "CENTRE", "program": "centre_gb300",
                "programVersion": "1.0.0", "convention": "CENTRE", "conventionVersion": "1.0",
                "hasPseudo": "N"}
    ds.vars = {
        "time": Variable("time", ("frame",), 5, {"units": "picosecond"}, t),
        "bond": Variable("bond", ("frame", "bond"), 5, {"units": "angstrom"}, b),
        "angle": Variable("angle", ("frame", "angle"), 5, {"units": "radian"}, a),
        "dihedral": Variable("dihedral", ("frame", "dihedral"), 5, {"units": "radian"}, d),
    }
    write(path, ds)


def read_entcontri(path: str):
    """entcontri_*.nc -> (ids [records][order] uint32, contri_S [records][est][sch][steps])."""
    ds = read(path)
    return ds.vars["id"].data.astype(np.uint32), ds.vars["contri_S"].data.astype(np.float64)
