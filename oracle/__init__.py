"""CPU oracle for the CENTRE entropy hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg (and its reference arm) import this package, and only as the checker or
the timed CPU baseline.  The product (``centre_gb300``) never imports it.

Two CPU implementations are wrapped here:

* ``Oracle``: the plain-C restatement in ``centre_oracle.c`` (built into
  ``liboracle.so`` by ``oracle/Makefile``).  Every function cites the
  reference file:line it follows.
* ``Reference``: the reference's own numeric sources (shaileshp51/centre
  ``src/Estimators.cpp``, ``src/Real2Int.cpp``, ``src/Centre.cpp``,
  ``src/Utils.cpp``, ``src/Convergance.cpp``) compiled from source into
  ``oracle/_ref/libcentre_ref.so`` with ``ref_shim.cpp``.  Available only
  where the reference checkout exists; used to pin ``Oracle``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ORACLE_SO = os.path.join(_HERE, "liboracle.so")
_REF_SO = os.path.join(_HERE, "_ref", "libcentre_ref.so")

BOND, ANGLE, DIHEDRAL = 1, 2, 3
ML, MM, CS, JS = 0, 1, 2, 3

_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")


def build(with_ref: bool = True) -> None:
    """Compile liboracle.so (and the reference shim when the reference
    sources are present)."""
    subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    if with_ref:
        # the recipe builds the shim only where the reference checkout exists
        # ($CENTRE_REFERENCE_ROOT, else the Makefile's REFROOT)
        cmd = ["make", "-s", "-C", _HERE, "ref-if-present"]
        refroot = os.environ.get("CENTRE_REFERENCE_ROOT")
        if refroot:
            cmd.append(f"REFROOT={refroot}")
        subprocess.run(cmd, check=True)


def ref_available() -> bool:
    return os.path.exists(_REF_SO)


def _u8(a):
    return np.ascontiguousarray(a, dtype=np.uint8)


class Oracle:
    """ctypes front-end over liboracle.so (the C restatement)."""

    def __init__(self, path: str = _ORACLE_SO):
        if not os.path.exists(path):
            build(with_ref=False)
        L = C.CDLL(path)
        self.L = L
        L.orc_discretize_block.argtypes = [C.c_int, _f32p, C.c_uint32, C.c_uint64, _u8p,
                                           C.c_int, C.c_uint8, C.c_int, _u8p, _f64p, C.c_int]
        L.orc_vmkde_minima.argtypes = [_f32p, C.c_uint64, C.c_uint8, C.c_double, C.c_uint32,
                                       C.c_double, C.c_uint32, _f64p, _u8p, _u8p]
        L.orc_bessel_i.argtypes = [C.c_int, C.c_double]
        L.orc_bessel_i.restype = C.c_double
        L.orc_bin1d.argtypes = [C.c_uint8, _u8p, C.c_int, C.c_uint64, C.c_double, C.c_double,
                                _u8p, _u64p, C.c_void_p]
        L.orc_bin2d.argtypes = [C.c_uint8, _u8p, C.c_int, C.c_uint64, C.c_double, C.c_double,
                                C.c_double, C.c_double, _u8p, _u8p, _u64p, C.c_void_p]
        L.orc_entropy1d_block.argtypes = [C.c_uint32, _u8p, _u8p, _f64p, C.c_uint64, C.c_uint8,
                                          _u8p, C.c_int, _u8p, C.c_int, C.c_int, C.c_int,
                                          _f64p, C.c_int]
        L.orc_entropy2d_pairs.argtypes = [C.c_uint64, _u32p, _u8p, _u8p, _f64p, C.c_uint64,
                                          C.c_uint8, _u8p, C.c_int, _u8p, C.c_int, C.c_int,
                                          C.c_int, _f64p, C.c_int]
        L.orc_boruvka_mst.argtypes = [C.c_uint32, C.c_uint64, _u32p, _u32p, _f64p, _u64p]
        L.orc_boruvka_mst.restype = C.c_int64

    def discretize(self, bat_type, data, schemes, bins_ref=None, optimize=True, nthreads=0):
        """data [ndof][nframes] f32 -> bins [ndof][nschemes][nframes], extremes [ndof][4]."""
        data = np.ascontiguousarray(data, dtype=np.float32)
        ndof, n = data.shape
        sch = _u8(schemes)
        bins = np.zeros((ndof, len(sch), n), np.uint8)
        ext = np.zeros((ndof, 4), np.float64)
        ref = int(bins_ref if bins_ref is not None else sch[0])
        rc = self.L.orc_discretize_block(bat_type, data, ndof, n, sch, len(sch), ref,
                                         int(optimize), bins, ext, nthreads)
        if rc:
            raise ValueError(f"oracle discretize failed ({rc})")
        return bins, ext

    def vmkde(self, data, nconf=5, kappa=1.0, step_sdo=5, conv=1e-4, max_iter=1000):
        data = np.ascontiguousarray(data, dtype=np.float32)
        mins = np.zeros(max(int(nconf), 1), np.float64)
        found = np.zeros(1, np.uint8)
        out = np.zeros(len(data), np.uint8)
        self.L.orc_vmkde_minima(data, len(data), nconf, kappa, step_sdo, conv, max_iter,
                                mins, found, out)
        return out, mins[: found[0]], int(found[0])

    def bessel_i(self, n, x):
        return self.L.orc_bessel_i(int(n), float(x))

    def bin1d(self, bins, nsteps, schemes, mn=0.0, mx=1.0):
        sch = _u8(schemes)
        b = _u8(bins)
        n = b.shape[-1]
        fr = np.zeros(nsteps * int(sch.astype(int).sum()), np.uint64)
        rc = self.L.orc_bin1d(nsteps, sch, len(sch), n, mn, mx, b.reshape(-1), fr, None)
        if rc:
            raise ValueError(f"oracle bin1d failed ({rc})")
        return fr

    def bin2d(self, b1, b2, nsteps, schemes):
        sch = _u8(schemes)
        b1 = _u8(b1)
        b2 = _u8(b2)
        n = b1.shape[-1]
        fr = np.zeros(nsteps * int((sch.astype(int) ** 2).sum()), np.uint64)
        rc = self.L.orc_bin2d(nsteps, sch, len(sch), n, 0.0, 1.0, 0.0, 1.0,
                              b1.reshape(-1), b2.reshape(-1), fr, None)
        if rc:
            raise ValueError(f"oracle bin2d failed ({rc})")
        return fr

    def entropy1d(self, types, bins, extremes, nsteps, schemes, ests=(ML,), jacobian=True,
                  kde=False, nthreads=0):
        bins = _u8(bins)
        ndof, nsch, n = bins.shape
        sch, es = _u8(schemes), _u8(ests)
        out = np.zeros((ndof, len(es), nsch, nsteps), np.float64)
        rc = self.L.orc_entropy1d_block(ndof, _u8(types), bins, np.ascontiguousarray(extremes),
                                        n, nsteps, sch, len(sch), es, len(es), int(jacobian),
                                        int(kde), out, nthreads)
        if rc:
            raise ValueError(f"oracle entropy1d failed ({rc})")
        return out

    def entropy2d(self, pairs, types, bins, extremes, nsteps, schemes, ests=(ML,),
                  jacobian=True, kde=False, nthreads=0):
        bins = _u8(bins)
        ndof, nsch, n = bins.shape
        pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
        sch, es = _u8(schemes), _u8(ests)
        out = np.zeros((len(pairs), len(es), nsch, nsteps), np.float64)
        rc = self.L.orc_entropy2d_pairs(len(pairs), pairs, _u8(types), bins,
                                        np.ascontiguousarray(extremes), n, nsteps, sch,
                                        len(sch), es, len(es), int(jacobian), int(kde), out,
                                        nthreads)
        if rc:
            raise ValueError(f"oracle entropy2d failed ({rc})")
        return out

    def mst(self, nv, src, dst, w):
        src = np.ascontiguousarray(src, np.uint32)
        dst = np.ascontiguousarray(dst, np.uint32)
        w = np.ascontiguousarray(w, np.float64)
        tree = np.zeros(max(nv, 1), np.uint64)
        nt = self.L.orc_boruvka_mst(nv, len(w), src, dst, w, tree)
        return tree[:nt].astype(np.int64)


class Reference:
    """ctypes front-end over the reference's own code (oracle/_ref)."""

    def __init__(self, path: str = _REF_SO):
        L = C.CDLL(path)
        self.L = L
        L.ref_real2int.argtypes = [C.c_int, _f32p, C.c_uint64, _u8p, C.c_int, C.c_uint8,
                                   C.c_int, _f64p, _u8p]
        L.ref_vmkde.argtypes = [_f32p, C.c_uint64, C.c_uint8, C.c_double, C.c_uint32,
                                C.c_double, C.c_uint32, _f64p, _u8p, _u8p]
        L.ref_bessel_i.argtypes = [C.c_int, C.c_double]
        L.ref_bessel_i.restype = C.c_double
        L.ref_entropy1d.argtypes = [C.c_int, _u8p, C.c_uint64, C.c_uint8, _u8p, C.c_int,
                                    C.c_double, C.c_double, _u8p, C.c_int, C.c_int, C.c_int,
                                    C.c_void_p, _f64p]
        L.ref_entropy2d.argtypes = [C.c_int, C.c_int, _u8p, _u8p, C.c_uint64, C.c_uint8, _u8p,
                                    C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                    _u8p, C.c_int, C.c_int, C.c_int, C.c_void_p, _f64p]
        L.ref_mst.argtypes = [C.c_uint32, C.c_uint64, _u32p, _u32p, _f64p, _u32p, _u32p, _f64p]
        L.ref_mst.restype = C.c_int64

    def discretize(self, bat_type, data, schemes, bins_ref=None, optimize=True):
        data = np.ascontiguousarray(data, dtype=np.float32)
        ndof, n = data.shape
        sch = _u8(schemes)
        ref = int(bins_ref if bins_ref is not None else sch[0])
        bins = np.zeros((ndof, len(sch), n), np.uint8)
        ext = np.zeros((ndof, 4), np.float64)
        for d in range(ndof):
            e = np.zeros(4, np.float64)
            o = np.zeros(len(sch) * n, np.uint8)
            rc = self.L.ref_real2int(bat_type, data[d], n, sch, len(sch), ref, int(optimize),
                                     e, o)
            if rc:
                raise ValueError("reference real2int failed")
            bins[d] = o.reshape(len(sch), n)
            ext[d] = e
        return bins, ext

    def vmkde(self, data, nconf=5, kappa=1.0, step_sdo=5, conv=1e-4, max_iter=1000):
        data = np.ascontiguousarray(data, dtype=np.float32)
        mins = np.zeros(max(int(nconf), 1), np.float64)
        found = np.zeros(1, np.uint8)
        out = np.zeros(len(data), np.uint8)
        self.L.ref_vmkde(data, len(data), nconf, kappa, step_sdo, conv, max_iter, mins, found,
                         out)
        return out, mins[: found[0]], int(found[0])

    def bessel_i(self, n, x):
        return self.L.ref_bessel_i(int(n), float(x))

    def entropy1d(self, type_, bins, mn, mx, nsteps, schemes, ests=(ML,), jacobian=True,
                  kde=False):
        bins = _u8(bins)
        nsch, n = bins.shape
        sch, es = _u8(schemes), _u8(ests)
        out = np.zeros((len(es), nsch, nsteps), np.float64)
        self.L.ref_entropy1d(type_, bins.reshape(-1), n, nsteps, sch, len(sch), mn, mx, es,
                             len(es), int(jacobian), int(kde), None, out.reshape(-1))
        return out

    def entropy2d(self, t1, t2, b1, b2, e1, e2, nsteps, schemes, ests=(ML,), jacobian=True,
                  kde=False):
        b1, b2 = _u8(b1), _u8(b2)
        nsch, n = b1.shape
        sch, es = _u8(schemes), _u8(ests)
        out = np.zeros((len(es), nsch, nsteps), np.float64)
        self.L.ref_entropy2d(t1, t2, b1.reshape(-1), b2.reshape(-1), n, nsteps, sch, len(sch),
                             e1[0], e1[1], e2[0], e2[1], es, len(es), int(jacobian), int(kde),
                             None, out.reshape(-1))
        return out

    def mst(self, nv, src, dst, w):
        src = np.ascontiguousarray(src, np.uint32)
        dst = np.ascontiguousarray(dst, np.uint32)
        w = np.ascontiguousarray(w, np.float64)
        ts = np.zeros(max(nv, 1), np.uint32)
        td = np.zeros(max(nv, 1), np.uint32)
        tw = np.zeros(max(nv, 1), np.float64)
        nt = self.L.ref_mst(nv, len(w), src, dst, w, ts, td, tw)
        return ts[:nt], td[:nt], tw[:nt]
