"""Python front-end over the C ABI (host numpy buffers or device tensors).

``Context`` wraps one ``centre_ctx``.  Methods without a suffix take and
return numpy arrays (the C entry points copy host<->device inside); ``*_dev``
methods take torch CUDA tensors (device pointers, asynchronous on the
context's stream).  Array layouts are the reference's (see
include/centre_gpu.h).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import CentreError, EntropyParams, make_params, SUMS_COLS, SUMS_NAMES  # noqa: F401
from ._lib import System, ScreenParams, make_screen_params, SCREEN_NPARAMS  # noqa: F401

BOND, ANGLE, DIHEDRAL = 1, 2, 3
ML, MM, CS, JS = 0, 1, 2, 3


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    return C.c_void_p(int(a.data_ptr()))  # torch tensor


def _addr(a):
    p = _ptr(a)
    return None if p is None else p.value


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Context:
    def __init__(self, device: int = 0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.centre_gpu_create(C.byref(h), int(device))
        if rc != 0:
            raise CentreError(rc, self.L.centre_gpu_strerror(rc).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.centre_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def check(self, rc: int):
        if rc != 0:
            msg = self.L.centre_gpu_last_error(self.h).decode()
            raise CentreError(rc, msg or self.L.centre_gpu_strerror(rc).decode())

    @property
    def launches(self) -> int:
        return int(self.L.centre_gpu_launch_count(self.h))

    def set_stream(self, stream_ptr: int):
        self.check(self.L.centre_gpu_set_stream(self.h, C.c_void_p(stream_ptr)))

    def enable_timing(self, on: bool = True):
        self.check(self.L.centre_gpu_enable_timing(self.h, int(bool(on))))

    def timer(self, which: int):
        """(milliseconds, launches) of a kernel class since timing was enabled:
        0 discretise, 1 1-D counts, 2 pair counts, 3 scoring."""
        ms = C.c_double()
        n = C.c_uint64()
        self.check(self.L.centre_gpu_timer(self.h, int(which), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def synchronize(self):
        self.check(self.L.centre_gpu_synchronize(self.h))

    # ---------------------------------------------------------- host API --
    def discretize(self, bat_type, data, schemes, bins_ref=None, optimize=True, bins_out=None,
                   ext_out=None):
        data = _c(data, np.float32)
        ndof, n = data.shape
        sch = _c(schemes, np.uint8)
        bins = bins_out if bins_out is not None else np.empty((ndof, len(sch), n), np.uint8)
        ext = ext_out if ext_out is not None else np.empty((ndof, 4), np.float64)
        ref = int(bins_ref if bins_ref is not None else sch[0])
        self.check(self.L.centre_gpu_discretize(self.h, int(bat_type), _ptr(data), ndof, n,
                                                _ptr(sch), len(sch), ref, int(bool(optimize)),
                                                _ptr(bins), _ptr(ext)))
        return bins, ext

    def discretize_vmkde(self, data, nmaxconf=5, kappa=1.0, sdo_nstep=5, sdo_conv=1e-4,
                         sdo_niter=1000):
        """von Mises KDE conformer bins of torsions [ndof][nframes] ->
        (bins [ndof][1][nframes], minima [ndof][nmaxconf] rad, nfound [ndof])."""
        data = _c(data, np.float32)
        ndof, n = data.shape
        bins = np.empty((ndof, 1, n), np.uint8)
        minima = np.zeros((ndof, nmaxconf), np.float64)
        nfound = np.zeros(ndof, np.uint8)
        self.check(self.L.centre_gpu_discretize_vmkde(self.h, _ptr(data), ndof, n, int(nmaxconf),
                                                      float(kappa), int(sdo_nstep),
                                                      float(sdo_conv), int(sdo_niter),
                                                      _ptr(bins), _ptr(minima), _ptr(nfound)))
        return bins, minima, nfound

    def discretize_gridkde(self, bat_type, data, ngrid, kappa=50.0):
        """Grid-KDE conformer bins of one DOF-type block [ndof][nframes]
        (torsions: von Mises kernel of concentration kappa on ngrid points of
        the circle; bonds/angles: Gaussian kernel, Silverman bandwidth, on
        ngrid points over the DOF's range) -> (bins [ndof][1][nframes],
        minima [ndof][ngrid] (first nmin used), nmin [ndof], nbins [ndof])."""
        data = _c(data, np.float32)
        ndof, n = data.shape
        bins = np.empty((ndof, 1, n), np.uint8)
        minima = np.zeros((ndof, ngrid), np.float64)
        nmin = np.zeros(ndof, np.uint8)
        nbins = np.zeros(ndof, np.uint8)
        self.check(self.L.centre_gpu_discretize_gridkde(self.h, int(bat_type), _ptr(data), ndof, n,
                                                        int(ngrid), float(kappa), _ptr(bins),
                                                        _ptr(minima), _ptr(nmin), _ptr(nbins)))
        return bins, minima, nmin, nbins

    def df_exp_eval(self, y):
        """The library's double-float e^y (y <= 0) for an array of doubles."""
        y = _c(y, np.float64)
        out = np.empty_like(y)
        self.check(self.L.centre_gpu_df_exp_eval(self.h, _ptr(y), y.size, _ptr(out)))
        return out

    def discretize_gridkde_dev(self, bat_type, data, ngrid, kappa, bins_out, minima_out,
                               nmin_out, nbins_out):
        """Device-pointer form of discretize_gridkde (torch CUDA tensors)."""
        ndof, n = int(data.shape[0]), int(data.shape[1])
        self.check(self.L.centre_gpu_discretize_gridkde_dev(
            self.h, int(bat_type), _ptr(data), ndof, n, int(ngrid), float(kappa), _ptr(bins_out),
            _ptr(minima_out), _ptr(nmin_out), _ptr(nbins_out)))

    def entropy1d(self, params: EntropyParams, types, bins, ext, want_freq=False, out=None):
        bins = _c(bins, np.uint8)
        types = _c(types, np.uint8)
        ext = _c(ext, np.float64)
        ndof = bins.shape[0]
        s1 = out if out is not None else np.empty(
            (ndof, params.nestimators, params.nschemes, params.nsteps), np.float64)
        freq = None
        if want_freq:
            nsum = sum(params.bin_schemes[i] for i in range(params.nschemes))
            freq = np.empty((ndof, params.nsteps, nsum), np.uint64)
        self.check(self.L.centre_gpu_entropy1d(self.h, C.byref(params), ndof, _ptr(types),
                                               _ptr(bins), _ptr(ext), _ptr(s1), _ptr(freq)))
        return (s1, freq) if want_freq else s1

    def entropy2d(self, params: EntropyParams, types, bins, ext, pairs=None, out=None):
        bins = _c(bins, np.uint8)
        types = _c(types, np.uint8)
        ext = _c(ext, np.float64)
        ndof = bins.shape[0]
        if pairs is not None:
            pairs = _c(pairs, np.uint32).reshape(-1, 2)
            npairs = len(pairs)
        else:
            npairs = ndof * (ndof - 1) // 2
        s2 = out if out is not None else np.empty(
            (npairs, params.nestimators, params.nschemes, params.nsteps), np.float64)
        self.check(self.L.centre_gpu_entropy2d(self.h, C.byref(params), ndof, _ptr(types),
                                               _ptr(bins), _ptr(ext), npairs, _ptr(pairs),
                                               _ptr(s2)))
        return s2

    def counts2d(self, params: EntropyParams, bins, pairs):
        bins = _c(bins, np.uint8)
        pairs = _c(pairs, np.uint32).reshape(-1, 2)
        nsq = sum(params.bin_schemes[i] ** 2 for i in range(params.nschemes))
        freq = np.empty((len(pairs), params.nsteps, nsq), np.uint64)
        self.check(self.L.centre_gpu_counts2d(self.h, C.byref(params), bins.shape[0], _ptr(bins),
                                              len(pairs), _ptr(pairs), _ptr(freq)))
        return freq

    def pair_moments(self, params: EntropyParams, bins, scheme=0):
        """Integer moments of every pair i<j: (clnc [npairs][nsteps] uint64,
        the sum over cells of round(c ln c * 2^scale); nnz [npairs][nsteps],
        the non-empty cells; scale)."""
        bins = _c(bins, np.uint8)
        ndof = bins.shape[0]
        npairs = ndof * (ndof - 1) // 2
        clnc = np.zeros((npairs, params.nsteps), np.uint64)
        nnz = np.zeros((npairs, params.nsteps), np.uint32)
        scale = C.c_int(0)
        self.check(self.L.centre_gpu_pair_moments(self.h, C.byref(params), ndof, _ptr(bins),
                                                  int(scheme), _ptr(clnc), _ptr(nnz),
                                                  C.byref(scale)))
        return clnc, nnz, scale.value

    def corr_gemm_dev(self, X, n, K, ldx, R, ldr):
        """R = X X^T on the tensor cores (X: CUDA bf16 [n][ldx], R: CUDA
        float32 [n][ldr])."""
        self.check(self.L.centre_gpu_corr_gemm_dev(self.h, _ptr(X), int(n), int(K), int(ldx),
                                                   _ptr(R), int(ldr)))

    def score(self, params: EntropyParams, types, s1, s2, pairs=None, build_tree=True,
              want_mi=True, mi_out=None):
        types = _c(types, np.uint8)
        s1 = _c(s1, np.float64)
        s2 = _c(s2, np.float64)
        ndof = len(types)
        G = params.nestimators * params.nschemes * params.nsteps
        if pairs is not None:
            pairs = _c(pairs, np.uint32).reshape(-1, 2)
        npairs = s2.shape[0]
        mi = (mi_out if mi_out is not None else np.empty_like(s2)) if want_mi else None
        mie = np.empty((G, SUMS_COLS), np.float64)
        mist = np.empty((G, SUMS_COLS), np.float64) if build_tree else None
        cap = max(ndof - 1, 0)
        tree = np.zeros((G, cap), np.uint32) if build_tree else None
        ntree = np.zeros(G, np.uint32) if build_tree else None
        self.check(self.L.centre_gpu_score(self.h, C.byref(params), ndof, _ptr(types), _ptr(s1),
                                           npairs, _ptr(pairs), _ptr(s2), int(bool(build_tree)),
                                           _ptr(mi), _ptr(mie), _ptr(mist), _ptr(tree),
                                           _ptr(ntree)))
        shp = (params.nestimators, params.nschemes, params.nsteps)
        out = {"mie": mie.reshape(*shp, SUMS_COLS)}
        if want_mi:
            out["mi"] = mi
        if build_tree:
            out["mist"] = mist.reshape(*shp, SUMS_COLS)
            out["tree"] = [tree[g, : ntree[g]].copy() for g in range(G)]
        return out

    # -------------------------------------------------------- device API --
    def discretize_dev(self, bat_type, data, schemes, bins_out, ext_out, bins_ref=None,
                       optimize=True):
        """data: CUDA float32 [ndof][n]; bins_out uint8 [ndof][nsch][n]; ext_out f64 [ndof][4]."""
        sch = _c(schemes, np.uint8)
        ndof, n = int(data.shape[0]), int(data.shape[1])
        ref = int(bins_ref if bins_ref is not None else sch[0])
        self.check(self.L.centre_gpu_discretize_dev(self.h, int(bat_type), _ptr(data), ndof, n,
                                                    _ptr(sch), len(sch), ref,
                                                    int(bool(optimize)), _ptr(bins_out),
                                                    _ptr(ext_out)))

    def entropy1d_dev(self, params, types, bins, ext, s1_out, freq_out=None):
        self.check(self.L.centre_gpu_entropy1d_dev(self.h, C.byref(params), int(bins.shape[0]),
                                                   _ptr(types), _ptr(bins), _ptr(ext),
                                                   _ptr(s1_out), _ptr(freq_out)))

    def entropy2d_dev(self, params, types, bins, ext, s2_out, pairs=None):
        ndof = int(bins.shape[0])
        npairs = int(pairs.shape[0]) if pairs is not None else ndof * (ndof - 1) // 2
        self.check(self.L.centre_gpu_entropy2d_dev(self.h, C.byref(params), ndof, _ptr(types),
                                                   _ptr(bins), _ptr(ext), npairs, _ptr(pairs),
                                                   _ptr(s2_out)))

    def score_dev(self, params, types_dev, s1, s2, pairs=None, build_tree=True, mi_out=None):
        ndof = int(types_dev.shape[0])
        npairs = int(s2.shape[0])
        G = params.nestimators * params.nschemes * params.nsteps
        mie = np.empty((G, SUMS_COLS), np.float64)
        mist = np.empty((G, SUMS_COLS), np.float64)
        cap = max(ndof - 1, 0)
        tree = np.zeros((G, cap), np.uint32)
        ntree = np.zeros(G, np.uint32)
        self.check(self.L.centre_gpu_score_dev(self.h, C.byref(params), ndof, _ptr(types_dev),
                                               _ptr(s1), npairs, _ptr(pairs), _ptr(s2),
                                               int(bool(build_tree)), _ptr(mi_out), _ptr(mie),
                                               _ptr(mist), _ptr(tree), _ptr(ntree)))
        return {"mie": mie, "mist": mist, "tree": [tree[g, : ntree[g]].copy() for g in range(G)]}

    def entropy_batch_dev(self, params, systems, build_tree=True):
        """Score several trajectories in one captured graph.

        systems: list of dicts with CUDA tensors ``types`` uint8 [ndof],
        ``bins`` uint8 [ndof][nsch][nframes], ``ext`` f64 [ndof][4] and
        outputs ``s1`` f64 [ndof][est][sch][steps], ``s2`` f64
        [npairs][est][sch][steps] (all pairs i<j), optional ``mi`` like s2.
        Returns per trajectory {"mie": [G][17], "mist": [G][17] or None}.
        """
        G = params.nestimators * params.nschemes * params.nsteps
        arr = (System * len(systems))()
        keep = []
        for k, sd in enumerate(systems):
            ndof, n = int(sd["bins"].shape[0]), int(sd["bins"].shape[2])
            mie = np.zeros((G, SUMS_COLS), np.float64)
            mist = np.zeros((G, SUMS_COLS), np.float64) if build_tree else None
            keep.append((mie, mist))
            arr[k] = System(ndof, n, *[_addr(x) for x in (
                sd["types"], sd["bins"], sd["ext"], sd["s1"], sd["s2"], sd.get("mi"), mie, mist)])
        self.check(self.L.centre_gpu_entropy_batch_dev(self.h, C.byref(params), len(systems),
                                                       arr))
        return [{"mie": m, "mist": t} for m, t in keep]

    # ---------------------------------------------------------- pair screen --
    def screen_dev(self, params, sparams, types, bins, ext, weights=None):
        """Learned neighbour selection (centre_gpu_screen_dev) on CUDA tensors.
        Returns (pairs: CUDA uint32-as-int32 tensor [npairs][2], weights
        float32 [SCREEN_NPARAMS], losses float32 [epochs])."""
        import torch
        ndof = int(bins.shape[0])
        w = (np.zeros(SCREEN_NPARAMS, np.float32) if weights is None
             else np.ascontiguousarray(weights, np.float32).copy())
        losses = np.zeros(max(int(sparams.epochs), 1), np.float32)
        cap = ndof * int(sparams.nneigh)
        pairs = torch.empty((cap, 2), dtype=torch.int32, device=bins.device)
        n = C.c_uint64(0)
        self.check(self.L.centre_gpu_screen_dev(self.h, C.byref(params), C.byref(sparams), ndof,
                                                _ptr(types), _ptr(bins), _ptr(ext), _ptr(w),
                                                _ptr(losses), cap, _ptr(pairs), C.byref(n)))
        return pairs[: n.value], w, losses[: int(sparams.epochs)]

    def screen_mlp_grad(self, weights, feats, targets):
        """One forward/backward pass of the screen network: (pred, grad, loss)."""
        w = np.ascontiguousarray(weights, np.float32)
        x = np.ascontiguousarray(feats, np.float32)
        y = np.ascontiguousarray(targets, np.float32)
        n = len(y)
        pred = np.empty(n, np.float32)
        grad = np.empty(SCREEN_NPARAMS, np.float32)
        loss = C.c_double(0)
        self.check(self.L.centre_gpu_screen_mlp_grad(self.h, _ptr(w), n, _ptr(x), _ptr(y),
                                                     _ptr(pred), _ptr(grad), C.byref(loss)))
        return pred, grad, loss.value
