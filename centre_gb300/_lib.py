"""ctypes binding of libcentre_gpu.so (C ABI in include/centre_gpu.h).

The library is built in-tree by ``centre_gb300.build``.  There is no CPU
fallback: if the library is missing or no sm_103 device is present, calls
raise ``CentreError``.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# CENTRE_GPU_LIB names another build of the library (e.g. one compiled with
# different tuning macros); the default is the in-tree build.
LIB_PATH = os.environ.get("CENTRE_GPU_LIB") or os.path.join(HERE, "libcentre_gpu.so")

SUMS_COLS = 17
SUMS_NAMES = ["BOND-S1", "ANGLE-S1", "DIHED-S1", "B/B-S2", "B/B-I2", "A/A-S2", "A/A-I2",
              "D/D-S2", "D/D-I2", "B/A-S2", "B/A-I2", "B/D-S2", "B/D-I2", "A/D-S2", "A/D-I2",
              "S1", "S2"]

COUNTS_AUTO, COUNTS_ATOMIC, COUNTS_TC = 0, 1, 2


class CentreError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"centre_gpu error {status}: {msg}")
        self.status = status


class System(C.Structure):
    """One trajectory of a batch (centre_system)."""
    _fields_ = [
        ("ndof", C.c_uint32),
        ("nframes", C.c_uint64),
        ("types", C.c_void_p),
        ("bins", C.c_void_p),
        ("extremes", C.c_void_p),
        ("s1", C.c_void_p),
        ("s2", C.c_void_p),
        ("mi", C.c_void_p),
        ("mie_sums", C.c_void_p),
        ("mist_sums", C.c_void_p),
    ]


class ScreenParams(C.Structure):
    """centre_screen_params: learned pair screen."""
    _fields_ = [
        ("feat_div", C.c_uint32),
        ("ntrain", C.c_uint32),
        ("nprefilter", C.c_uint32),
        ("nneigh", C.c_uint32),
        ("epochs", C.c_uint32),
        ("batch", C.c_uint32),
        ("lr", C.c_float),
        ("train", C.c_uint8),
        ("init_weights", C.c_uint8),
        ("seed", C.c_uint64),
    ]


SCREEN_NPARAMS = 5057


def make_screen_params(feat_div=5, ntrain=200_000, nprefilter=256, nneigh=64, epochs=3,
                       batch=4096, lr=2e-3, train=True, init_weights=True, seed=1):
    return ScreenParams(int(feat_div), int(ntrain), int(nprefilter), int(nneigh), int(epochs),
                        int(batch), float(lr), 1 if train else 0, 1 if init_weights else 0,
                        int(seed))


class EntropyParams(C.Structure):
    _fields_ = [
        ("nframes", C.c_uint64),
        ("nsteps", C.c_uint8),
        ("nschemes", C.c_uint8),
        ("nestimators", C.c_uint8),
        ("jacobian", C.c_uint8),
        ("kde", C.c_uint8),
        ("counts_form", C.c_uint8),
        ("bin_schemes", C.c_uint8 * 16),
        ("estimators", C.c_uint8 * 4),
    ]


def make_params(nframes, nsteps, schemes, estimators=(0,), jacobian=True, kde=False,
                counts_form=COUNTS_AUTO) -> EntropyParams:
    p = EntropyParams()
    p.nframes = int(nframes)
    p.nsteps = int(nsteps)
    p.nschemes = len(schemes)
    p.nestimators = len(estimators)
    p.jacobian = 1 if jacobian else 0
    p.kde = 1 if kde else 0
    p.counts_form = int(counts_form)
    for i, s in enumerate(schemes):
        p.bin_schemes[i] = int(s)
    for i, e in enumerate(estimators):
        p.estimators[i] = int(e)
    return p


_vp = C.c_void_p
_SIGS = {
    "centre_gpu_create": (C.c_int, [C.POINTER(_vp), C.c_int]),
    "centre_gpu_destroy": (None, [_vp]),
    "centre_gpu_strerror": (C.c_char_p, [C.c_int]),
    "centre_gpu_last_error": (C.c_char_p, [_vp]),
    "centre_gpu_set_stream": (C.c_int, [_vp, _vp]),
    "centre_gpu_synchronize": (C.c_int, [_vp]),
    "centre_gpu_launch_count": (C.c_uint64, [_vp]),
    "centre_gpu_enable_timing": (C.c_int, [_vp, C.c_int]),
    "centre_gpu_timer": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]),
    "centre_gpu_discretize": (C.c_int, [_vp, C.c_int, _vp, C.c_uint32, C.c_uint64, _vp,
                                        C.c_uint32, C.c_uint8, C.c_int, _vp, _vp]),
    "centre_gpu_discretize_dev": (C.c_int, [_vp, C.c_int, _vp, C.c_uint32, C.c_uint64, _vp,
                                            C.c_uint32, C.c_uint8, C.c_int, _vp, _vp]),
    "centre_gpu_discretize_vmkde": (C.c_int, [_vp, _vp, C.c_uint32, C.c_uint64, C.c_uint8,
                                              C.c_double, C.c_uint32, C.c_double, C.c_uint32,
                                              _vp, _vp, _vp]),
    "centre_gpu_df_exp_eval": (C.c_int, [_vp, _vp, C.c_uint64, _vp]),
    "centre_gpu_discretize_gridkde": (C.c_int, [_vp, C.c_int, _vp, C.c_uint32, C.c_uint64,
                                                C.c_uint32, C.c_double, _vp, _vp, _vp, _vp]),
    "centre_gpu_discretize_gridkde_dev": (C.c_int, [_vp, C.c_int, _vp, C.c_uint32, C.c_uint64,
                                                    C.c_uint32, C.c_double, _vp, _vp, _vp,
                                                    _vp]),
    "centre_gpu_entropy1d": (C.c_int, [_vp, C.POINTER(EntropyParams), C.c_uint32, _vp, _vp,
                                       _vp, _vp, _vp]),
    "centre_gpu_entropy1d_dev": (C.c_int, [_vp, C.POINTER(EntropyParams), C.c_uint32, _vp, _vp,
                                           _vp, _vp, _vp]),
    "centre_gpu_entropy2d": (C.c_int, [_vp, C.POINTER(EntropyParams), C.c_uint32, _vp, _vp,
                                       _vp, C.c_uint64, _vp, _vp]),
    "centre_gpu_entropy2d_dev": (C.c_int, [_vp, C.POINTER(EntropyParams), C.c_uint32, _vp,
                                           _vp, _vp, C.c_uint64, _vp, _vp]),
    "centre_gpu_entropy2d_static": (C.c_int, [C.POINTER(EntropyParams), C.c_uint32, _vp, _vp,
                                              _vp, _vp, _vp]),
    "centre_gpu_counts2d": (C.c_int, [_vp, C.POINTER(EntropyParams), C.c_uint32, _vp,
                                      C.c_uint64, _vp, _vp]),
    "centre_gpu_pair_moments": (C.c_int, [_vp, C.POINTER(EntropyParams), C.c_uint32, _vp,
                                          C.c_int, _vp, _vp, _vp]),
    "centre_gpu_corr_gemm_dev": (C.c_int, [_vp, _vp, C.c_uint32, C.c_uint32, C.c_uint32, _vp,
                                           C.c_uint32]),
    "centre_gpu_score": (C.c_int, [_vp, C.POINTER(EntropyParams), C.c_uint32, _vp, _vp,
                                   C.c_uint64, _vp, _vp, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    "centre_gpu_score_dev": (C.c_int, [_vp, C.POINTER(EntropyParams), C.c_uint32, _vp, _vp,
                                       C.c_uint64, _vp, _vp, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    "centre_gpu_entropy_batch_dev": (C.c_int, [_vp, C.POINTER(EntropyParams), C.c_uint32,
                                               C.POINTER(System)]),
    "centre_gpu_screen_dev": (C.c_int, [_vp, C.POINTER(EntropyParams), C.POINTER(ScreenParams),
                                        C.c_uint32, _vp, _vp, _vp, _vp, _vp, C.c_uint64, _vp,
                                        C.POINTER(C.c_uint64)]),
    "centre_gpu_screen": (C.c_int, [_vp, C.POINTER(EntropyParams), C.POINTER(ScreenParams),
                                    C.c_uint32, _vp, _vp, _vp, _vp, _vp, C.c_uint64, _vp,
                                    C.POINTER(C.c_uint64)]),
    "centre_gpu_screen_mlp_grad": (C.c_int, [_vp, _vp, C.c_uint64, _vp, _vp, _vp, _vp,
                                             C.POINTER(C.c_double)]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load the library and declare every C-ABI signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise CentreError(-7, f"{path} is missing: build it with "
                              "`python -m centre_gb300.build` (nvcc, sm_103a)")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    return list(_SIGS)
