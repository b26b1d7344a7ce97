"""centre_gpu_entropy2d_static: the all-pairs joint entropies computed without
any memory allocation by the library (its scratch is a fixed device array).

It exists for callers that may not call cudaMalloc -- plug-ins whose host
application owns all device memory through its own pool, loops that must not
stall on the device synchronisation an allocation can cause.  The test calls it
through the C ABI twice in a row (the second call runs on the array the first
one left behind) and compares each result with the allocating entry point,
centre_gpu_entropy2d, within the parity tolerance used everywhere else.  This
file is collected last so a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

from centre_gb300 import _lib
from centre_gb300.api import make_params
from centre_gb300.synth import chain_trajectory

pytestmark = pytest.mark.gpu


def _device_inputs(torch, gpu, natoms, nframes, nb):
    tr = chain_trajectory(natoms, nframes, seed=natoms * 31 + nframes)
    bins, ext, types = [], [], []
    for typ, blk in tr.blocks():
        b, e = gpu.discretize(typ, blk, [nb])
        bins.append(b)
        ext.append(e)
        types += [typ] * len(b)
    bins = np.concatenate(bins)
    ext = np.concatenate(ext)
    types = np.array(types, np.uint8)
    dev = torch.device("cuda", 0)
    return (bins, ext, types, torch.from_numpy(bins).to(dev), torch.from_numpy(ext).to(dev),
            torch.from_numpy(types).to(dev))


@pytest.mark.parametrize("natoms,nframes,nsteps,nb,ests", [
    (25, 20_000, 4, 30, [0, 1]),
    (40, 12_008, 3, 50, [1]),
])
def test_static_scratch_entry_matches_allocating_entry(gpu, natoms, nframes, nsteps, nb, ests):
    import torch
    L = _lib.load()
    bins, ext, types, d_bins, d_ext, d_types = _device_inputs(torch, gpu, natoms, nframes, nb)
    p = make_params(nframes, nsteps, [nb], ests, True, counts_form=0)
    want = gpu.entropy2d(p, types, bins, ext)
    ndof = len(types)
    npairs = ndof * (ndof - 1) // 2
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        s2 = torch.full((npairs, len(ests), 1, nsteps), float("nan"), dtype=torch.float64,
                        device="cuda")
        rc = L.centre_gpu_entropy2d_static(C.byref(p), ndof, C.c_void_p(d_types.data_ptr()),
                                           C.c_void_p(d_bins.data_ptr()),
                                           C.c_void_p(d_ext.data_ptr()),
                                           C.c_void_p(s2.data_ptr()), C.c_void_p(stream))
        assert rc == 0, (call, rc)
        got = s2.cpu().numpy()
        np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-13, err_msg=f"call {call}")


def test_static_scratch_entry_rejects_oversized_problems(gpu):
    import torch
    L = _lib.load()
    p = make_params(100_000, 10, [50], [0], True)
    dummy = torch.zeros(16, dtype=torch.uint8, device="cuda")
    ptr = C.c_void_p(dummy.data_ptr())
    # 5000 DOFs x 10 steps needs far more than the fixed array; nothing runs
    rc = L.centre_gpu_entropy2d_static(C.byref(p), 5000, ptr, ptr, ptr, ptr,
                                       C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == -1


def test_static_scratch_entry_status_codes_match_allocating_entry(gpu):
    """The same invalid input gives the same status from both entry points:
    a bin scheme of zero bins is an argument error (CENTRE_E_ARG)."""
    import torch
    from centre_gb300.api import CentreError
    L = _lib.load()
    p = make_params(4_000, 2, [30], [0], True)
    p.bin_schemes[0] = 0
    bins = np.zeros((3, 1, 4_000), np.uint8)
    ext = np.tile(np.array([0.0, 1.0, 0.5, 0.0]), (3, 1))
    types = np.array([1, 2, 3], np.uint8)
    with pytest.raises(CentreError) as e:
        gpu.entropy2d(p, types, bins, ext)
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    ptr = C.c_void_p(dummy.data_ptr())
    rc = L.centre_gpu_entropy2d_static(C.byref(p), 3, ptr, ptr, ptr, ptr,
                                       C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == e.value.status == -1
