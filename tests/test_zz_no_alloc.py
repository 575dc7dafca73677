"""The allocation-free gaussian stream entry point.

gic_gaussian_stream_noalloc serves callers that cannot call cudaMalloc (code
that must stay inside another runtime's device-memory pool or budget): they pass
their own device output buffer and stream, and the library uses only a fixed
file-scope device scratch array.  Checked through the C ABI against the
allocating entry point, gic_gaussian_stream, bit for bit, on calls in a row.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, seed, n, stream):
    import torch
    out = torch.full((n,), float('nan'), dtype=torch.float64, device='cuda')
    rc = lib.gic_gaussian_stream_noalloc(seed, n, ctypes.c_void_p(out.data_ptr()),
                                         ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    return rc, out.cpu().numpy()


def test_noalloc_stream_matches_allocating_entry_point(built):
    import torch
    import genetic_gb300 as g
    from genetic_gb300 import _lib
    lib = _lib.load()
    side = torch.cuda.Stream()
    with g.ICGenerator() as gen:
        # calls in a row: a long stream, a short one of another seed (anything
        # left in the shared scratch by the first would show), the largest size
        # the scratch takes, on the default and on a side stream
        for seed, n, stream in ((8896131, 600001, torch.cuda.current_stream()), (42, 1000, side),
                                (7, lib_max(), side), (8896131, 600001, torch.cuda.current_stream())):
            rc, got = _noalloc(lib, seed, n, stream)
            assert rc == _lib.GIC_OK
            assert np.array_equal(got, gen.gaussian_stream(seed, n)), (seed, n)


def lib_max():
    return 1 << 20  # GIC_NOALLOC_MAX_GAUSSIANS


def test_noalloc_rejects_sizes_beyond_its_scratch(built):
    import torch
    from genetic_gb300 import _lib
    lib = _lib.load()
    out = torch.empty(4, dtype=torch.float64, device='cuda')
    too_many = lib_max() + 1
    rc = lib.gic_gaussian_stream_noalloc(1, too_many, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _lib.GIC_ERR_INVALID_ARG
