"""The allocation-free gaussian stream entry point.

gic_gaussian_stream_noalloc serves callers that cannot call cudaMalloc (code
that must stay inside another runtime's device-memory pool or budget): they pass
their own device output buffer and stream, and the library uses only a fixed
file-scope device scratch array.  Checked through the C ABI against the
allocating entry point, gic_gaussian_stream, bit for bit, on two calls in a row.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_stream_matches_allocating_entry_point(built):
    import torch
    import genetic_gb300 as g
    from genetic_gb300 import _lib
    lib = _lib.load()
    stream = torch.cuda.current_stream()
    with g.ICGenerator() as gen:
        # two calls in a row: a long stream, then a short one of another seed,
        # so anything left in the shared scratch by the first would show
        for seed, n in ((8896131, 600001), (42, 1000)):
            out = torch.full((n,), float('nan'), dtype=torch.float64, device='cuda')
            rc = lib.gic_gaussian_stream_noalloc(seed, n, ctypes.c_void_p(out.data_ptr()),
                                                 ctypes.c_void_p(stream.cuda_stream))
            assert rc == _lib.GIC_OK
            torch.cuda.synchronize()
            want = gen.gaussian_stream(seed, n)
            assert np.array_equal(out.cpu().numpy(), want)


def test_noalloc_rejects_sizes_beyond_its_scratch(built):
    import torch
    from genetic_gb300 import _lib
    lib = _lib.load()
    out = torch.empty(4, dtype=torch.float64, device='cuda')
    too_many = (1 << 20) + 1
    rc = lib.gic_gaussian_stream_noalloc(1, too_many, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _lib.GIC_ERR_INVALID_ARG
