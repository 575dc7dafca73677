"""GB300-native implementation of genetIC's field-realisation hot path.

The CUDA kernels and the C ABI live in libgicgpu.so (built by build.py);
`ICGenerator` drives them with genetIC's paramfile vocabulary.
"""
from .generator import ICGenerator, run_paramfile  # noqa: F401
from ._lib import GicError  # noqa: F401
from . import transfer  # noqa: F401
