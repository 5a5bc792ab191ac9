"""Drop-in replacement for dadi's `dadi.cuda` package.

`dadi_gb300.install()` registers this package as `dadi.cuda`, after which
`dadi.cuda_enabled(True)` (dadi/__init__.py:30-48, which only does
`from . import cuda`) succeeds and dadi's Integration functions route their
CUDA branches (dadi/Integration.py:340-345, 496-502, 663-669, 1101-1106,
1223-1229) to the sm_103a kernels through `dadi.cuda.Integration`.  Unlike the
reference backend (dadi/cuda/__init__.py:1-35) nothing here creates a CUDA
context, library handle or global state at import.
"""
from . import Integration  # noqa: F401


def transpose_gpuarray(in_gpu, out_gpu):
    """dadi.cuda.transpose_gpuarray (dadi/cuda/__init__.py:22-28): out_gpu =
    in_gpu transposed, for 2-D device arrays (CUDA tensors here, PyCUDA
    gpuarrays in the reference); ValueError unless out_gpu is (M, L) for an
    (L, M) input."""
    L, M = in_gpu.shape
    if tuple(out_gpu.shape) != (M, L):
        raise ValueError
    out_gpu.copy_(in_gpu.t())
