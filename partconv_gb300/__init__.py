"""GB300-native multi-level partitioned FFT convolution.

A drop-in for the partitioned-convolution path of ebattenberg/partconv:
``PartConvMulti`` / ``PartConvMultiRelaxed`` over a C ABI
(``include/partconv_gb300.h``) whose kernels are hand-written for sm_103a.
"""
from ._native import PartConvError, PC_INTERLEAVED, PC_PLANAR  # noqa: F401
from .multi import PartConvMulti, PartConvMultiRelaxed, Waiter, check_layout  # noqa: F401


def build(force: bool = False) -> str:
    """Compile the CUDA library in-tree (nvcc, sm_103a)."""
    from . import _build

    return _build.build(force=force)


def library_path() -> str:
    from . import _build

    return _build.LIB_PATH
