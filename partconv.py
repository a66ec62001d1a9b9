"""``import partconv``: the module name of the reference's Python binding
(``%module partconv``, src/partconv.i:3) bound to the GB300 engine.

Scripts written against the reference module (src/tune.py:2 does
``import partconv``) run unchanged with this repository on ``sys.path``: every
name comes from ``partconv_gb300.partconv`` -- ``PartConvFilter``,
``PartConvMax``, ``DelayBuffer``, ``DoubleBuffer``, ``intArray``,
``doubleArray`` and ``PartConvMulti``.
"""
from partconv_gb300.partconv import (  # noqa: F401
    DelayBuffer,
    DoubleBuffer,
    PartConvError,
    PartConvFilter,
    PartConvMax,
    PartConvMulti,
    PartConvMultiRelaxed,
    Waiter,
    doubleArray,
    intArray,
)

__all__ = ["PartConvFilter", "PartConvMax", "DelayBuffer", "DoubleBuffer", "intArray", "doubleArray",
           "PartConvMulti", "PartConvMultiRelaxed", "Waiter", "PartConvError"]
