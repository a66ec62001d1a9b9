"""CPU oracle for the partitioned-convolution path.

TEST INFRASTRUCTURE ONLY: the reference the GPU path is compared against and
the timed CPU baseline.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` import this package.  The product library
(``partconv_gb300``) never imports, links or calls it.

The C++ restatement lives in ``pc_oracle.cpp`` (see its header for the
reference lines each part follows); this module is a thin ctypes wrapper.
"""
from .oracle import (  # noqa: F401
    build,
    lib,
    layout_check,
    OracleMulti,
    OracleFilter,
    rfft,
    irfft,
    conv_direct_f64,
    run_streams,
    run_leveled,
)
