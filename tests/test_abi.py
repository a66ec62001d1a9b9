"""The C-ABI library: loads, exports every symbol the header declares, and
its host-side logic (layout validation, argument checks) behaves like the
oracle's.  No compute calls: runs without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle
from partconv_gb300 import _native as nat
from partconv_gb300.multi import check_layout

from conftest import HAS_GPU, ROOT

HEADER = os.path.join(ROOT, "include", "partconv_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pc[fmds]?_[a-z_]+)\s*\(", text)))


def test_header_declares_the_abi():
    names = declared_functions()
    assert "pc_run" in names and "pc_setup_config" in names and "pc_check_layout" in names
    assert set(names) == set(nat.SIGNATURES), "ctypes signatures must mirror the header"


def test_library_exports_every_declared_symbol():
    lib = nat.lib()
    assert os.path.exists(nat.lib_path())
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_status_codes_match_header():
    text = open(HEADER).read()
    for name in ("PC_OK", "PC_ERR_ARG", "PC_ERR_LAYOUT", "PC_ERR_CONFIG", "PC_ERR_IO", "PC_ERR_CUDA",
                 "PC_ERR_NOMEM", "PC_ERR_STATE", "PC_ERR_LIMIT", "PC_INTERLEAVED", "PC_PLANAR", "PC_MAX_BLOCK",
                 "PC_MAX_LEVELS"):
        m = re.search(r"#define\s+%s\s+(\d+)" % name, text)
        assert m and int(m.group(1)) == getattr(nat, name), name


def _random_layout(rng):
    M = int(rng.integers(1, 5))
    n0 = int(2 ** rng.integers(4, 9))
    N = [n0]
    for _ in range(M - 1):
        N.append(N[-1] * int(2 ** rng.integers(1, 4)))
    P = [int(rng.integers(1, 17)) for _ in range(M)]
    s = sum(n * p for n, p in zip(N[:-1], P[:-1]))
    ir_len = int(s + rng.integers(-N[-1], 4 * N[-1]))
    return N, P, max(ir_len, 1)


@pytest.mark.parametrize("relaxed", [False, True])
def test_layout_check_agrees_with_oracle(relaxed):
    rng = np.random.default_rng(11 + relaxed)
    n_ok = 0
    for _ in range(400):
        N, P, L = _random_layout(rng)
        if N[-1] > nat.PC_MAX_BLOCK:
            continue
        a = check_layout(N, P, L, relaxed=relaxed)
        b = oracle.layout_check(N, P, L, relaxed=relaxed)
        assert (a[0] == 0) == (b[0] == 0), (N, P, L, a, b)
        if a[0] == 0:
            n_ok += 1
            assert list(a[1]) == list(b[1])
            assert list(a[2]) == list(b[2])
    assert n_ok > 20


def test_layout_limits():
    # blocks up to 65536 (a 131072-point real transform) are accepted, the
    # next power of two is not
    st, P, _, msg = check_layout([256, 2048, 16384, 65536], [8, 7, 7, 1], 300000)
    assert st == 0 and P[-1] == 3, msg
    st, _, _, msg = check_layout([256, 2048, 16384, 131072], [8, 7, 7, 1], 300000)
    assert st == nat.PC_ERR_LIMIT and "limit" in msg
    st, _, _, msg = check_layout([16] * 17, [1] * 17, 1000)
    assert st == nat.PC_ERR_LIMIT


def test_calls_before_setup_return_errors():
    lib = nat.lib()
    h = lib.pc_create(0)
    assert h
    x = np.zeros(256, np.float32)
    y = np.zeros(256, np.float32)
    assert lib.pc_run(h, y.ctypes.data_as(nat._f32p), x.ctypes.data_as(nat._f32p), 256) == nat.PC_ERR_STATE
    assert b"setup" in lib.pc_last_error(h)
    st = nat.PCRtStats()
    assert lib.pc_rt_drive(h, x.ctypes.data_as(nat._f32p), y.ctypes.data_as(nat._f32p), 256, 0.0, 0,
                           C.byref(st)) != nat.PC_OK
    assert lib.pc_rt_drive(None, x.ctypes.data_as(nat._f32p), y.ctypes.data_as(nat._f32p), 256, 0.0, 0,
                           C.byref(st)) == nat.PC_ERR_ARG
    assert lib.pc_reset(h) == nat.PC_OK
    assert lib.pc_cleanup(h) == nat.PC_OK
    lib.pc_destroy(h)


def test_step_blocks_argument_checks():
    lib = nat.lib()
    h = lib.pc_create(0)
    for k in (1, 2, 4, 8):
        assert lib.pc_set_step_blocks(h, k) == nat.PC_OK
    for k in (0, 3, 16, -1):
        assert lib.pc_set_step_blocks(h, k) == nat.PC_ERR_ARG
    assert b"step blocks" in lib.pc_last_error(h)
    assert lib.pc_set_step_blocks(None, 2) == nat.PC_ERR_ARG
    lib.pc_destroy(h)


def test_setup_config_errors_without_exiting(tmp_path):
    lib = nat.lib()
    h = lib.pc_create(0)
    assert lib.pc_setup_config(h, str(tmp_path / "missing.config").encode(), 1, 0, 0.0) == nat.PC_ERR_CONFIG
    bad = tmp_path / "bad.config"
    bad.write_text("44100 64 1 1\n")
    assert lib.pc_setup_config(h, str(bad).encode(), 1, 0, 0.0) == nat.PC_ERR_CONFIG
    nofile = tmp_path / "nofile.config"
    nofile.write_text("44100 64 1 1 1 1\nmissing.wav 0 0 0 0.2 2 64 6 256\n")
    assert lib.pc_setup_config(h, str(nofile).encode(), 1, 0, 0.0) == nat.PC_ERR_IO
    wrong_n0 = tmp_path / "n0.config"
    wrong_n0.write_text("44100 64 1 1 1 1\nx.wav 0 0 0 0.2 2 128 6 256\n")
    assert lib.pc_setup_config(h, str(wrong_n0).encode(), 1, 0, 0.0) == nat.PC_ERR_CONFIG
    assert b"buffer_size" in lib.pc_last_error(h)
    lib.pc_destroy(h)


@pytest.mark.skipif(HAS_GPU, reason="checks the no-device error path")
def test_setup_without_device_fails_cleanly():
    from partconv_gb300 import PartConvMulti, PartConvError

    m = PartConvMulti()
    with pytest.raises(PartConvError) as ei:
        m.setup_layout(48000, 64, 1, 1, [dict(ir=np.ones(300, np.float32), N=[64, 128], P=[2, 0])])
    assert ei.value.code == nat.PC_ERR_CUDA
