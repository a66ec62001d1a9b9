"""The drop-in boundary: pc.config + WAV set-up, the C++ PartConvMulti shim
(include/partconvMulti.h) and the Python ``partconv`` module surface."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from partconv_gb300 import _native as nat
from partconv_gb300 import partconv
from partconv_gb300 import workloads as wl

from conftest import HAS_GPU, ROOT
from wavutil import write_config, write_wav

TOL = 1e-5


# ---------------------------------------------------------------- C++ shim
@pytest.fixture(scope="module")
def cpp_driver(tmp_path_factory):
    lib = nat.lib()   # builds the library
    out = tmp_path_factory.mktemp("cpp") / "pcm_driver"
    libdir = os.path.dirname(nat.lib_path())
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests/cpp/pcm_driver.cpp"),
           "-L", libdir, "-lpartconv_gb300", f"-Wl,-rpath,{libdir}", "-pthread", "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True)
    assert lib is not None
    return str(out)


def test_cpp_shim_builds_and_reports_errors(cpp_driver, tmp_path):
    r = subprocess.run([cpp_driver, str(tmp_path / "none.config"), "x", "y"], capture_output=True, text=True)
    assert r.returncode == 10 + nat.PC_ERR_CONFIG
    assert "Unable to open config file" in r.stderr
    cfg = tmp_path / "pc.config"
    cfg.write_text("48000 64 1 1 1 1\nmissing.wav 0 0 0 0.5 2 64 4 256\n")
    r = subprocess.run([cpp_driver, str(cfg), "x", "y"], capture_output=True, text=True)
    assert r.returncode == 10 + nat.PC_ERR_IO


def _config_case(tmp_path, rng):
    """Two inputs, three outputs, IRs in three WAV encodings, a muted PC, a
    repeat line, a PC without its last part count."""
    h1 = 0.5 * wl.decaying_ir(rng, 3000, 0.2)
    h2 = 0.5 * wl.decaying_ir(rng, 9000, 0.3)
    h3 = 0.5 * wl.decaying_ir(rng, 1200, 0.1)
    b1 = write_wav(tmp_path / "a.wav", np.stack([h1, -h1], 1), fmt="pcm16")   # stereo: channel 0 is used
    b2 = write_wav(tmp_path / "b.wav", h2, fmt="pcm24")
    b3 = write_wav(tmp_path / "c.wav", h3, fmt="float32")
    pcs = [dict(file="a.wav", in_ch=0, out_ch=0, scale=0.5, N=[64, 256], P=[4, 0]),
           dict(file="b.wav", in_ch=1, out_ch=0, scale=1.5, N=[64, 256, 1024], P=[4, 3, 0]),
           dict(file="c.wav", in_ch=1, out_ch=2, scale=-1.0, mute=0, N=[64], P=[0]),
           dict(file="a.wav", in_ch=0, out_ch=1, scale=1.0, mute=1, N=[64, 512], P=[8, 0])]
    write_config(tmp_path / "pc.config", 48000, 64, 2, 3, pcs, repeats=2, drop_last_parts=True)
    decoded = {"a.wav": b1, "b.wav": b2, "c.wav": b3}
    opcs = []
    for rep in range(2):
        for p in pcs:
            opcs.append(dict(ir=decoded[p["file"]], N=p["N"], P=p["P"], in_ch=p["in_ch"], out_ch=p["out_ch"],
                             scale=p["scale"], mute=1 if rep else p.get("mute", 0)))
    frames = 64 * 300
    x = (0.1 * rng.standard_normal((frames, 2))).astype(np.float32)
    return tmp_path / "pc.config", x, opcs


@pytest.mark.gpu
@pytest.mark.parametrize("relaxed", [0, 1])
def test_cpp_shim_config_run_matches_oracle(gpu, cpp_driver, tmp_path, relaxed):
    cfg, x, opcs = _config_case(tmp_path, np.random.default_rng(31))
    x.tofile(tmp_path / "in.f32")
    r = subprocess.run([cpp_driver, str(cfg), str(tmp_path / "in.f32"), str(tmp_path / "out.f32"), str(relaxed)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    y = np.fromfile(tmp_path / "out.f32", np.float32).reshape(-1, 3)
    ref = oracle.OracleMulti(64, 2, 3, opcs, relaxed=bool(relaxed)).run(x)
    for o in range(3):
        if np.abs(ref[:, o]).max() == 0:
            assert np.all(y[:, o] == 0)
        else:
            assert wl.rel_l2(y[:, o], ref[:, o]) <= TOL


@pytest.mark.gpu
def test_python_setup_from_config(gpu, tmp_path):
    cfg, x, opcs = _config_case(tmp_path, np.random.default_rng(32))
    m = partconv.PartConvMulti()
    assert m.setup(str(cfg)) == 0
    assert (m.buffer_size, m.numInputChannels, m.numOutputChannels, m.FS) == (64, 2, 3, 48000)
    assert m.max_block_size == 1024
    N, P = m.layout(1)
    assert N == [64, 256, 1024] and P[-1] == int(np.ceil((9000 - 64 * 4 - 256 * 3) / 1024))
    y = m.process(x)
    ref = oracle.OracleMulti(64, 2, 3, opcs).run(x)
    assert wl.rel_l2(y[:, 0], ref[:, 0]) <= TOL and wl.rel_l2(y[:, 2], ref[:, 2]) <= TOL


# ------------------------------------------------------- Python partconv module
def test_carrays():
    a = partconv.intArray(4)
    for i in range(4):
        a[i] = 3 * i
    assert [a[i] for i in range(4)] == [0, 3, 6, 9] and len(a) == 4
    d = partconv.doubleArray(3)
    d[2] = 1.5
    assert d[2] == 1.5 and d[0] == 0.0


def test_filter_rejects_strict_violations_like_reference():
    # PartConvFilter::setup returns 1 (partconv.cpp:148-166) -- no GPU needed
    f = partconv.PartConvFilter()
    N = partconv.intArray(3)
    P = partconv.intArray(3)
    for i, (n, p) in enumerate([(256, 8), (2048, 7), (16384, 7)]):
        N[i], P[i] = n, p
    assert f.setup(3, N, P, np.ones(131072, np.float32)) == 1
    assert "sufficient delay" in f.last_error


@pytest.mark.gpu
@pytest.mark.parametrize("N,P,L", [([64, 256, 1024], [6, 6, 0], 6000), ([128, 512, 4096], [14, 14, 0], 20000),
                                   ([256], [0], 3000)])
def test_filter_fine_grained_matches_oracle(gpu, N, P, L):
    rng = np.random.default_rng(L)
    h = wl.decaying_ir(rng, L, 0.2)
    f = partconv.PartConvFilter()
    assert f.setup(len(N), N, P, h) == 0
    o = oracle.OracleFilter(N, P, h)
    assert list(f.num_parts) == list(o.num_parts)
    N0 = N[0]
    ys, rs, yr, rr = [], [], [], []
    x = (0.1 * rng.standard_normal(N0 * (L // N0 + 3 * N[-1] // N0 + 8))).astype(np.float32)
    for relaxed in (0, 1):
        f.reset()
        o.reset()
        for b in range(len(x) // N0):
            blk = x[b * N0:(b + 1) * N0]
            if relaxed:
                f.sync_levels_relaxed()
                o.sync_levels_relaxed()
                yr.append(f.output_relaxed())
                rr.append(o.output_relaxed())
            else:
                f.sync_levels()
                o.sync_levels()
            f.input(blk)
            o.input(blk)
            for lv in range(len(N)):
                if b % (N[lv] // N0) == 0:
                    f.runLevel(lv)
                    o.runLevel(lv)
            if not relaxed:
                ys.append(f.output())
                rs.append(o.output())
    y, r = np.concatenate(ys), np.concatenate(rs)
    assert wl.rel_l2(y, r) <= TOL
    assert wl.rel_l2(y, wl.conv_fp64(x, h, len(x))) <= TOL
    assert wl.rel_l2(np.concatenate(yr), np.concatenate(rr)) <= TOL


@pytest.mark.gpu
def test_filter_bench_like_tune_py(gpu):
    # src/tune.py:21-55: setup with no IR, bench every level, cleanup
    f = partconv.PartConvFilter()
    f.FS = 44100
    N, P = partconv.intArray(2), partconv.intArray(2)
    N[0], P[0], N[1], P[1] = 64, 6, 256, 4
    assert f.setup(2, N, P, None, 2, "wisdom.wis") == 0
    load = partconv.doubleArray(3)
    for lv in range(2):
        t = f.bench(lv, 200, 3, 0.1)
        assert 0 < t < 0.1
        load[lv] = t * 100 * 44100 / N[lv]
    assert load[0] > 0 and load[1] > 0
    assert f.cleanup() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("n,m,k", [(2, 2, 2), (3, 3, 1), (2, 6, 3)])
def test_partconvmax_channel_modes(gpu, n, m, k):
    rng = np.random.default_rng(n * 10 + k)
    L = 5000
    imp = np.stack([wl.decaying_ir(rng, L, 0.2) for _ in range(k)]).astype(np.float32)
    pm = partconv.PartConvMax()
    assert pm.setup(48000, n, m, k, imp.ravel(), L, 1, [64, 256, 1024], 3, 1) == 0
    # the mapping of partconv.cpp:661-708 and the part counts of :718-728
    if n == m == k:
        pairs = [(i, i, i) for i in range(k)]
    elif k == 1:
        pairs = [(0, j, j) for j in range(n)]
    else:
        pairs = [(i, j, i * n + j) for i in range(k) for j in range(n)]
    N, P = [64, 256, 1024], [2 * 256 // 64 - 2, 2 * 1024 // 256 - 2, 0]
    frames = 64 * 200
    x = (0.1 * rng.standard_normal((frames, n))).astype(np.float32)
    ys = []
    outs = [np.zeros(64, np.float32) for _ in range(m)]
    for b in range(frames // 64):
        pm.run(outs, [x[b * 64:(b + 1) * 64, j] for j in range(n)])
        ys.append(np.stack(outs, 1).copy())
    y = np.concatenate(ys)
    ref = oracle.OracleMulti(64, n, m, [dict(ir=imp[i], N=N, P=P, in_ch=ic, out_ch=oc) for i, ic, oc in pairs]).run(x)
    for o in range(m):
        assert wl.rel_l2(y[:, o], ref[:, o]) <= TOL
    assert pm.frameNum == frames // 64


def test_partconvmax_rejects_unsupported_modes():
    assert partconv.PartConvMax().setup(48000, 2, 3, 2, np.zeros(20, np.float32), 10, 1, [64, 256], 2, 1) == 1


@pytest.mark.gpu
def test_delay_and_double_buffer_semantics(gpu):
    # DelayBuffer(frameSize, blockSize, delay): blocks come out delay -
    # framesPerBlock - 1 frames late (partconv.cpp:1401-1472)
    db = partconv.DelayBuffer(4, 2, 5)
    frames = [np.full(4, i + 1, np.float32) for i in range(12)]
    got = []
    for i, fr in enumerate(frames):
        db.write(fr)
        if i % 2 == 0:
            db.prepNextRead()
            got.append(db.read()[::4].tolist())
    # readFrameDelay = 2: after writing frame i (value i+1) the block read
    # holds frames i-2 and i-1 (zeros before the first writes)
    assert got == [[0, 0], [1, 2], [3, 4], [5, 6], [7, 8], [9, 10]]
    d2 = partconv.DelayBuffer(4, 1, 2)   # 3 one-frame blocks: read 2, write 0
    d2.prepNextRead()                    # read block 0 == write block 0
    with pytest.raises(partconv.PartConvError):
        d2.read()
    dbuf = partconv.DoubleBuffer(8)
    dbuf.getWriteBuffer().fill_(2.0)
    assert float(dbuf.getReadBuffer().sum()) == 0.0
    dbuf.swap()
    assert float(dbuf.getReadBuffer().sum()) == 16.0
    dbuf.reset()
    assert float(dbuf.getReadBuffer().sum()) == 0.0


def test_top_level_partconv_module_name():
    """``import partconv`` -- the reference binding's module name
    (src/partconv.i:3), imported by src/tune.py:2 -- gives the same classes as
    partconv_gb300.partconv."""
    import importlib

    top = importlib.import_module("partconv")
    for name in ("PartConvFilter", "PartConvMax", "DelayBuffer", "DoubleBuffer", "intArray", "doubleArray",
                 "PartConvMulti"):
        assert getattr(top, name) is getattr(partconv, name)
    a = top.intArray(4)
    a[2] = 7
    assert a[2] == 7 and top.doubleArray(2)[1] == 0.0


def test_waiter_signals_across_threads():
    """Waiter (src/partconvMulti.h:152-165): waitFor returns once another
    thread has changed the value to the target, and times out otherwise."""
    import threading

    from partconv_gb300.multi import Waiter

    w = Waiter(0)
    assert not w.waitFor(1, timeout=0.01)
    t = threading.Timer(0.05, w.changeAndSignal, args=(1,))
    t.start()
    assert w.waitFor(1, timeout=5.0)
    t.join()
    w.changeAndSignal(2)
    assert w.waitFor(2, timeout=0.01) and not w.waitFor(1, timeout=0.01)
