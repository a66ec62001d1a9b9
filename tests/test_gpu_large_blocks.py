"""Levels with blocks above 16384 samples (up to 65536: a 131072-point real
transform), which the engine runs on a cluster of 8 CTAs per fire.

The reference accepts any power-of-two block (src/partconv.cpp:87-103), and
its own src/pc.config uses top levels of 65536 and 32768.  These tests run
config lines of that file unmodified through pc_setup_config (with seeded IR
WAV files of the format of the reference's reverbs/ recordings: 16-bit PCM,
stereo, 44.1 kHz, 661500 frames) and random layouts with large top levels,
against the oracle (relative L2 <= 1e-5 per output channel)."""
import numpy as np
import pytest

import oracle
from partconv_gb300 import PartConvMulti, PartConvMultiRelaxed
from partconv_gb300 import workloads as wl
from wavutil import write_wav

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _reverb_wav(path, seed, frames=661500, fs=44100):
    """A decaying-noise stereo recording stand-in; returns channel 0 as the
    engine's WAV reader must recover it."""
    rng = np.random.default_rng(seed)
    h = wl.decaying_ir(rng, frames, 3.0, fs=fs).astype(np.float64)
    h *= 0.9 / np.max(np.abs(h))
    return write_wav(path, np.stack([h, -0.5 * h], 1), fs=fs, fmt="pcm16")


# src/pc.config of the reference: its header line, line 2 (top level 65536)
# and lines 16-17 (top level 32768, two channels), as written there
CONFIG_65536 = ("44100 64 1 1 1 30 \n"
                "../reverbs/hamilton_mausoleum.wav 0 0 0 0.2 6 64 6 256 6 1024 6 4096 6 16384 6 65536 9\n")
CONFIG_32768 = ("44100 64 2 2 2 1\n"
                "../reverbs/hamilton_mausoleum.wav 0 0 0 0.2 4 64 14 512 14 4096 14 32768 19\n"
                "../reverbs/hamilton_mausoleum.wav 0 1 1 0.2 4 64 14 512 14 4096 14 32768 19 Garcia's\n")


@pytest.mark.parametrize("text,layout,n_ch", [
    (CONFIG_65536, ([64, 256, 1024, 4096, 16384, 65536], [6, 6, 6, 6, 6, 9]), 1),
    (CONFIG_32768, ([64, 512, 4096, 32768], [14, 14, 14, 19]), 2),
])
def test_reference_config_lines_run_through_setup_config(gpu, tmp_path, text, layout, n_ch):
    (tmp_path / "reverbs").mkdir()
    (tmp_path / "src").mkdir()
    h = _reverb_wav(tmp_path / "reverbs" / "hamilton_mausoleum.wav", 11)
    cfg = tmp_path / "src" / "pc.config"
    cfg.write_text(text)
    m = PartConvMulti()
    m.setup(str(cfg))
    info = m.info()
    assert info.buffer_size == 64 and info.max_block_size == layout[0][-1]
    Ns, Ps = m.layout(0)
    assert list(Ns) == layout[0] and list(Ps) == layout[1]
    rng = np.random.default_rng(12)
    n_x = 64 * 64
    frames = -(-(n_x + len(h)) // 64) * 64
    x = np.zeros((frames, n_ch), np.float32)
    x[:n_x] = (0.1 * rng.standard_normal((n_x, n_ch))).astype(np.float32)
    y = m.process(x)
    pcs = [dict(ir=h, N=layout[0], P=layout[1], in_ch=c, out_ch=c, scale=0.2) for c in range(n_ch)]
    ref = oracle.OracleMulti(64, n_ch, n_ch, pcs).run(x)
    for c in range(n_ch):
        err = _rel(y[:, c], ref[:, c])
        print(f"config top {layout[0][-1]} channel {c}: rel L2 vs oracle {err:.2e}")
        assert err <= TOL


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_large_top_levels_match_oracle(gpu, seed):
    """Two or three PCs per handle with relaxed or strict layouts whose top
    level is 32768 or 65536, mixed into two outputs; pc_run block by block and
    pc_process give the same bits; the Relaxed variant is one block later."""
    rng = np.random.default_rng(100 + seed)
    N0 = int(rng.choice([128, 256]))
    pcs = []
    for i in range(int(rng.integers(2, 4))):
        top = int(rng.choice([32768, 65536]))
        strict = bool(rng.integers(0, 2))
        N = [N0]
        while N[-1] < top:
            N.append(min(top, N[-1] * int(rng.choice([4, 8]))))
        P, s = [], 0
        for L_ in range(len(N) - 1):   # enough parts for the next level's slack, plus 0..2
            target = 2 * N[L_ + 1] - 2 * N0 if strict else N[L_ + 1]
            p = max(1, -(-(target - s) // N[L_])) + int(rng.integers(0, 3))
            P.append(p)
            s += N[L_] * p
        P.append(1)
        L = s + int(rng.integers(1, 2 * top))
        pcs.append(dict(ir=wl.decaying_ir(rng, L, float(rng.uniform(0.3, 2.0))), N=N, P=P, in_ch=i % 2,
                        out_ch=int(rng.integers(0, 2)), scale=float(rng.uniform(0.5, 1.5))))
    L = max(len(p["ir"]) for p in pcs)
    frames = -(-(L + 8 * N0) // N0) * N0
    x = np.zeros((frames, 2), np.float32)
    x[:8 * N0] = (0.1 * rng.standard_normal((8 * N0, 2))).astype(np.float32)
    m = PartConvMulti()
    m.setup_layout(48000, N0, 2, 2, pcs)
    pcs = [p | dict(P=list(m.layout(i)[1])) for i, p in enumerate(pcs)]
    y = m.process(x)
    ref = oracle.OracleMulti(N0, 2, 2, pcs).run(x)
    for o in range(2):
        if not np.any(ref[:, o]):
            assert not np.any(y[:, o])
            continue
        err = _rel(y[:, o], ref[:, o])
        print(f"seed {seed} output {o}: rel L2 vs oracle {err:.2e}")
        assert err <= TOL
    # block by block: the same bits
    m.reset()
    yb = np.zeros_like(y)
    out = np.zeros(N0 * 2, np.float32)
    for b in range(frames // N0):
        m.run(out, np.ascontiguousarray(x[b * N0:(b + 1) * N0]), N0)
        yb[b * N0:(b + 1) * N0] = out.reshape(N0, 2)
    assert np.array_equal(yb, y)
    r = PartConvMultiRelaxed()
    r.setup_layout(48000, N0, 2, 2, pcs)
    yr = r.process(x)
    assert np.array_equal(yr[N0:], y[:-N0]) and not np.any(yr[:N0])


def test_large_top_level_with_four_blocks_per_step(gpu):
    """Several base blocks per step: the 65536 level's fires run deferred
    beside the steps."""
    rng = np.random.default_rng(7)
    N, P = [256, 2048, 16384, 65536], [14, 14, 14, 1]
    h = wl.decaying_ir(rng, 300000, 2.0)
    pcs = [dict(ir=h, N=N, P=P)]
    frames = -(-(len(h) + 4096) // 1024) * 1024
    x = np.zeros((frames, 1), np.float32)
    x[:4096] = (0.1 * rng.standard_normal((4096, 1))).astype(np.float32)
    m = PartConvMulti(step_blocks=4)
    m.setup_layout(48000, 256, 1, 1, pcs)
    assert m.info().step_blocks == 4
    y = m.process(x)
    pcs[0]["P"] = list(m.layout(0)[1])
    ref = oracle.OracleMulti(256, 1, 1, pcs).run(x)
    assert _rel(y[:, 0], ref[:, 0]) <= TOL


@pytest.mark.parametrize("N,P,L", [([1024, 4096, 16384, 32768], [6, 6, 2, 0], 130000),
                                   ([4096, 16384, 65536], [6, 6, 0], 254000)])
def test_filter_large_levels_match_oracle(gpu, N, P, L):
    """PartConvFilter (the fine-grained API tune.py drives) with levels of
    32768 and 65536 samples: the reference's sync_levels -> input ->
    runLevel -> output sequence (src/partconvMulti.cpp:849-909), strict and
    relaxed, against the oracle's PartConvFilter and an FP64 convolution."""
    from partconv_gb300 import partconv

    rng = np.random.default_rng(L)
    h = wl.decaying_ir(rng, L, 1.0)
    f = partconv.PartConvFilter()
    assert f.setup(len(N), N, P, h) == 0, f.last_error
    o = oracle.OracleFilter(N, P, h)
    assert list(f.num_parts) == list(o.num_parts)
    N0 = N[0]
    x = np.zeros(N0 * (L // N0 + 2 * N[-1] // N0 + 4), np.float32)
    x[:L // 2] = (0.1 * rng.standard_normal(L // 2)).astype(np.float32)
    for relaxed in (0, 1):
        f.reset()
        o.reset()
        ys, rs = [], []
        for b in range(len(x) // N0):
            blk = x[b * N0:(b + 1) * N0]
            if relaxed:
                f.sync_levels_relaxed()
                o.sync_levels_relaxed()
                ys.append(f.output_relaxed())
                rs.append(o.output_relaxed())
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
        err = wl.rel_l2(y, r)
        print(f"{N} relaxed={relaxed}: rel L2 vs oracle {err:.2e}")
        assert err <= TOL
        if not relaxed:
            assert wl.rel_l2(y, wl.conv_fp64(x, h, len(x))) <= TOL
    assert f.cleanup() == 0


def test_filter_bench_large_level(gpu):
    """tune.py's bench() on a layout whose top level is 65536 samples."""
    from partconv_gb300 import partconv

    f = partconv.PartConvFilter()
    N, P = partconv.intArray(3), partconv.intArray(3)
    for i, (n, p) in enumerate([(4096, 6), (16384, 6), (65536, 2)]):
        N[i], P[i] = n, p
    assert f.setup(3, N, P, None, 2, "wisdom.wis") == 0
    for lv in range(3):
        t = f.bench(lv, 20, 3, 0.1)
        assert 0 < t < 0.1
    assert f.cleanup() == 0


@pytest.mark.parametrize("streams", [1, 3, 9])
def test_in_step_large_levels_on_clusters_or_ctas(gpu, streams):
    """Minimum-slack layouts whose 8192- and 16384-sample levels fire within
    their step: with at most eight such fires per handle they run on 8-CTA
    clusters, with more on one CTA each.  Both match the oracle; pc_run
    block by block and pc_process give the same bits."""
    rng = np.random.default_rng(40 + streams)
    N0 = 256
    layouts = [([256, 2048, 16384], [8, 7, 1]), ([256, 1024, 8192], [4, 7, 1])]
    pcs = []
    for i in range(streams):
        N, P = layouts[i % 2]
        L = sum(n * p for n, p in zip(N[:-1], P[:-1])) + int(rng.integers(N[-1], 3 * N[-1]))
        pcs.append(dict(ir=wl.decaying_ir(rng, L, 0.5), N=N, P=P, in_ch=i, out_ch=i))
    L = max(len(p["ir"]) for p in pcs)
    frames = -(-(L + 8 * N0) // N0) * N0
    x = np.zeros((frames, streams), np.float32)
    x[:16 * N0] = (0.1 * rng.standard_normal((16 * N0, streams))).astype(np.float32)
    m = PartConvMulti()
    m.setup_layout(48000, N0, streams, streams, pcs)
    pcs = [p | dict(P=list(m.layout(i)[1])) for i, p in enumerate(pcs)]
    y = m.process(x)
    ref = oracle.OracleMulti(N0, streams, streams, pcs).run(x)
    for o in range(streams):
        err = _rel(y[:, o], ref[:, o])
        print(f"{streams} streams, output {o}: rel L2 vs oracle {err:.2e}")
        assert err <= TOL
    m.reset()
    yb = np.zeros_like(y)
    out = np.zeros(N0 * streams, np.float32)
    for b in range(frames // N0):
        m.run(out, np.ascontiguousarray(x[b * N0:(b + 1) * N0]), N0)
        yb[b * N0:(b + 1) * N0] = out.reshape(N0, streams)
    assert np.array_equal(yb, y)
