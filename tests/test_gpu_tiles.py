"""Kernel tile shapes (pc_set_tiles): bins and parts per spread task, the
shape the autotuner picks.  Every accepted shape must give the oracle's
result (relative L2 <= 1e-5 per output channel), pc_run block by block and
pc_process must agree bit for bit, and shapes outside the accepted set are
refused."""
import numpy as np
import pytest

import oracle
from partconv_gb300 import PartConvMulti, PartConvError
from partconv_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _case():
    rng = np.random.default_rng(21)
    # many parts on every level: level 0 and both larger levels have spread
    # tasks with several partial-sum rows; one strict (deferred) layout, one
    # minimum-slack layout
    pcs = [dict(ir=wl.decaying_ir(rng, 250000, 1.5), N=[256, 2048, 16384], P=[30, 14, 1], in_ch=0, out_ch=0),
           dict(ir=wl.decaying_ir(rng, 60000, 0.8), N=[256, 2048], P=[40, 1], in_ch=1, out_ch=1),
           dict(ir=wl.decaying_ir(rng, 40000, 0.8), N=[256, 1024], P=[4, 1], in_ch=0, out_ch=1)]
    L = max(len(p["ir"]) for p in pcs)
    frames = -(-(L + 4096) // 256) * 256
    x = np.zeros((frames, 2), np.float32)
    x[:4096] = (0.1 * rng.standard_normal((4096, 2))).astype(np.float32)
    return pcs, x, frames


CASE = _case()
REF = None


def _ref(pcs_fixed, x):
    global REF
    if REF is None:
        REF = oracle.OracleMulti(256, 2, 2, pcs_fixed).run(x)
    return REF


@pytest.mark.parametrize("bins", [64, 128, 256, 512])
@pytest.mark.parametrize("parts", [4, 16, 64])
def test_every_tile_shape_matches_oracle(gpu, bins, parts):
    pcs, x, frames = CASE
    m = PartConvMulti(tiles=(bins, parts))
    m.setup_layout(48000, 256, 2, 2, pcs)
    info = m.info()
    assert (info.spread_bins, info.spread_parts) == (bins, parts)
    y = m.process(x)
    ref = _ref([p | dict(P=list(m.layout(i)[1])) for i, p in enumerate(pcs)], x)
    for o in range(2):
        err = _rel(y[:, o], ref[:, o])
        assert err <= TOL, (bins, parts, o, err)
    if (bins, parts) in ((64, 4), (512, 64)):   # block by block: the same bits
        m.reset()
        yb = np.zeros_like(y)
        out = np.zeros(512, np.float32)
        for b in range(frames // 256):
            m.run(out, np.ascontiguousarray(x[b * 256:(b + 1) * 256]), 256)
            yb[b * 256:(b + 1) * 256] = out.reshape(256, 2)
        assert np.array_equal(yb, y)


def test_tile_shapes_outside_the_set_are_refused(gpu):
    for bins, parts in ((48, 16), (1024, 16), (32, 16), (128, 65), (128, -1)):
        with pytest.raises(PartConvError):
            PartConvMulti(tiles=(bins, parts))
