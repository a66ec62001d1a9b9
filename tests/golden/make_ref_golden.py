"""Regenerate tests/golden/ref_golden.npz: seeded inputs, IRs and layouts with
the outputs of the reference's OWN code -- PartConvFilter compiled from the
reference's src/partconv.cpp and src/buffers.cpp into oracle/_ref/ (see
oracle/Makefile.ref; FFTW is stood in for by the oracle's transform) and
driven through PartConvMulti::run's callback sequence (strict) and
PartConvMultiRelaxed::run's (one block later).

Only layouts the reference's setup accepts (its strict slack check) appear.
The Relaxed outputs are not stored: the reference's own Relaxed run equals
its strict output one base block later, bit for bit (a CPU test checks this
where the reference builds), so ``load`` derives them by that shift.
The fixtures pin the GPU path to the reference on hosts where the reference
cannot be built (the aarch64 GPU host: its MAC is SSE3).

Run from the repository root, on an x86_64 host with the reference checkout:
    python tests/golden/make_ref_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_golden.npz")

# name -> (buffer_size, n_in, n_out, [pc specs], input samples); every layout
# passes the reference's check 2 N0 + s_L >= 2 N_L (src/partconv.cpp:148-166)
CASES = {
    # three levels, N_L = 4 N_{L-1}, minimum strict slack
    "ref_strict3": (64, 1, 1, [dict(N=[64, 256, 1024], P=[6, 6, 0], L=9000, in_ch=0, out_ch=0)], 4096),
    # the shape the autotuner picks for the batched 32-stream workload
    "ref_chain_256_2048_16384": (256, 1, 1, [dict(N=[256, 2048, 16384], P=[14, 14, 0], L=48000, in_ch=0,
                                                  out_ch=0)], 4096),
    # five levels from a 32-sample base block (the reference's pc.config "32's" style)
    "ref_deep5": (32, 1, 1, [dict(N=[32, 128, 512, 2048, 8192], P=[6, 6, 6, 6, 0], L=40000, in_ch=0,
                                  out_ch=0)], 2048),
    # one level
    "ref_single": (256, 1, 1, [dict(N=[256], P=[0], L=3000, in_ch=0, out_ch=0)], 4096),
    # mixing: two inputs, two outputs, scale and mute, output sums in PC order
    "ref_mix": (128, 2, 2, [dict(N=[128, 1024], P=[14, 0], L=5000, in_ch=0, out_ch=0),
                            dict(N=[128], P=[0], L=2500, in_ch=1, out_ch=0, scale=0.5),
                            dict(N=[128, 1024], P=[14, 0], L=3000, in_ch=0, out_ch=1, mute=1),
                            dict(N=[128, 512], P=[6, 0], L=1800, in_ch=1, out_ch=1, scale=-1.25)], 3072),
    # a 32768-sample top level (the fires of blocks above 16384 run on clusters
    # of CTAs on the GPU), as the reference's own pc.config layouts use
    "ref_large_32768": (256, 1, 1, [dict(N=[256, 2048, 32768], P=[14, 30, 0], L=110000, in_ch=0, out_ch=0)],
                        4096),
}


def decaying(rng, n, t60, fs=48000):
    h = rng.standard_normal(n) * np.exp(-6.91 * np.arange(n) / (t60 * fs))
    return (h / np.linalg.norm(h)).astype(np.float32)


def case_inputs(ci, bs, n_in, specs, n_x):
    """Seeded IRs, layouts (last part count from the reference's setup) and
    the flushed input of one case."""
    from oracle import ref

    rng = np.random.default_rng(np.random.PCG64(9000 + ci))
    pcs = []
    for s in specs:
        h = decaying(rng, s["L"], 0.25)
        st, P = ref.layout_check(s["N"], [max(p, 1) for p in s["P"]], s["L"])
        assert st == 0, s
        pcs.append(dict(ir=h, N=list(s["N"]), P=[int(p) for p in P], in_ch=s["in_ch"], out_ch=s["out_ch"],
                        scale=float(s.get("scale", 1.0)), mute=int(s.get("mute", 0))))
    L = max(len(p["ir"]) for p in pcs)
    frames = -(-(n_x + L) // bs) * bs
    x = np.zeros((frames, n_in), np.float32)
    x[:n_x] = (0.1 * rng.standard_normal((n_x, n_in))).astype(np.float32)
    return pcs, x, frames


def make():
    from oracle import ref

    out = {}
    for ci, (name, (bs, n_in, n_out, specs, n_x)) in enumerate(CASES.items()):
        pcs, x, frames = case_inputs(ci, bs, n_in, specs, n_x)
        y = ref.RefMulti(bs, n_in, n_out, pcs).run(x)
        out[f"{name}/meta"] = np.array([bs, n_in, n_out, len(pcs), frames], np.int64)
        out[f"{name}/x"] = x
        out[f"{name}/y"] = y
        for k, p in enumerate(pcs):
            out[f"{name}/pc{k}/ir"] = p["ir"]
            out[f"{name}/pc{k}/N"] = np.array(p["N"], np.int32)
            out[f"{name}/pc{k}/P"] = np.array(p["P"], np.int32)
            out[f"{name}/pc{k}/chan"] = np.array([p["in_ch"], p["out_ch"], p["mute"]], np.int32)
            out[f"{name}/pc{k}/scale"] = np.array([p["scale"]], np.float32)
    np.savez_compressed(PATH, **out)
    return PATH


def relaxed_from_strict(y, bs):
    """PartConvMultiRelaxed's output: the strict output one block later."""
    yr = np.zeros_like(y)
    yr[bs:] = y[:-bs]
    return yr


def load():
    """{case: dict(bs, n_in, n_out, frames, x, y, y_relaxed, pcs)}"""
    z = np.load(PATH)
    cases = {}
    for name in sorted({k.split("/")[0] for k in z.files}):
        bs, n_in, n_out, npc, frames = (int(v) for v in z[f"{name}/meta"])
        pcs = []
        for k in range(npc):
            ch = z[f"{name}/pc{k}/chan"]
            pcs.append(dict(ir=z[f"{name}/pc{k}/ir"], N=[int(v) for v in z[f"{name}/pc{k}/N"]],
                            P=[int(v) for v in z[f"{name}/pc{k}/P"]], in_ch=int(ch[0]), out_ch=int(ch[1]),
                            mute=int(ch[2]), scale=float(z[f"{name}/pc{k}/scale"][0])))
        y = z[f"{name}/y"]
        cases[name] = dict(bs=bs, n_in=n_in, n_out=n_out, frames=frames, x=z[f"{name}/x"], y=y,
                           y_relaxed=relaxed_from_strict(y, bs), pcs=pcs)
    return cases


if __name__ == "__main__":
    print(make())
