"""Regenerate tests/golden/golden.npz: seeded inputs, IRs and layouts with
the oracle's float32 outputs (strict-latency PartConvMulti and the Relaxed
variant).  The fixtures let the GPU tests check the CUDA path without
running the oracle, and the CPU tests check that the oracle still produces
them and that they agree with an FP64 convolution.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402


def decaying(rng, n, t60, fs=48000):
    h = rng.standard_normal(n) * np.exp(-6.91 * np.arange(n) / (t60 * fs))
    return (h / np.linalg.norm(h)).astype(np.float32)


# name -> (buffer_size, n_in, n_out, [pc specs], input samples)
CASES = {
    # cfg1's three-level shape at a quarter of its block sizes (relaxed slack)
    "mono3": (64, 1, 1, [dict(N=[64, 512, 4096], P=[8, 7, 0], L=10000, in_ch=0, out_ch=0)], 6144),
    # a layout that passes the reference's strict slack check
    "strict": (64, 1, 1, [dict(N=[64, 256, 1024], P=[6, 6, 0], L=3000, in_ch=0, out_ch=0)], 2048),
    # mixing: two inputs, two outputs, scale and mute, output sums in PC order
    "mix": (128, 2, 2, [dict(N=[128, 1024], P=[8, 0], L=5000, in_ch=0, out_ch=0),
                        dict(N=[128], P=[0], L=2500, in_ch=1, out_ch=0, scale=0.5),
                        dict(N=[128, 1024], P=[8, 0], L=3000, in_ch=0, out_ch=1, mute=1),
                        dict(N=[128, 512], P=[4, 0], L=1800, in_ch=1, out_ch=1, scale=-1.25)], 3072),
}


def make():
    out = {}
    for ci, (name, (bs, n_in, n_out, specs, n_x)) in enumerate(CASES.items()):
        rng = np.random.default_rng(np.random.PCG64(7000 + ci))
        pcs = []
        for k, s in enumerate(specs):
            h = decaying(rng, s["L"], 0.2)
            st, P, _, msg = oracle.layout_check(s["N"], [max(p, 1) for p in s["P"]], s["L"], relaxed=True)
            assert st == 0, (name, msg)
            pcs.append(dict(ir=h, N=list(s["N"]), P=[int(p) for p in P], in_ch=s["in_ch"], out_ch=s["out_ch"],
                            scale=float(s.get("scale", 1.0)), mute=int(s.get("mute", 0))))
        L = max(len(p["ir"]) for p in pcs)
        frames = -(-(n_x + L) // bs) * bs
        x = np.zeros((frames, n_in), np.float32)
        x[:n_x] = (0.1 * rng.standard_normal((n_x, n_in))).astype(np.float32)
        y = oracle.OracleMulti(bs, n_in, n_out, pcs).run(x)
        yr = oracle.OracleMulti(bs, n_in, n_out, pcs, relaxed=True).run(x)
        out[f"{name}/meta"] = np.array([bs, n_in, n_out, len(pcs), frames], np.int64)
        out[f"{name}/x"] = x
        out[f"{name}/y"] = y
        out[f"{name}/y_relaxed"] = yr
        for k, p in enumerate(pcs):
            out[f"{name}/pc{k}/ir"] = p["ir"]
            out[f"{name}/pc{k}/N"] = np.array(p["N"], np.int32)
            out[f"{name}/pc{k}/P"] = np.array(p["P"], np.int32)
            out[f"{name}/pc{k}/chan"] = np.array([p["in_ch"], p["out_ch"], p["mute"]], np.int32)
            out[f"{name}/pc{k}/scale"] = np.array([p["scale"]], np.float32)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")
    np.savez_compressed(path, **out)
    return path


def load(path=None):
    """{case: dict(bs, n_in, n_out, frames, x, y, y_relaxed, pcs)}"""
    path = path or os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")
    z = np.load(path)
    cases = {}
    for name in CASES:
        bs, n_in, n_out, npc, frames = (int(v) for v in z[f"{name}/meta"])
        pcs = []
        for k in range(npc):
            ch = z[f"{name}/pc{k}/chan"]
            pcs.append(dict(ir=z[f"{name}/pc{k}/ir"], N=[int(v) for v in z[f"{name}/pc{k}/N"]],
                            P=[int(v) for v in z[f"{name}/pc{k}/P"]], in_ch=int(ch[0]), out_ch=int(ch[1]),
                            mute=int(ch[2]), scale=float(z[f"{name}/pc{k}/scale"][0])))
        cases[name] = dict(bs=bs, n_in=n_in, n_out=n_out, frames=frames, x=z[f"{name}/x"], y=z[f"{name}/y"],
                           y_relaxed=z[f"{name}/y_relaxed"], pcs=pcs)
    return cases


if __name__ == "__main__":
    print(make())
