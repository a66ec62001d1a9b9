"""Test helpers: write WAV files in several encodings and pc.config files."""
import struct

import numpy as np


def write_wav(path, data, fs=48000, fmt="pcm16"):
    """data: [frames] or [frames, channels] float in [-1, 1).  Returns the
    float32 samples a reader must recover for channel 0."""
    d = np.asarray(data, np.float64)
    if d.ndim == 1:
        d = d[:, None]
    frames, ch = d.shape
    if fmt == "pcm16":
        q = np.clip(np.round(d * 32768.0), -32768, 32767).astype("<i2")
        payload, code, bits = q.tobytes(), 1, 16
        back = q[:, 0].astype(np.float32) / np.float32(32768.0)
    elif fmt == "pcm24":
        q = np.clip(np.round(d * 8388608.0), -8388608, 8388607).astype(np.int32)
        b = q.astype("<i4").view(np.uint8).reshape(frames, ch, 4)[:, :, :3]
        payload, code, bits = b.tobytes(), 1, 24
        back = (q[:, 0].astype(np.float32) / np.float32(8388608.0)).astype(np.float32)
    elif fmt == "float32":
        q = d.astype("<f4")
        payload, code, bits = q.tobytes(), 3, 32
        back = q[:, 0].astype(np.float32)
    else:
        raise ValueError(fmt)
    block = ch * bits // 8
    fmt_chunk = struct.pack("<HHIIHH", code, ch, fs, fs * block, block, bits)
    riff = b"WAVE" + b"fmt " + struct.pack("<I", len(fmt_chunk)) + fmt_chunk
    riff += b"LIST" + struct.pack("<I", 4) + b"INFO"          # an extra chunk readers must skip
    riff += b"data" + struct.pack("<I", len(payload)) + payload
    with open(path, "wb") as f:
        f.write(b"RIFF" + struct.pack("<I", len(riff)) + riff)
    return back


def write_config(path, fs, buffer_size, n_in, n_out, pcs, repeats=1, drop_last_parts=False):
    """pcs: dicts file, mute, in_ch, out_ch, scale, N, P (format of
    src/pc.config:43-44)."""
    lines = [f"{fs} {buffer_size} {n_in} {n_out} {len(pcs)} {repeats}"]
    for p in pcs:
        lv = []
        for i, (n, q) in enumerate(zip(p["N"], p["P"])):
            last = i == len(p["N"]) - 1
            lv.append(f"{n}" if (last and drop_last_parts) else f"{n} {q}")
        lines.append(f"{p['file']} {p.get('mute', 0)} {p['in_ch']} {p['out_ch']} {p.get('scale', 1.0)} "
                     f"{len(p['N'])} " + " ".join(lv))
    lines.append("")
    lines.append("# trailing notes are ignored")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
