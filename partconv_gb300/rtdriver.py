"""Headless real-time driver for PartConvMulti.

The reference runs PartConvMulti from an audio device's callback
(src/pcRTMulti.cpp:138-185 with PortAudio, :303-506 with ALSA) and reports
output underflows.  Without an audio device, ``RealtimeDriver`` feeds a
signal block by block at the device's pace through the C ABI's
``pc_rt_drive`` (a native loop on a monotonic clock), collects the output,
and reports deadline misses and release-to-return latency per callback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat
from .multi import PartConvMulti


class RealtimeDriver:
    """Drive ``pc`` (a set-up PartConvMulti or PartConvMultiRelaxed)."""

    def __init__(self, pc: PartConvMulti):
        self.pc = pc

    def run(self, x: np.ndarray, realtime: bool = True, period_s: float = 0.0):
        """x: interleaved [frames, numInputChannels] float32, frames a multiple
        of buffer_size.  Returns (y [frames, numOutputChannels], stats dict).
        period_s = 0 uses buffer_size / FS."""
        pc = self.pc
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, pc.numInputChannels)
        frames = x.shape[0]
        if frames % pc.buffer_size:
            raise nat.PartConvError(nat.PC_ERR_ARG, "frames must be a multiple of buffer_size")
        y = np.zeros((frames, pc.numOutputChannels), np.float32)
        st = nat.PCRtStats()
        nat.check(pc._h, pc._lib.pc_rt_drive(pc._h, x.ctypes.data_as(nat._f32p), y.ctypes.data_as(nat._f32p),
                                             int(frames), float(period_s), int(bool(realtime)), C.byref(st)))
        blocks = frames // pc.buffer_size
        pc._frame_num += blocks
        if pc.doneWaiter is not None and pc.lastFrame and pc._frame_num >= pc.lastFrame:
            pc.doneWaiter.changeAndSignal(1)
        stats = {f: getattr(st, f) for f, _ in nat.PCRtStats._fields_}
        stats["miss_rate"] = st.misses / max(st.callbacks, 1)
        return y, stats
