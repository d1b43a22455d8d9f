"""Observer output written from the GPU in the reference's file formats.

* Trajectory ``.bin``: frames of ``[float t][float s*n]``
  (BinaryObserverFirstOrder::SaveSystemState, BinaryObserverFirstOrder.cpp:101-123,
  which wraps positions into the unit box and phases into [0, 2 pi);
  BinaryObserverSecondOrder::SaveSystemState, BinaryObserverSecondOrder.cpp:101-116,
  which writes the state as it is).  Frames are computed on the GPU
  (``spss_frame_async``) into page-locked buffers; a background thread writes
  them, so the file I/O overlaps the steps that follow.
* Summary ``.txt``: ``t  |R|  arg R`` per line, R the phase order parameter
  (SaveSummaryStatistics; accumulated in FP64 here, in complex<float> there).
* Restart: the last frame of a ``.bin`` file as the initial state
  (SimulationEngineFirstOrder::InitializeSystemStateFromPreviousSolution,
  SimulationEngineFirstOrder.cpp:69-93).
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import _native as N
from .context import PinnedArray


def frame(ctx, wrapped=True):
    """One frame of `ctx` (s*n float32), synchronously."""
    out = np.empty(ctx.length, dtype=np.float32)
    mode = N.FRAME_WRAPPED if wrapped else N.FRAME_RAW
    N.check(ctx.L.spss_frame_async(ctx.h, mode, N.fptr(out), out.size), "spss_frame_async")
    ctx.synchronize()
    return out


class TrajectoryWriter:
    """The reference's binary observer on a GPU context: call it once per step
    with the time; every `every`-th call saves a frame (and a summary line).
    `wrapped` defaults to the reference's choice for the model (first order
    wrapped, second order raw); the reference saves every 100 steps (first
    order) or 10 (second order)."""

    def __init__(self, ctx, trajectory_path, summary_path=None, every=None, wrapped=None):
        self.ctx = ctx
        self.every = every if every is not None else (100 if ctx.model == 1 else 10)
        self.mode = N.FRAME_WRAPPED if (wrapped if wrapped is not None else ctx.model == 1) else N.FRAME_RAW
        self.traj = open(trajectory_path, "wb")
        self.summ = open(summary_path, "w") if summary_path else None
        self.bufs = [PinnedArray(ctx.length, np.float32), PinnedArray(ctx.length, np.float32)]
        self.pending = [None, None]
        self.pool = ThreadPoolExecutor(max_workers=1)
        self.counter = 0
        self.next = 0

    def _write(self, t, buf):
        np.array([t], dtype=np.float32).tofile(self.traj)
        buf.array.tofile(self.traj)

    def __call__(self, t):
        if self.counter % self.every == 0:
            b = self.next
            if self.pending[b] is not None:
                self.pending[b].result()  # the buffer's previous frame is on disk
            N.check(self.ctx.L.spss_frame_async(self.ctx.h, self.mode, N.fptr(self.bufs[b].array), self.ctx.length),
                    "spss_frame_async")
            if self.summ is not None:
                r = self.ctx.order_parameters()  # synchronises the stream, so the frame has landed too
                self.summ.write("%g\t%g\t%g\n" % (np.float32(t), np.float32(r[0]), np.float32(r[1])))
            else:
                self.ctx.synchronize()
            self.pending[b] = self.pool.submit(self._write, float(t), self.bufs[b])
            self.next = 1 - b
        self.counter += 1

    def close(self):
        for f in self.pending:
            if f is not None:
                f.result()
        self.pool.shutdown(wait=True)
        self.traj.close()
        if self.summ is not None:
            self.summ.close()
        for b in self.bufs:
            b.free()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def read_frames(path, n, s):
    """All frames of a .bin file: (times [k], states [k][s*n]) as float32."""
    raw = np.fromfile(path, dtype=np.float32)
    per = 1 + s * n
    if raw.size % per:
        raise ValueError("%s: size is not a whole number of frames of %d floats" % (path, per))
    raw = raw.reshape(-1, per)
    return raw[:, 0].copy(), raw[:, 1:].copy()


def read_last_frame(path, n, s):
    """The restart state: (t, state as float64 s*n) from the last frame of a
    .bin file, as InitializeSystemStateFromPreviousSolution reads it."""
    per = 4 * (1 + s * n)
    size = os.path.getsize(path)
    if size < per or size % per:
        raise ValueError("%s holds no whole frame of %d particles x %d values" % (path, n, s))
    with open(path, "rb") as f:
        f.seek(size - per)
        raw = np.frombuffer(f.read(per), dtype=np.float32)
    return float(raw[0]), raw[1:].astype(np.float64)
