"""Trajectory files in the reference's .bin format, without a GPU: reading
all frames and the restart frame (SimulationEngineFirstOrder.cpp:69-93) of a
file written here frame by frame as the reference's observers write them."""
import os
import tempfile

import numpy as np
import pytest

from spsslangevinintegration_gb300.observers import read_frames, read_last_frame


def write_reference_file(path, times, states):
    with open(path, "wb") as f:
        for t, x in zip(times, states):
            np.array([t], dtype=np.float32).tofile(f)
            np.asarray(x, dtype=np.float32).tofile(f)


def test_read_frames_and_last_frame():
    rng = np.random.default_rng(0)
    n, s = 37, 6
    times = [0.1, 0.2, 0.3]
    states = [rng.random(n * s) for _ in times]
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "traj.bin")
        write_reference_file(path, times, states)
        t, frames = read_frames(path, n, s)
        np.testing.assert_array_equal(t, np.array(times, dtype=np.float32))
        for got, x in zip(frames, states):
            np.testing.assert_array_equal(got, x.astype(np.float32))
        t_last, x_last = read_last_frame(path, n, s)
        assert t_last == np.float32(0.3)
        np.testing.assert_array_equal(x_last, states[-1].astype(np.float32).astype(np.float64))


def test_truncated_file_is_rejected():
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "bad.bin")
        np.zeros(10, dtype=np.float32).tofile(path)
        with pytest.raises(ValueError):
            read_frames(path, 3, 4)
        with pytest.raises(ValueError):
            read_last_frame(path, 3, 4)
