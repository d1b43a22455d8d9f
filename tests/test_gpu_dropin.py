"""The C++ drop-in classes (include/spss/spss.hpp) compiled into a program that
drives them like the reference's engines; results checked against the oracle
(tolerance 1e-11 relative: FP64 path)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from helpers import per_component_close, reference_frame
from spsslangevinintegration_gb300.observers import read_frames

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_example(out):
    from spsslangevinintegration_gb300 import build

    lib = build.build_library()
    exe = os.path.join(out, "dropin_example")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "dropin_example.cpp"), "-o", exe, "-pthread",
                    "-L" + os.path.dirname(lib), "-lspss_gpu", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def test_dropin_classes_match_oracle():
    from golden.make_golden import initial_state
    from oracle import binding as ob

    with tempfile.TemporaryDirectory() as d:
        exe = build_example(d)
        fo = initial_state(1, 400, seed=71)
        so = initial_state(2, 500, seed=72, v0=0.01)
        fo.tofile(os.path.join(d, "fo_init.bin"))
        so.tofile(os.path.join(d, "so_init.bin"))
        r = subprocess.run([exe, d], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        fo_gpu = np.fromfile(os.path.join(d, "fo_final.bin"))
        so_gpu = np.fromfile(os.path.join(d, "so_final.bin"))
        noise = np.fromfile(os.path.join(d, "so_noise.bin"))
        times, frames = read_frames(os.path.join(d, "fo_traj.bin"), 400, 4)
        summary = np.loadtxt(os.path.join(d, "fo_summary.txt"))
        restart = np.fromfile(os.path.join(d, "fo_restart.bin"))
        residency = np.fromfile(os.path.join(d, "so_residency.bin"))
        addnoise = {m: (np.fromfile(os.path.join(d, m + "_addnoise.bin")),
                        np.fromfile(os.path.join(d, m + "_addnoise_z.bin"))) for m in ("fo", "so")}

    sysm = ob.System(1, 400, 0.1, v0=0.3, xi=0.1, sigma=1.0, alpha=0.2, D_phi=0.1, flavor=0)
    x, t = fo.copy(), 0.0
    expected = []
    for k in range(10):
        t += 0.01
        sysm.step(ob.RK4, 0, x, t, 0.01)
        if k % 2 == 0:
            expected.append((t, reference_frame(x, 4, wrapped=True)))
    per_component_close(fo_gpu, x, 4, 1e-11, "first-order RK4 drop-in")
    # the trajectory file: 5 frames in the reference's format, each the
    # float frame of the state (1 float ulp: the states agree to 1e-11)
    assert len(times) == 5
    np.testing.assert_array_equal(times, np.array([e[0] for e in expected], dtype=np.float32))
    for got, (_, ref) in zip(frames, expected):
        np.testing.assert_allclose(got, ref, rtol=2.5e-7, atol=1e-7)
    assert summary.shape == (5, 3)
    # restart reads the last frame back
    np.testing.assert_array_equal(restart[:-1], frames[-1].astype(np.float64))
    assert restart[-1] == np.float64(times[-1])

    sysm = ob.System(2, 500, 0.07, v0=0.5, xi_r=1.0, D_r=0.02, xi_phi=1.0, D_phi=0.1, sigma=1.0, flavor=0)
    x, t = so.copy(), 0.0
    for k in range(5):
        t += 0.005
        sysm.step(ob.SE, 0, x, t, 0.005, noise[k * 1500:(k + 1) * 1500])
        ob.apply_pbc(2, x)
    per_component_close(so_gpu, x, 6, 1e-11, "second-order SE drop-in")

    # AddNoise writes sqrt(2 D) times the step's normals into the noise
    # components and leaves the others as they were
    # (ParticleSystemFirstOrder.cpp:698-708, ParticleSystemSecondOrder.cpp:439-451)
    d, z = addnoise["fo"]
    d = d.reshape(300, 4)
    np.testing.assert_array_equal(d[:, :3], 7.0)
    np.testing.assert_allclose(d[:, 3], np.sqrt(2.0 * 0.25) * z, rtol=1e-15)
    assert abs(z.mean()) < 0.2 and 0.8 < z.std() < 1.2
    d, z = addnoise["so"]
    d, z = d.reshape(500, 6), z.reshape(500, 3)
    np.testing.assert_array_equal(d[:, [0, 1, 4]], 7.0)
    np.testing.assert_allclose(d[:, 2], np.sqrt(2.0 * 0.02) * z[:, 0], rtol=1e-15)
    np.testing.assert_allclose(d[:, 3], np.sqrt(2.0 * 0.02) * z[:, 1], rtol=1e-15)
    np.testing.assert_allclose(d[:, 5], np.sqrt(2.0 * 0.1) * z[:, 2], rtol=1e-15)

    # observers read the GPU copy of a stepped array (the same state as the
    # host array) until spss::HostStateChanged, then the host array
    r_gpu = ob.order_parameters(2, x)
    assert abs(residency[0] - r_gpu[0]) <= 1e-12 and abs(residency[2] - r_gpu[0]) <= 1e-12
    assert residency[4] == 1.0 and residency[5] == 0.0
