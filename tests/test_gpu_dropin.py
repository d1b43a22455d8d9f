"""The C++ drop-in classes (include/spss/spss.hpp) compiled into a program that
drives them like the reference's engines; results checked against the oracle
(tolerance 1e-11 relative: FP64 path)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from helpers import per_component_close

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_example(out):
    from spsslangevinintegration_gb300 import build

    lib = build.build_library()
    exe = os.path.join(out, "dropin_example")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "dropin_example.cpp"), "-o", exe,
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

    sysm = ob.System(1, 400, 0.1, v0=0.3, xi=0.1, sigma=1.0, alpha=0.2, D_phi=0.1, flavor=0)
    x, t = fo.copy(), 0.0
    for _ in range(10):
        t += 0.01
        sysm.step(ob.RK4, 0, x, t, 0.01)
    per_component_close(fo_gpu, x, 4, 1e-11, "first-order RK4 drop-in")

    sysm = ob.System(2, 500, 0.07, v0=0.5, xi_r=1.0, D_r=0.02, xi_phi=1.0, D_phi=0.1, sigma=1.0, flavor=0)
    x, t = so.copy(), 0.0
    for k in range(5):
        t += 0.005
        sysm.step(ob.SE, 0, x, t, 0.005, noise[k * 1500:(k + 1) * 1500])
        ob.apply_pbc(2, x)
    per_component_close(so_gpu, x, 6, 1e-11, "second-order SE drop-in")
