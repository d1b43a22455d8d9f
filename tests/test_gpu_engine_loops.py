"""The reference's engine loops compiled against the drop-in classes
(tests/cpp/engine_loops.cpp) and run on the GB300 path (FP32 pair and stage
arithmetic), checked against the FP64 oracle replaying the normals each step
drew:

  A  ParticleSystemSecondOrder + StochasticEulerStepper + PBC + BinaryObserverSecondOrder
     (SimulationEngineSecondOrder.cpp:118-143);
  B  ParticleSystemSecondOrderPtr on the Verlet list + StochasticRungeKuttaStepperPtr +
     BinaryObserverSecondOrderPtr (SimulationEngineSecondOrderPtr.cpp:83-99);
  C  ParticleSystemFirstOrderPtr + StochasticRungeKuttaStepperPtr + BinaryObserverFirstOrderPtr,
     then the averaging pass with AveragingObserverPtr (SimulationEngineFirstOrderPtr.cpp:122-161).

Tolerances: final states as the fast path's 50-step parity (99.9 % of
particles within 1e-3 relative, median within 1e-5); trajectory frames (float
state, first order wrapped) within 1e-4 of the oracle state's frame (positions
under the minimum image); summary lines |R| within 1e-5 and arg R within
1e-4 (the observers reduce in FP64 on the GPU); the averaged angular
velocities within 1e-4 relative of their scale.  File names follow the
reference observers' naming.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from helpers import reference_frame, state_err
from spsslangevinintegration_gb300.observers import read_frames

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N = 4096
DT = 0.005


def build(out):
    from spsslangevinintegration_gb300 import build as b

    lib = b.build_library()
    exe = os.path.join(out, "engine_loops")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "engine_loops.cpp"), "-o", exe, "-pthread",
                    "-L" + os.path.dirname(lib), "-lspss_gpu", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def initial(model, seed, v=0.01):
    rng = np.random.default_rng(seed)
    s = 4 if model == 1 else 6
    x = np.zeros((N, s))
    x[:, 0], x[:, 1] = rng.random(N), rng.random(N)
    phi = rng.uniform(-np.pi, np.pi, N)
    if model == 1:
        x[:, 2], x[:, 3] = phi, rng.uniform(-0.5, 0.5, N)
    else:
        x[:, 2], x[:, 3], x[:, 4], x[:, 5] = v * np.cos(phi), v * np.sin(phi), phi, rng.uniform(-0.5, 0.5, N)
    return x.reshape(-1)


def check_state(got, ref, s, what):
    err = state_err(got, ref, s).max(axis=1)
    assert np.quantile(err, 0.999) <= 1e-3, (what, float(np.quantile(err, 0.999)))
    assert np.median(err) <= 1e-5, (what, float(np.median(err)))


def check_frame(got, ref_state, s, wrapped, what):
    ref = reference_frame(ref_state, s, wrapped).reshape(-1, s).astype(np.float64)
    got = got.reshape(-1, s).astype(np.float64)
    d = got - ref
    d[:, :2] -= np.round(d[:, :2])
    if wrapped:
        d[:, 2] -= 2 * np.pi * np.round(d[:, 2] / (2 * np.pi))
    scale = np.abs(ref).max(axis=0)
    scale[:2] = 1.0
    err = (np.abs(d) / (np.abs(ref) + scale)).max(axis=1)
    assert np.quantile(err, 0.999) <= 1e-4, (what, float(np.quantile(err, 0.999)))


def check_summary(lines, states, times, model, what):
    from oracle import binding as ob

    assert lines.shape == (len(states), 3), (what, lines.shape)
    for row, x, t in zip(lines, states, times):
        r = ob.order_parameters(model, x)
        assert row[0] == pytest.approx(np.float32(t), rel=1e-6), what
        assert abs(row[1] - r[0]) <= 1e-5, (what, row[1], r[0])
        assert abs(np.angle(np.exp(1j * (row[2] - r[1])))) <= 1e-4 / max(r[0], 1e-3), (what, row[2], r[1])


def replay(system, stepper, variant, x, noise, per, t0, steps, wrap, after_step=None):
    from oracle import binding as ob

    t = t0
    for k in range(steps):
        t += DT
        system.step(stepper, variant, x, t, DT, noise[k * per * N:(k + 1) * per * N])
        if wrap:
            ob.apply_pbc(2, x)
        if after_step:
            after_step(k, t, x)
    return x


def test_engine_loops_on_the_fast_path_match_the_oracle():
    from oracle import binding as ob

    with tempfile.TemporaryDirectory() as d:
        exe = build(d)
        inits = {"a": initial(2, 1), "b": initial(2, 2), "c": initial(1, 3)}
        for k, v in inits.items():
            v.tofile(os.path.join(d, k + "_init.bin"))
        r = subprocess.run([exe, d], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        steps = [int(v) for v in open(os.path.join(d, "steps.txt")).read().split()]
        out = {k: np.fromfile(os.path.join(d, k + "_final.bin")) for k in ("a", "b", "c", "c_avg")}
        noise = {k: np.fromfile(os.path.join(d, k + "_noise.bin")) for k in ("a", "b", "c", "c_avg")}
        so_sim = "v0_0.01_xir_1_Dr_0.0001_xiphi_1_Dphi_0.1_sigma_1_rho_0.03_alpha_0.2_N_4096_0_%d"
        fa = read_frames(os.path.join(d, so_sim % 0 + ".bin"), N, 6)
        sa = np.loadtxt(os.path.join(d, "summary_statistics_" + so_sim % 0 + ".txt"))
        fb = read_frames(os.path.join(d, so_sim % 1 + ".bin"), N, 6)
        sb = np.loadtxt(os.path.join(d, "summary_statistics_" + so_sim % 1 + ".txt"))
        fo_sim = "v0_0.01_xi_0.1_sigma_1_rho_0.03_alpha_0.3_Dphi_0.01_N_4096_0_2"
        fc = read_frames(os.path.join(d, fo_sim + ".bin"), N, 4)
        sc = np.loadtxt(os.path.join(d, fo_sim + ".txt"))
        avg = np.fromfile(os.path.join(d, "averaged_angular_velocities_v0_0.01_xi_0.1_sigma_1_rho_0.03_alpha_0.3"
                                          "_Dphi_0.01_N_4096_2.bin"), dtype=np.float32)
    assert steps[0] == steps[1] and steps[2] > 100 and steps[3] > 10

    # A and B: the second-order loops (frames and summary lines every 10th call)
    for key, variant, stepper, per, frames, summary, kw in (
            ("a", 0, ob.SE, 3, fa, sa, {}),
            ("b", 4, ob.SRK, 6, fb, sb, dict(r_max=1.3 * 0.03, nc_verlet=int(1.0 / (1.3 * 0.03))))):
        sysm = ob.System(2, N, 0.03, v0=0.01, xi_r=1.0, D_r=1e-4, xi_phi=1.0, D_phi=0.1, sigma=1.0, alpha=0.2,
                         flavor=0 if key == "a" else 1, **kw)
        x = inits[key].copy()
        frame_states, summary_states, summary_times = [x.copy()], [], []

        def keep(k, t, xs):
            if (k + 1) % 10 == 0:
                frame_states.append(xs.copy())
            if k % 10 == 0:
                summary_states.append(xs.copy())
                summary_times.append(t)

        replay(sysm, stepper, variant, x, noise[key], per, 0.0, steps[0], True, keep)
        check_state(out[key], x, 6, key)
        times, fr = frames
        assert len(fr) == len(frame_states), (key, len(fr))
        for got, ref in zip(fr, frame_states):
            check_frame(got, ref, 6, False, key)
        check_summary(summary, summary_states, summary_times, 2, key)

    # C: the first-order loop (every 100th call), positions never wrapped
    sysm = ob.System(1, N, 0.03, v0=0.01, xi=0.1, sigma=1.0, alpha=0.3, D_phi=0.01, flavor=1)
    x = inits["c"].copy()
    frame_states, summary_states, summary_times = [x.copy()], [], []

    def keep_c(k, t, xs):
        if (k + 1) % 100 == 0:
            frame_states.append(xs.copy())
        if k % 100 == 0:
            summary_states.append(xs.copy())
            summary_times.append(t)

    replay(sysm, ob.SRK, 0, x, noise["c"], 2, 0.0, steps[2], False, keep_c)
    check_state(out["c"], x, 4, "c")
    times, fr = fc
    assert len(fr) == len(frame_states) == 2
    for got, ref in zip(fr, frame_states):
        check_frame(got, ref, 4, True, "c")
    check_summary(sc, summary_states, summary_times, 1, "c")

    # the averaging pass continues the same system on a copy of the state
    omega_sum = np.zeros(N)

    def acc(k, t, xs):
        omega_sum[:] += xs.reshape(N, 4)[:, 3]

    replay(sysm, ob.SRK, 0, x, noise["c_avg"], 2, 0.0, steps[3], False, acc)
    check_state(out["c_avg"], x, 4, "c_avg")
    ref_avg = omega_sum / steps[3]
    assert np.max(np.abs(avg - ref_avg)) <= 1e-4 * np.max(np.abs(ref_avg))
