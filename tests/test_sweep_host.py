"""Host-side logic of the parameter sweeps and the surrogate, without a GPU:
the seeded replica table, the mapping of physical points to the reference's
unit box, the initial states, the phase-diagram grid and the network's
feature and target extraction."""
import numpy as np

from spsslangevinintegration_gb300 import _native as N
from spsslangevinintegration_gb300 import surrogate as S
from spsslangevinintegration_gb300 import sweep


def test_replica_table_is_seeded_and_in_range():
    a = sweep.replica_table(512, seed=3)
    b = sweep.replica_table(512, seed=3)
    assert a == b and a != sweep.replica_table(512, seed=4)
    n = np.array([p["n"] for p in a])
    assert n.min() >= 1024 and n.max() <= 65536
    # log-uniform: the median is near the geometric mean of the range
    assert 5000 < np.median(n) < 13000
    assert all(0.0 <= p["sigma"] <= 3.0 and 0.01 <= p["D"] <= 1.0 and p["m"] in (0.1, 1.0, 10.0) for p in a)
    assert {p["m"] for p in a} == {0.1, 1.0, 10.0}


def test_unit_box_mapping_of_a_point():
    point = dict(n=4096, sigma=1.5, D=0.2, m=10.0, density=2.0, R=1.0, v0=0.5)
    kw = sweep.system_params(point, seed=7, replica=3, skin=0.3, D_r=0.01)
    L = np.sqrt(4096 / 2.0)
    assert kw["model"] == 2 and kw["n"] == 4096 and kw["precision"] == N.PRECISION_F32
    assert np.isclose(kw["rho"], 1.0 / L) and np.isclose(kw["v0"], 0.5 / L)
    assert np.isclose(kw["xi_r"], 0.1) and np.isclose(kw["xi_phi"], 0.1)
    assert np.isclose(kw["sigma"], 0.15) and np.isclose(kw["D_phi"], 0.2 / 100.0)
    assert np.isclose(kw["D_r"], 0.01 / (100.0 * L * L))
    assert np.isclose(kw["r_max"], 1.3 / L) and kw["nc_verlet"] == int(L / 1.3)
    assert kw["seed"] == 7 and kw["replica"] == 3
    assert "r_max" not in sweep.system_params(point)


def test_initial_state_follows_the_reference_initialisation():
    n, L = 5000, 50.0
    x = sweep.initial_state(n, L, 11).reshape(n, 6)
    assert np.all((x[:, :2] >= 0.0) & (x[:, :2] < 1.0))
    assert np.all((x[:, 4] >= -np.pi) & (x[:, 4] < np.pi))
    np.testing.assert_allclose(np.hypot(x[:, 2], x[:, 3]), 1.0 / L, rtol=1e-12)
    np.testing.assert_allclose(np.arctan2(x[:, 3], x[:, 2]), x[:, 4], atol=1e-12)
    assert np.all(x[:, 5] == 0.0)
    np.testing.assert_array_equal(x.reshape(-1), sweep.initial_state(n, L, 11))


def test_phase_diagram_grid_and_training_points():
    g = S.grid_points(nsigma=8, nd=5)
    assert len(g) == 40
    sig = np.array([p["sigma"] for p in g]).reshape(5, 8)
    d = np.array([p["D"] for p in g]).reshape(5, 8)
    np.testing.assert_allclose(sig[0], np.linspace(0.0, 3.0, 8))
    assert np.all(d == d[:, :1])  # D constant along a row, sigma varies fastest
    np.testing.assert_allclose(d[:, 0], np.geomspace(0.01, 1.0, 5), rtol=1e-12)
    t = S.training_points(1000, seed=2)
    assert t == S.training_points(1000, seed=2)
    assert all(p["n"] == 1024 and 0.0 <= p["sigma"] <= 3.0 and 0.01 <= p["D"] <= 1.0 for p in t)


def test_features_and_run_values():
    pts = [dict(n=1024, sigma=0.5, D=0.1, m=1.0, density=2.0, R=1.0, v0=0.5),
           dict(n=1024, sigma=2.0, D=0.01, m=10.0, density=2.0, R=1.0, v0=0.5)]
    f = S.point_features(pts)
    np.testing.assert_allclose(f, [[0.5, -1.0, 2.0, 0.0, 0.5], [2.0, -2.0, 2.0, 1.0, 0.5]])
    stats = np.array([[0.7, 0.01, 0.4, 0.02, 200.0], [0.1, 0.03, 0.9, 0.001, 200.0]])
    np.testing.assert_array_equal(S.run_values(stats), [[0.7, 0.4], [0.1, 0.9]])
