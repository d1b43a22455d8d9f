"""The odeint path's Dormand-Prince 5(4) method checked against mathematics,
not against another transcription of it.

Boost.Odeint (the reference's integrator, SimulationEngineFirstOrder.cpp:158-165)
is not in the reference tree and its version is not pinned, so Boost's own
step sequence cannot be reproduced here.  What is pinned instead:

  * the tableau in csrc/dopri5.cu (read from the source, exact rational
    arithmetic): row sums equal the nodes, the propagated (fifth-order)
    weights satisfy all 17 order conditions up to order 5, the embedded
    weights all 8 up to order 4 and not all of order 5 (Butcher's rooted-tree
    conditions, Hairer, Norsett & Wanner, Solving ODE I, sec. II.2);
  * the continuous extension (the dense-output coefficients in the same
    file, in the form the integrator evaluates): for every theta its weights
    satisfy the order-4 conditions with theta^q / q! right-hand sides and
    reproduce the step's end point at theta = 1 (sec. II.6);
  * the integrator (CPU restatement oracle/dopri5_oracle.py, the same method
    as the GPU's, tests/test_gpu_dopri5.py) on a problem with a closed-form
    solution: uncoupled first-order particles without friction,
    phi = phi0 + omega0 t, x = x0 + v0 (sin phi - sin phi0) / omega0,
    y = y0 - v0 (cos phi - cos phi0) / omega0: the error at every observer
    time stays within 10 x the requested tolerance, and the number of
    accepted steps grows like tol^(-1/5) (ratio within [4, 10] for a 10^4
    tighter tolerance, 10^(4/5) = 6.3 for a fifth-order method).
"""
import os
import re
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "spsslangevinintegration_gb300", "csrc", "dopri5.cu")


def _number(term):
    """An exact rational from a source literal such as "19372.0 / 6561.0" or "0"."""
    parts = [Fraction(int(float(x))) for x in term.split("/")]
    assert all(float(x) == int(float(x)) for x in term.split("/")), term
    return parts[0] / parts[1] if len(parts) == 2 else parts[0]


def _array(name):
    text = open(SRC).read()
    m = re.search(r"constexpr double %s\[[^\]]*\](?:\[[^\]]*\])?\s*=\s*\{(.*?)\};" % name, text, re.S)
    assert m, name
    body = m.group(1)
    rows = re.findall(r"\{([^{}]*)\}", body)
    if not rows:
        return [_number(t) for t in body.split(",") if t.strip()]
    return [[_number(t) for t in row.split(",") if t.strip()] for row in rows]


def _tableau():
    c = _array("kC")
    A = _array("kA")
    e = _array("kE")
    d = _array("kD")
    A = [row + [Fraction(0)] * (7 - len(row)) for row in A]
    return c, A, e, d


def _conditions(b, c, A, order):
    """Residuals of Butcher's order conditions up to `order` for weights b."""
    s = len(b)
    Ac = [sum(A[i][j] * c[j] for j in range(s)) for i in range(s)]
    Ac2 = [sum(A[i][j] * c[j] ** 2 for j in range(s)) for i in range(s)]
    Ac3 = [sum(A[i][j] * c[j] ** 3 for j in range(s)) for i in range(s)]
    AAc = [sum(A[i][j] * Ac[j] for j in range(s)) for i in range(s)]
    AcAc = [sum(A[i][j] * c[j] * Ac[j] for j in range(s)) for i in range(s)]
    AAc2 = [sum(A[i][j] * Ac2[j] for j in range(s)) for i in range(s)]
    AAAc = [sum(A[i][j] * AAc[j] for j in range(s)) for i in range(s)]

    def dot(v):
        return sum(b[i] * v[i] for i in range(s))

    F = Fraction
    conds = [(dot([1] * s), F(1))]
    if order >= 2:
        conds += [(dot(c), F(1, 2))]
    if order >= 3:
        conds += [(dot([x ** 2 for x in c]), F(1, 3)), (dot(Ac), F(1, 6))]
    if order >= 4:
        conds += [(dot([x ** 3 for x in c]), F(1, 4)), (dot([c[i] * Ac[i] for i in range(s)]), F(1, 8)),
                  (dot(Ac2), F(1, 12)), (dot(AAc), F(1, 24))]
    if order >= 5:
        conds += [(dot([x ** 4 for x in c]), F(1, 5)), (dot([c[i] ** 2 * Ac[i] for i in range(s)]), F(1, 10)),
                  (dot([c[i] * Ac2[i] for i in range(s)]), F(1, 15)), (dot([c[i] * AAc[i] for i in range(s)]), F(1, 30)),
                  (dot([Ac[i] ** 2 for i in range(s)]), F(1, 20)), (dot(Ac3), F(1, 20)), (dot(AcAc), F(1, 40)),
                  (dot(AAc2), F(1, 60)), (dot(AAAc), F(1, 120))]
    return [got - want for got, want in conds]


def test_tableau_rows_and_order_conditions():
    c, A, e, _ = _tableau()
    for i in range(7):
        assert sum(A[i]) == c[i]
    b = A[6][:6] + [Fraction(0)]  # first same as last: the last stage is evaluated at the new point
    assert all(r == 0 for r in _conditions(b, c, A, 5))
    assert len(_conditions(b, c, A, 5)) == 17
    b_hat = [b[j] - e[j] for j in range(7)]
    assert all(r == 0 for r in _conditions(b_hat, c, A, 4))
    assert any(r != 0 for r in _conditions(b_hat, c, A, 5))


def test_continuous_extension_is_order_four():
    sympy = pytest.importorskip("sympy")
    c, A, e, d = _tableau()
    th = sympy.Symbol("theta")
    S = [sympy.Rational(x.numerator, x.denominator) for x in c]
    M = [[sympy.Rational(x.numerator, x.denominator) for x in row] for row in A]
    b = M[6][:6] + [sympy.Integer(0)]
    D = [sympy.Rational(x.numerator, x.denominator) for x in d]
    e1 = [1, 0, 0, 0, 0, 0, 0]
    e7 = [0, 0, 0, 0, 0, 0, 1]
    # y(theta) = x + theta (yd + (1 - theta)(bspl + theta (r4 + (1 - theta) r5))) with
    # yd = h sum b k, bspl = h k1 - yd, r4 = yd - h k7 - bspl, r5 = h sum D k
    w = [sympy.expand(th * (b[j] + (1 - th) * ((e1[j] - b[j]) + th * ((2 * b[j] - e1[j] - e7[j]) + (1 - th) * D[j]))))
         for j in range(7)]
    for j in range(7):
        assert sympy.simplify(w[j].subs(th, 1) - b[j]) == 0
    Ac = [sum(M[i][j] * S[j] for j in range(7)) for i in range(7)]
    Ac2 = [sum(M[i][j] * S[j] ** 2 for j in range(7)) for i in range(7)]
    AAc = [sum(M[i][j] * Ac[j] for j in range(7)) for i in range(7)]
    checks = [
        (sum(w), th), (sum(w[j] * S[j] for j in range(7)), th ** 2 / 2),
        (sum(w[j] * S[j] ** 2 for j in range(7)), th ** 3 / 3), (sum(w[j] * Ac[j] for j in range(7)), th ** 3 / 6),
        (sum(w[j] * S[j] ** 3 for j in range(7)), th ** 4 / 4), (sum(w[j] * S[j] * Ac[j] for j in range(7)), th ** 4 / 8),
        (sum(w[j] * Ac2[j] for j in range(7)), th ** 4 / 12), (sum(w[j] * AAc[j] for j in range(7)), th ** 4 / 24)]
    for got, want in checks:
        assert sympy.expand(got - want) == 0


def _closed_form(x0, t, v0):
    s = x0.reshape(-1, 4)
    phi0, om0 = s[:, 2], s[:, 3]
    phi = phi0 + om0 * t
    out = s.copy()
    out[:, 0] = s[:, 0] + v0 * (np.sin(phi) - np.sin(phi0)) / om0
    out[:, 1] = s[:, 1] - v0 * (np.cos(phi) - np.cos(phi0)) / om0
    out[:, 2] = phi
    return out.reshape(-1)


def closed_form_case(n=200, seed=5):
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 4))
    x[:, 0], x[:, 1] = rng.random(n), rng.random(n)
    x[:, 2] = rng.uniform(-np.pi, np.pi, n)
    x[:, 3] = rng.uniform(0.5, 2.0, n) * rng.choice([-1.0, 1.0], n)
    # sigma = 0 and xi = 0: every particle moves on its own circle
    return dict(model=1, n=n, rho=0.05, flavor="ptr", v0=0.3, xi=0.0, sigma=0.0, alpha=0.0), x.reshape(-1)


def test_restated_integrator_on_a_closed_form_solution():
    from helpers import oracle_system
    from oracle import dopri5_oracle as dp

    p, x0 = closed_form_case()
    steps = {}
    for tol in (1e-6, 1e-10):
        orc = oracle_system(p)
        times, states, steps[tol] = dp.integrate(orc, 1, x0, 0.0, 3.0, 0.25, tol, tol)
        orc.close()
        for t, x in zip(times, states):
            exact = _closed_form(x0, t, p["v0"])
            assert np.max(np.abs(x - exact) / (1.0 + np.abs(exact))) <= 10 * tol, (tol, t)
    ratio = steps[1e-10] / steps[1e-6]
    assert 4.0 <= ratio <= 10.0, steps
