"""CPU oracle of the adaptive Dormand-Prince 5(4) integration with dense
output (test infrastructure only; the product is spss_integrate_dopri5).

The reference integrates with Boost.Odeint's dense-output dopri5
(SimulationEngineFirstOrder.cpp:158-165); Boost is not in the reference tree
and its version is not pinned, so this restates the published method exactly
as the GPU version does — the Dormand-Prince tableau (first same as last),
odeint's documented default error norm and step-size rule, and the continuous
extension of Hairer, Norsett & Wanner — over the FP64 oracle's right-hand side
(``binding.System.evaluate``).  Parity of the integrator with Boost itself is
unpinned; parity of the right-hand side is pinned by the golden fixtures.
"""
import numpy as np

C = [0.0, 1 / 5, 3 / 10, 4 / 5, 8 / 9, 1.0, 1.0]
A = [[],
     [1 / 5],
     [3 / 40, 9 / 40],
     [44 / 45, -56 / 15, 32 / 9],
     [19372 / 6561, -25360 / 2187, 64448 / 6561, -212 / 729],
     [9017 / 3168, -355 / 33, 46732 / 5247, 49 / 176, -5103 / 18656],
     [35 / 384, 0.0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84]]
E = [71 / 57600, 0.0, -71 / 16695, 71 / 1920, -17253 / 339200, 22 / 525, -1 / 40]
D = [-12715105075 / 11282082432, 0.0, 87487479700 / 32700410799, -10690763975 / 1880347072,
     701980252875 / 199316789632, -1453857185 / 822651844, 69997945 / 29380423]


def integrate(system, variant, x, t0, t1, dt_out, eps_abs, eps_rel):
    """Returns (observer times, states at those times, accepted steps); x is
    the initial FP64 AoS state."""
    x = np.array(x, dtype=np.float64)
    zeros = np.zeros_like(x)
    k = [np.zeros_like(x) for _ in range(7)]

    def rhs(y, out):
        system.evaluate(variant, y, zeros, out, 0.0, 0.0)

    times, states = [t0], [x.copy()]
    n_out = int(np.floor((t1 - t0) / dt_out + 1e-9))
    h, t, idx, steps = dt_out, t0, 1, 0
    rhs(x, k[0])
    while idx <= n_out:
        for s in range(1, 7):
            acc = np.zeros_like(x)
            for j in range(s):
                if A[s][j] != 0.0:
                    acc += A[s][j] * k[j]
            y = x + h * acc
            if s == 6:
                xnew = y
            rhs(y, k[s])
        e = np.zeros_like(x)
        for j in range(7):
            if E[j] != 0.0:
                e += E[j] * k[j]
        err = np.max(np.abs(h * e) / (eps_abs + eps_rel * (np.abs(x) + h * np.abs(k[0]))))
        if err > 1.0:
            h *= max(0.9 * err ** (-1 / 3), 0.2)
            continue
        steps += 1
        t_new = t + h
        d = np.zeros_like(x)
        for j in range(7):
            if D[j] != 0.0:
                d += D[j] * k[j]
        yd = xnew - x
        bspl = h * k[0] - yd
        r4 = yd - h * k[6] - bspl
        r5 = h * d
        while idx <= n_out and t0 + idx * dt_out <= t_new * (1 + 1e-15):
            th = (t0 + idx * dt_out - t) / h
            times.append(t0 + idx * dt_out)
            states.append(x + th * (yd + (1 - th) * (bspl + th * (r4 + (1 - th) * r5))))
            idx += 1
        if idx > n_out:
            break
        x = xnew
        k[0], k[6] = k[6], k[0]
        t = t_new
        if err < 0.5:
            h *= 0.9 * max(err, 5.0 ** -5) ** (-1 / 5)
    return np.array(times), np.array(states), steps
