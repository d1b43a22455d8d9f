"""CPU oracle of the learned surrogate (test infrastructure only: the tests,
the smoke check and the benchmark's CPU leg use it as the checker; the
product never calls it).

The network of include/spss_surrogate.h — 5 -> 128 -> 128 -> 128 -> 4, exact
(erf) GELU after the hidden layers — restated in FP64 numpy.  With
``bf16=True`` the values are rounded to BF16 exactly where the GPU kernels
round them (inputs, weight copies, hidden activations, the back-propagated
dZ operands), so the GPU's remaining differences are FP32 accumulation order
and FP32 GELU; with ``bf16=False`` it is the plain FP64 network, whose
gradient the tests pin against central finite differences.  The reference
has no learned part, so nothing here follows reference code.
"""
import numpy as np
from scipy.special import erf

IN, H, OUT = 5, 128, 4
SHAPES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
          ("W4", (OUT, H)), ("b4", (OUT,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(flat):
    """Flat parameter vector (spss_surrogate.h order) -> dict of arrays (FP64)."""
    flat = np.asarray(flat, dtype=np.float64)
    assert flat.size == NPARAMS
    out, o = {}, 0
    for name, shape in SHAPES:
        size = int(np.prod(shape))
        out[name] = flat[o:o + size].reshape(shape)
        o += size
    return out


def pack(params):
    return np.concatenate([np.asarray(params[name], dtype=np.float64).reshape(-1) for name, _ in SHAPES])


def to_bf16(x):
    """Round to the nearest BF16 (ties to even), via FP32, returned as FP64."""
    f = np.asarray(x, dtype=np.float32)
    bits = f.view(np.uint32).astype(np.uint64)
    rounded = ((bits + 0x7FFF + ((bits >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    out = rounded.view(np.float32).astype(np.float64)
    # NaN and infinity pass through unchanged
    special = ~np.isfinite(f)
    if np.any(special):
        out = np.where(special, f.astype(np.float64), out)
    return out


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def forward(flat, x, bf16=True):
    """Outputs [n][4] and the cache the backward pass needs."""
    P = unpack(flat)
    r = to_bf16 if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    a = r(x)
    cache = {"a0": a}
    for l, (W, b) in enumerate((("W1", "b1"), ("W2", "b2"), ("W3", "b3")), start=1):
        z = a @ r(P[W]).T + P[b]
        a = r(gelu(z))
        cache["z%d" % l], cache["a%d" % l] = z, a
    y = a @ r(P["W4"]).T + P["b4"]
    return y, cache


def loss_and_gradient(flat, x, t, w=None, bf16=True):
    """loss = (1/n) sum_i sum_o w_o (y_io - t_io)^2 and its gradient (flat)."""
    P = unpack(flat)
    r = to_bf16 if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    w = np.ones(OUT) if w is None else np.asarray(w, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    n = x.shape[0]
    y, c = forward(flat, x, bf16=bf16)
    d = y - t
    loss = float(np.sum(w * d * d) / n)
    dz = r(2.0 * w * d / n)  # [n][4]
    g = {"W4": dz.T @ c["a3"], "b4": dz.sum(axis=0)}
    Wn = {"3": "W4", "2": "W3", "1": "W2"}
    for l in (3, 2, 1):
        da = dz @ r(P[Wn[str(l)]])
        dz = r(da * gelu_grad(c["z%d" % l]))
        g["W%d" % l] = dz.T @ c["a%d" % (l - 1)]
        g["b%d" % l] = dz.sum(axis=0)
    return loss, pack(g)


def adam_step(flat, grad, m1, m2, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update (the optimiser the training kernels run), FP64."""
    m1 = beta1 * m1 + (1.0 - beta1) * grad
    m2 = beta2 * m2 + (1.0 - beta2) * grad * grad
    mh = m1 / (1.0 - beta1 ** step)
    vh = m2 / (1.0 - beta2 ** step)
    return flat - lr * mh / (np.sqrt(vh) + eps), m1, m2


def init_params(seed):
    """Uniform +-1/sqrt(fan_in) weights, zero biases (a seeded FP64 draw; the
    library's own initialisation uses its own generator)."""
    rng = np.random.default_rng(seed)
    P = {}
    for name, shape in SHAPES:
        if name.startswith("W"):
            bound = 1.0 / np.sqrt(shape[1])
            P[name] = rng.uniform(-bound, bound, shape)
        else:
            P[name] = np.zeros(shape)
    return pack(P)
