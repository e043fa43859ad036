"""CPU: the surrogate network's NumPy oracle. Without bf16 rounding its
gradient is checked against central finite differences of its own loss, so
the backward pass that the GPU gradient is compared with is itself pinned."""
import numpy as np

from oracle import surrogate_oracle as SO


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e-3, 0.0])
    r = SO.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0 + 2 ** -7
    assert r[3] == -2.5 and r[5] == 0.0
    assert abs(r[4] - 3.0e-3) <= 2 ** -8 * 3.0e-3


def test_oracle_gradient_finite_differences():
    rng = np.random.default_rng(0)
    offs, P = SO.offsets()
    params = np.zeros(P)
    for (ci, co, _), (wo, bo) in zip(SO.LAYERS, offs):
        params[wo:bo] = rng.normal(0, np.sqrt(2.0 / (27 * ci)), bo - wo)
        params[bo:bo + co] = rng.normal(0, 0.05, co)
    m = 4
    feats = rng.uniform(-1, 1, (1, m, m, m, 16))
    targ = rng.uniform(0, 1, (1, m, m, m))
    loss, g = SO.loss_and_grad(params, feats, targ, rounding=False)
    h = 1e-6
    for k, (wo, bo) in enumerate(offs):
        for idx in (wo + 7, wo + (bo - wo) // 2, bo):  # two weights and a bias per layer
            e = np.zeros(P)
            e[idx] = h
            fd = (SO.loss_and_grad(params + e, feats, targ, rounding=False)[0] -
                  SO.loss_and_grad(params - e, feats, targ, rounding=False)[0]) / (2 * h)
            assert abs(fd - g[idx]) <= 1e-6 * max(abs(fd), 1e-3), (k, idx, fd, g[idx])
