"""The FP64 network oracle against finite differences (no GPU)."""
import numpy as np

from oracle import mlp_ref


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(2)
    nin, H, K, D = 5, 8, 3, 2
    nout = K + 2 * K * D
    _, n = mlp_ref.offsets(nin, H, nout)
    p = rng.normal(0, 0.4, n)
    x = rng.normal(size=(7, nin))
    t = rng.normal(size=(7, D))
    loss, g = mlp_ref.gradients(p, x, t, nin, H, K, D, bf16=False)
    for idx in rng.choice(n, 25, replace=False):
        e = np.zeros(n)
        e[idx] = 1e-6
        lp, _ = mlp_ref.gradients(p + e, x, t, nin, H, K, D, bf16=False)
        lm, _ = mlp_ref.gradients(p - e, x, t, nin, H, K, D, bf16=False)
        assert abs((lp - lm) / 2e-6 - g[idx]) < 1e-6 + 1e-5 * abs(g[idx])


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.001953125, -3.14159, 1e-30], np.float32)
    r = mlp_ref.to_bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0          # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: round to even
    assert r[2] == 1.0          # 1 + 2^-9 rounds down
    assert abs(r[3] + 3.140625) < 1e-6
