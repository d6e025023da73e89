"""CPU: pin the learned-predictor oracle (oracle/mlp_port.py).  Without BF16
rounding its analytic gradient must match central finite differences of its
own loss; its BF16 rounding must match the hardware rule (nearest, ties to
even) on hand-picked bit patterns."""
import numpy as np

from oracle import mlp_port as mp


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    m = 8
    X = rng.uniform(-1, 1, (m, mp.IN_PAD))
    X[:, 129:] = 0.0
    T = rng.uniform(-1, 1, (m, mp.OUT))
    p = rng.normal(0, 0.2, mp.NPARAMS)
    p[mp.P_B1:mp.P_W2] = 0.05  # keep hidden units away from the ReLU kink
    loss, g = mp.loss_and_grad(p, X, T, rnd=False)
    idx = np.concatenate([rng.choice(np.arange(a, b), 12, replace=False) for a, b in
                          [(mp.P_W1, mp.P_B1), (mp.P_B1, mp.P_W2), (mp.P_W2, mp.P_B2),
                           (mp.P_B2, mp.P_W3), (mp.P_W3, mp.P_B3), (mp.P_B3, mp.NPARAMS)]])
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (mp.loss_and_grad(pp, X, T, rnd=False)[0] - mp.loss_and_grad(pm, X, T, rnd=False)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_bf16_rounding_rule():
    one = np.float32(1.0)
    ulp = np.float32(2.0 ** -7)
    vals = np.array([one, one + ulp / 2, one + ulp + ulp / 2, -one - ulp / 4, np.float32(3.0e38),
                     np.float32(1e-40)], np.float32)
    got = mp.bf16(vals)
    assert got[0] == 1.0
    assert got[1] == 1.0                    # tie -> even (1.0)
    assert got[2] == 1.0 + 2 * ulp          # tie -> even (1 + 2 ulp)
    assert got[3] == -1.0
    assert np.isfinite(got[4])
    assert np.array_equal(mp.from_bits(mp.bf16_bits(vals)), got)
