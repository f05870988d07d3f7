"""The MLP oracle (oracle/mlp_oracle.py) on the CPU: its analytic gradients against central finite
differences of its own float64 loss, and its bf16 rounding against a reference conversion."""
import numpy as np

from oracle import mlp_oracle as M


def test_bf16_rounding_matches_torch_style_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 65504.0, 1e-3], np.float32)
    r = M.bf16(x)
    # bf16 keeps 8 significant bits; ties go to even
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] - (-3.140625)) < 1e-12
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)


def test_analytic_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.standard_normal(M.NPARAM) * 0.1
    x = rng.random((32, M.IN))
    y = (rng.random((32, M.OUT)) < 0.5).astype(np.float64)
    _, g = M.loss_and_grads(p, x, y, bf16_rounding=False)
    for idx in list(rng.integers(0, M.NPARAM, 40)) + [M.P_B3, M.P_B3 + 2, M.P_W1 + 5, M.P_B1 + 7]:
        e = np.zeros(M.NPARAM)
        e[idx] = 1e-6
        lp, _ = M.loss_and_grads(p + e, x, y, bf16_rounding=False)
        lm, _ = M.loss_and_grads(p - e, x, y, bf16_rounding=False)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[idx]) <= 1e-6 + 1e-4 * abs(fd), (idx, fd, g[idx])
