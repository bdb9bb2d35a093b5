"""The numpy MLP reference used to check the device training kernels: its
backward pass against finite differences (FP64, no BF16 rounding). CPU only."""
import numpy as np

from oracle import mlp_ref as M


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    w = rng.normal(size=M.NPARAM) * 0.3
    X = rng.normal(size=(40, 16))
    y = rng.uniform(0.2, 0.8, size=40)
    loss, g, _ = M.forward_backward(w, X, y, bf=False)
    h = 1e-6
    idx = rng.choice(M.NPARAM, size=60, replace=False)
    idx = np.concatenate([idx, [M.OFF_B4, M.OFF_W4, M.OFF_B1, M.OFF_W1]])
    for k in idx:
        wp, wm = w.copy(), w.copy()
        wp[k] += h
        wm[k] -= h
        num = (M.forward_backward(wp, X, y, bf=False)[0] - M.forward_backward(wm, X, y, bf=False)[0]) / (2 * h)
        assert abs(num - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-8


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.0078125, 3.14159, -2.5e-5], dtype=np.float32)
    r = M.bf16(a)
    assert r[0] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] - 3.140625) < 1e-12
