"""CPU checks of the sign-risk network's FP64 restatement (oracle/mlp_oracle.py): its
BF16 rounding against torch's, and its backward formulas against central finite
differences of the unrounded loss."""
import numpy as np
import pytest

from oracle import mlp_oracle as M


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(0, 1, 20000), rng.normal(0, 1e-30, 100), rng.normal(0, 1e30, 100),
                        [0.0, -0.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -(1.0 + 2 ** -8)]]).astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(M.bf16(x), ref)


def test_backward_formulas_finite_differences():
    rng = np.random.default_rng(1)
    P = rng.normal(0, 0.3, M.N_PARAMS)
    X = rng.normal(0, 1, (16, M.F))
    y = (rng.random(16) < 0.3).astype(np.float64)
    w = rng.uniform(0.5, 2.0, 16)
    _, g = M.loss_and_grad(P, X, y, w, rounding=False)
    idx = np.concatenate([rng.choice(M.N_PARAMS, 200, replace=False), [M.ob3, M.ow3, M.ob2, M.ob1]])
    eps = 1e-6
    for i in idx:
        e = np.zeros(M.N_PARAMS)
        e[i] = eps
        fd = (M.loss(P + e, X, y, w, rounding=False) - M.loss(P - e, X, y, w, rounding=False)) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-5 * (1 + abs(g[i])), (i, fd, g[i])
