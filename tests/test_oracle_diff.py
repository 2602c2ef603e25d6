"""The oracle's adjoint of the differentiable batch (binary64) against
central finite differences of the oracle's forward with the bisection tree
held fixed (h = 1e-3 px), for both fill rules and paths crossing the image
edges (the x rules)."""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.mark.parametrize("rule,margin", [(0, 0.0), (1, 0.0), (0, 12.0)])
def test_oracle_adjoint_matches_finite_differences(rule, margin):
    rng = np.random.default_rng(3 + rule)
    P, S, W, H = 5, 6, 48, 40
    ctrl = rng.uniform(-margin, [W + margin, H + margin], size=(P, 3 * S, 2))
    target = ctrl + rng.normal(0.0, 2.0, ctrl.shape)
    T = O.diff_forward(target, P, S, W, H, rule=rule)

    def loss(c, frozen=None):
        A = O.diff_forward(c, P, S, W, H, rule=rule, frozen=frozen)
        return float(((A - T) ** 2).sum()), A

    _, A = loss(ctrl)
    grad = O.diff_backward(ctrl, P, S, W, H, A, 2.0 * (A - T), rule=rule)
    h = 1e-3
    for _ in range(30):
        p, j, c = rng.integers(P), rng.integers(3 * S), rng.integers(2)
        cp, cm = ctrl.copy(), ctrl.copy()
        cp[p, j, c] += h
        cm[p, j, c] -= h
        fd = (loss(cp, frozen=ctrl)[0] - loss(cm, frozen=ctrl)[0]) / (2 * h)
        assert abs(grad[p, j, c] - fd) <= 1e-4 * max(1.0, abs(fd)), (p, j, c, grad[p, j, c], fd)
