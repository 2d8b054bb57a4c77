"""The NumPy restatement of the learned-start network (oracle/mlp_ref.py) against
finite differences of its own loss (the network has no counterpart in the
reference, so the oracle's gradient formulas are pinned this way), and its
BF16-rounded gradient against the unrounded one. CPU only."""
import numpy as np

from oracle import mlp_ref as R


def small_problem(width=64, n_bits=12, dim=40, npts=3, seed=0):
    rng = np.random.default_rng(seed)
    _, n, k0 = R.layout(n_bits, width)
    w = (rng.standard_normal(n) * 0.3).astype(np.float64)
    ids = rng.choice(1 << n_bits, size=dim, replace=False).astype(np.uint64)
    conds = [(0.5 * p, 0.05 * p) for p in range(npts)]
    targets = rng.standard_normal(npts * dim)
    return w, n_bits, width, ids, conds, targets


def test_gradient_matches_finite_differences():
    w, nb, W, ids, conds, tg = small_problem()
    g = R.grad_exact(w, nb, W, ids, conds, tg)
    rng = np.random.default_rng(1)
    for _ in range(4):
        v = rng.standard_normal(w.size)
        v /= np.linalg.norm(v)
        h = 1e-5
        fd = (R.loss_exact(w + h * v, nb, W, ids, conds, tg) - R.loss_exact(w - h * v, nb, W, ids, conds, tg)) / (2 * h)
        assert abs(fd - g @ v) <= 1e-6 * max(1.0, abs(fd)), (fd, g @ v)


def test_bf16_gradient_close_to_exact():
    w, nb, W, ids, conds, tg = small_problem()
    w32 = w.astype(np.float32)
    L, g = R.loss_grad(w32, nb, W, ids, conds, tg)
    ge = R.grad_exact(w32.astype(np.float64), nb, W, ids, conds, tg)
    assert np.linalg.norm(g - ge) <= 3e-2 * np.linalg.norm(ge)
    assert abs(L - R.loss_exact(w32.astype(np.float64), nb, W, ids, conds, tg)) <= 1e-2


def test_bf16_rounding():
    """Nearest BF16 (8-bit significand), ties to even."""
    x = np.array([1.0, 1.00390625, 1.01171875, 1.005, -3.14159, 0.0], np.float32)
    y = R.bf16(x)
    assert list(y[:4]) == [1.0, 1.0, 1.015625, 1.0078125]
    assert abs(y[4] + 3.140625) < 1e-7 and y[5] == 0.0
