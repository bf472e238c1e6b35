"""The CPU reference of the warm-start network (the checker of the GPU
training kernels): BF16 rounding, and its backward pass against finite
differences of the same network evaluated without rounding."""
import numpy as np

from oracle import mlp_ref


def _blob(seed=0):
    rng = np.random.default_rng(seed)
    b = np.zeros(mlp_ref.OFF_OS + mlp_ref.OUT, np.float64)
    b[:mlp_ref.NPARAM] = rng.normal(0, 0.3, mlp_ref.NPARAM)
    b[mlp_ref.OFF_MU:mlp_ref.OFF_IS] = rng.normal(0, 1, mlp_ref.IN)
    b[mlp_ref.OFF_IS:mlp_ref.OFF_OS] = rng.uniform(0.5, 2, mlp_ref.IN)
    b[mlp_ref.OFF_OS:] = rng.uniform(0.5, 2, mlp_ref.OUT)
    return b


def test_bf16_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 0.0, 1e-40], np.float32)
    r = mlp_ref.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                 # tie -> even mantissa
    assert r[2] == 1.0 + 2 ** -6       # tie -> even (up)
    assert r[3] == -2.5 and r[4] == 0.0
    # every result is representable in BF16
    assert np.all((r.view(np.uint32) & 0xFFFF) == 0)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    blob = _blob(2)
    x = rng.normal(0, 1, (12, mlp_ref.IN))
    y = rng.normal(0, 1, (12, mlp_ref.OUT))
    loss, g = mlp_ref.loss_and_grad(blob, x, y, rounding=False)
    idx = list(range(0, mlp_ref.NPARAM, 97)) + [mlp_ref.OFF_B4, mlp_ref.OFF_B1 + 3, mlp_ref.OFF_W4 + 5]
    eps = 1e-6
    for i in idx:
        bp = blob.copy()
        bm = blob.copy()
        bp[i] += eps
        bm[i] -= eps
        lp, _ = mlp_ref.loss_and_grad(bp, x, y, rounding=False)
        lm, _ = mlp_ref.loss_and_grad(bm, x, y, rounding=False)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])
