"""The CPU oracle of the surrogate MLP: its backward pass is the gradient of
its loss (finite differences in FP64), and its BF16 rounding matches the
definition (no GPU needed)."""
import numpy as np

from mlp_oracle import MlpOracle, bf16


def _random_net(rng, dims, scale=1.0):
    layers = []
    for i in range(len(dims) - 1):
        W = rng.normal(0, scale * np.sqrt(2.0 / dims[i]), (dims[i + 1], dims[i]))
        b = rng.normal(0, 0.1, dims[i + 1])
        layers.append((W, b))
    return layers


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.1415927, 0.0, 65504.0, 1e-30], dtype=np.float32)
    r = bf16(x)
    # representable values stay, halfway 1 + 2^-8 + 2^-9 rounds to even, others to nearest
    assert r[0] == 1.0 and r[1] == np.float32(1.0)  # 1 + 2^-8 is halfway: ties to even
    assert r[4] == 0.0
    u = r.view(np.uint32)
    assert np.all(u & 0xFFFF == 0)
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8)


def test_exact_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    dims = [7, 16, 16, 5]
    layers = _random_net(rng, dims)
    x = rng.normal(0, 1, (32, dims[0]))
    t = rng.normal(0, 1, (32, dims[-1]))
    norm = dict(in_mean=rng.normal(0, 0.1, dims[0]), in_std=rng.uniform(0.5, 2, dims[0]),
                out_mean=rng.normal(0, 0.1, dims[-1]), out_std=rng.uniform(0.5, 2, dims[-1]))
    o = MlpOracle(layers, exact=True, **norm)
    loss, grads = o.gradients(x, t)
    h = 1e-6
    for l, (W, b) in enumerate(layers):
        for (i, j) in [(0, 0), (W.shape[0] - 1, W.shape[1] - 1), (1, 2)]:
            Wp = [(Wk.copy(), bk.copy()) for Wk, bk in layers]
            Wp[l][0][i, j] += h
            lp, _ = MlpOracle(Wp, exact=True, **norm).gradients(x, t)
            Wm = [(Wk.copy(), bk.copy()) for Wk, bk in layers]
            Wm[l][0][i, j] -= h
            lm, _ = MlpOracle(Wm, exact=True, **norm).gradients(x, t)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - grads[l][0][i, j]) <= 1e-6 * max(1.0, abs(fd)), (l, i, j, fd, grads[l][0][i, j])
        bp = [(Wk.copy(), bk.copy()) for Wk, bk in layers]
        bp[l][1][0] += h
        bm = [(Wk.copy(), bk.copy()) for Wk, bk in layers]
        bm[l][1][0] -= h
        fd = (MlpOracle(bp, exact=True, **norm).gradients(x, t)[0] - MlpOracle(bm, exact=True, **norm).gradients(x, t)[0]) / (2 * h)
        assert abs(fd - grads[l][1][0]) <= 1e-6 * max(1.0, abs(fd))


def test_bf16_oracle_close_to_exact():
    rng = np.random.default_rng(1)
    dims = [20, 64, 64, 9]
    layers = _random_net(rng, dims)
    x = rng.normal(0, 1, (256, dims[0]))
    t = rng.normal(0, 1, (256, dims[-1]))
    norm = dict(in_mean=np.zeros(dims[0]), in_std=np.ones(dims[0]), out_mean=np.zeros(dims[-1]),
                out_std=np.ones(dims[-1]))
    _, ge = MlpOracle(layers, exact=True, **norm).gradients(x, t)
    _, gb = MlpOracle(layers, exact=False, **norm).gradients(x, t)
    for (We, be), (Wb, bb) in zip(ge, gb):
        assert np.linalg.norm(We - Wb) <= 0.05 * np.linalg.norm(We)
