"""The surrogate MLP on the tensor cores (tcgen05 GEMMs through the C ABI)
against its CPU oracle.

Tolerances: the oracle applies the same BF16 rounding points as the GPU, so
they differ only by FP32 summation order and erff/expf ulps, which now and
then flips one BF16 rounding of an activation: outputs agree to 1e-2 of
their scale (mean 2e-3), gradients to 2e-2 in relative norm per layer.
"""
import os

import numpy as np
import pytest

from mlp_oracle import MlpOracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built():
    import __graft_entry__
    __graft_entry__.build()
    return True


def _net(n_in, n_out, members=2, depth=4, seed=3):
    from fcs import _lib
    return _lib.Mlp(n_in, n_out, width=256, depth=depth, members=members, seed=seed)


def _oracle(mlp, member, exact=False):
    im, is_, om, os_ = mlp.get_normalization()
    return MlpOracle(mlp.unflatten(mlp.get_params(member)), im, is_, om, os_, exact=exact)


@pytest.mark.parametrize("n_in,n_out,n", [(114, 113, 300), (13, 12, 128), (203, 202, 1000)])
def test_forward_matches_oracle(built, n_in, n_out, n):
    rng = np.random.default_rng(n_in)
    mlp = _net(n_in, n_out)
    mlp.set_normalization(rng.normal(0, 0.5, n_in), rng.uniform(0.5, 2.0, n_in), rng.normal(0, 1, n_out),
                          rng.uniform(0.1, 3.0, n_out))
    x = rng.normal(0, 1, (n, n_in)).astype(np.float32)
    for member in range(mlp.members):
        y = mlp.forward(member, x)
        ref, _, _ = _oracle(mlp, member).forward(x)
        scale = np.abs(ref).max()
        err = np.abs(y - ref)
        assert err.max() <= 1e-2 * scale, (member, err.max(), scale)
        assert err.mean() <= 2e-3 * scale
    mlp.close()


def test_forward_device_pointers(built):
    import torch
    rng = np.random.default_rng(5)
    mlp = _net(30, 20, members=1)
    x = rng.normal(0, 1, (257, 30)).astype(np.float32)
    yh = mlp.forward(0, x)
    yd = mlp.forward(0, torch.from_numpy(x).cuda(), device=True)
    np.testing.assert_array_equal(yd.cpu().numpy(), yh)
    mlp.close()


def test_gradients_match_oracle(built):
    rng = np.random.default_rng(7)
    n_in, n_out, n = 114, 113, 512
    mlp = _net(n_in, n_out, members=1)
    mlp.set_normalization(np.zeros(n_in), np.ones(n_in), rng.normal(0, 0.1, n_out), rng.uniform(0.5, 2, n_out))
    x = rng.normal(0, 1, (n, n_in)).astype(np.float32)
    t = rng.normal(0, 1, (n, n_out)).astype(np.float32)
    loss, g = mlp.gradients(0, x, t)
    g_layers = mlp.unflatten(g)
    lo, go = _oracle(mlp, 0).gradients(x, t)
    le, ge = _oracle(mlp, 0, exact=True).gradients(x, t)
    assert abs(loss - lo) <= 1e-3 * lo
    for l, ((dW, db), (oW, ob), (eW, eb)) in enumerate(zip(g_layers, go, ge)):
        assert np.linalg.norm(dW - oW) <= 2e-2 * np.linalg.norm(oW), l
        assert np.linalg.norm(db - ob) <= 2e-2 * np.linalg.norm(ob), l
        # and the BF16 gradient is a gradient of the FP64 loss
        assert np.linalg.norm(dW - eW) <= 0.1 * np.linalg.norm(eW), l
    mlp.close()


def test_training_fits_a_smooth_map(built, tmp_path):
    rng = np.random.default_rng(11)
    n_in, n_out, n = 16, 8, 16384
    A = rng.normal(0, 1, (n_in, n_out)) / np.sqrt(n_in)
    x = rng.normal(0, 1, (n, n_in)).astype(np.float32)
    t = (np.tanh(x @ A) + 0.1 * (x[:, :n_out] ** 2)).astype(np.float32)
    mlp = _net(n_in, n_out, members=2)
    mlp.set_normalization(x.mean(0), x.std(0), t.mean(0), t.std(0))
    hist = mlp.train(x, t, epochs=8, batch=1024, lr=2e-3)
    assert np.all(np.isfinite(hist))
    for m in range(2):
        assert hist[m, -1] < 0.1 * hist[m, 0], hist[m]
    # unseen inputs
    xv = rng.normal(0, 1, (2048, n_in)).astype(np.float32)
    tv = np.tanh(xv @ A) + 0.1 * (xv[:, :n_out] ** 2)
    yv = mlp.forward(0, xv)
    assert np.mean((yv - tv) ** 2) < 0.05 * np.var(tv)
    # save / load round trip
    path = str(tmp_path / "mlp.bin")
    mlp.save(path)
    from fcs import _lib
    m2 = _lib.Mlp(path=path)
    np.testing.assert_array_equal(m2.forward(1, xv), mlp.forward(1, xv))
    assert m2.members == 2 and m2.n_in == n_in
    m2.close()
    mlp.close()
