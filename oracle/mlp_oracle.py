"""CPU oracle of the surrogate MLP (test infrastructure only: used by tests/,
never by the library).

The surrogate has no counterpart in the reference, so this is a plain numpy
statement of the network the library's tensor-core kernels compute, with
the same rounding points:

  x_n  = bf16((x - in_mean) * (1 / in_std))
  z_l  = h_{l-1} . bf16(W_l)^T + b_l          (FP32 accumulation)
  h_l  = bf16(GELU(z_l)),  GELU(z) = z/2 (1 + erf(z / sqrt 2))
  y    = h_d . bf16(W_d)^T + b_d              (normalised output)
  loss = mean over samples and outputs of (y - (t - out_mean) / out_std)^2
  backward: dOut = bf16(2 (y - t_n) / (n n_out)),
            dz_l = bf16((dz_{l+1} . bf16(W_{l+1})) * GELU'(bf16(z_l))),
            dW_l = dz_l^T . h_{l-1},  db_l = sum over samples of dz_l.

`exact=True` drops every BF16 rounding and works in FP64 (the gradient
of the same loss without reduced precision).
"""
import numpy as np
from scipy.special import erf


def bf16(a):
    """Round FP32 values to the nearest BF16 (ties to even), kept as FP32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    out = ((u + r) & 0xFFFF0000).astype(np.uint32)
    return out.view(np.float32)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


class MlpOracle:
    def __init__(self, layers, in_mean, in_std, out_mean, out_std, exact=False):
        """layers: [(W[out][in], b[out])] in order."""
        self.exact = exact
        dt = np.float64 if exact else np.float32
        self.dt = dt
        self.layers = [(np.asarray(W, dt), np.asarray(b, dt)) for W, b in layers]
        self.in_mean = np.asarray(in_mean, dt)
        self.in_rstd = (1.0 / np.asarray(in_std, dt)).astype(dt)
        self.out_mean = np.asarray(out_mean, dt)
        self.out_std = np.asarray(out_std, dt)

    def _r(self, a):
        return a.astype(self.dt) if self.exact else bf16(a)

    def forward(self, x, normalised=False):
        """Returns y (de-normalised unless normalised=True) and the saved activations."""
        x = np.asarray(x, self.dt)
        h = self._r((x - self.in_mean) * self.in_rstd)
        acts, zs = [h], []
        for W, b in self.layers[:-1]:
            z = (h @ self._r(W).T + b).astype(self.dt)
            zs.append(self._r(z))
            h = self._r(gelu(z).astype(self.dt))
            acts.append(h)
        W, b = self.layers[-1]
        y = (h @ self._r(W).T + b).astype(self.dt)
        if not normalised:
            y = y * self.out_std + self.out_mean
        return y, acts, zs

    def gradients(self, x, target):
        """loss and [(dW, db)] per layer, as the library's fcs_mlp_gradients."""
        y, acts, zs = self.forward(x, normalised=True)
        n, n_out = y.shape
        tn = (np.asarray(target, self.dt) - self.out_mean) / self.out_std
        d = y - tn
        loss = float(np.mean(d.astype(np.float64) ** 2))
        dz = self._r((2.0 / (n * n_out)) * d)
        grads = [None] * len(self.layers)
        for l in range(len(self.layers) - 1, -1, -1):
            h_in = acts[l]
            grads[l] = ((dz.T @ h_in).astype(self.dt), dz.sum(axis=0).astype(self.dt))
            if l > 0:
                W, _ = self.layers[l]
                dh = (dz @ self._r(W)).astype(self.dt)
                dz = self._r(dh * gelu_grad(zs[l - 1]))
        return loss, grads
