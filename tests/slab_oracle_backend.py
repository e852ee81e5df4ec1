"""TEST INFRASTRUCTURE — a CPU stand-in for CudaSlabBackend, built on the oracle.

The z-slab host logic (ambient_image_processor_gb300/slab.py) is tested on the CPU
with this backend: the loop steps are the oracle's own iteration (oracle.tgv2_step),
the divergence is the oracle's, and the separable contractions are FP64 numpy sums
taken in a fixed order (index 0 to N-1) for every output value, so a value does not
depend on how many lines or columns a call holds.  A split run must then reproduce a
single-volume run of the same backend bit for bit."""
import math

import numpy as np
import torch

import oracle
from ambient_image_processor_gb300 import slab

# field-mask bit -> oracle state key
_BITS = {0: "f", 1: "u", 2: "v_x", 3: "v_y", 4: "v_z", 5: "u_bar", 6: "vbar_x", 7: "vbar_y",
         8: "vbar_z", 9: "p_x", 10: "p_y", 11: "p_z", 12: "q_xx", 13: "q_yy", 14: "q_zz",
         15: "q_xy", 16: "q_xz", 17: "q_yz"}


def _keys(mask):
    return [_BITS[b] for b in range(18) if mask & (1 << b)]


def dct_matrices(n):
    k = np.arange(n)[:, None]
    m = np.arange(n)[None, :]
    C = np.cos(math.pi * (m + 0.5) * k / n)  # forward: row k, column m
    S = (C * np.where(np.arange(n) == 0, 1.0, 2.0)[:, None]).T  # inverse: row m, column k
    return C, S


def contract(M, x, axis):
    """out[.., k, ..] = sum_n M[k, n] x[.., n, ..] along `axis`, summed n = 0, 1, ...
    for every output value."""
    x = np.moveaxis(x, axis, -1)
    acc = np.zeros(x.shape[:-1] + (M.shape[0],))
    for n in range(M.shape[1]):
        acc += x[..., n:n + 1] * M[:, n]
    return np.moveaxis(acc, -1, axis)


class OracleSlabBackend:
    def __init__(self, geo, lambda_=1.0, alpha0=2.0, alpha1=1.0):
        self.geo = geo
        self.prm = dict(lambda_=lambda_, alpha0=alpha0, alpha1=alpha1)
        self.Dl = geo.local_depth
        self.st = None

    def init(self, f_local):
        self.st = oracle.tgv2_initial_state(np.ascontiguousarray(f_local.numpy()))

    def step(self):
        oracle.tgv2_step(self.st, 1, **self.prm)

    def read(self, mask, plane):
        return torch.from_numpy(np.concatenate([self.st[k][plane].ravel() for k in _keys(mask)]))

    def read_all(self, mask):
        return torch.from_numpy(np.concatenate([self.st[k].ravel() for k in _keys(mask)]))

    def write(self, mask, plane, buf):
        a = buf.numpy()
        n = self.geo.width * self.geo.height
        for j, k in enumerate(_keys(mask)):
            self.st[k][plane] = a[j * n:(j + 1) * n].reshape(self.geo.height, self.geo.width)

    def poisson_xy(self, vx, vy, vz):
        d = oracle.divergence(*(np.asarray(t.numpy(), np.float64) for t in (vx, vy, vz)))
        d = contract(dct_matrices(self.geo.width)[0], d, 2)
        return torch.from_numpy(contract(dct_matrices(self.geo.height)[0], d, 1))

    def pencil_z(self, pencil, column_begin):
        W, H, D = self.geo.width, self.geo.height, self.geo.depth
        x = pencil.numpy()
        C, S = dct_matrices(D)
        y = contract(C, x, 0) * 8.0
        cols = column_begin + np.arange(x.shape[1])
        kx, ky = cols % W, cols // W
        kz = np.arange(D)[:, None]
        den = 6.0 - 2.0 * np.cos(math.pi * kx / W) - 2.0 * np.cos(math.pi * ky / H) \
            - 2.0 * np.cos(math.pi * kz / D)
        y = np.where((kx == 0) & (ky == 0) & (kz == 0), 0.0, y / np.where(den == 0, 1.0, den))
        return torch.from_numpy(contract(S, y, 0))

    def poisson_inverse_yx(self, own, total_depth):
        W, H = self.geo.width, self.geo.height
        y = contract(dct_matrices(H)[1], own.numpy(), 1)
        return torch.from_numpy(contract(dct_matrices(W)[1], y, 2) / (8.0 * W * H * total_depth))
