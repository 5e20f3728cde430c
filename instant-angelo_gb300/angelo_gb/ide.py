"""Integrated directional encoding (Ref-NeRF, Verbin et al. 2022, eq. 6-8),
the reflected-direction encoding of the reference's reflection textures
(models/utils.py:209-273, used by models/texture.py:73-99 when use_ide).

For degrees l = 1, 2, 4, ..., 2^(deg-1) and orders m = 0..l, the encoding of a
direction xyz with roughness kappa_inv is

    Y_l^m(xyz) exp(-l (l + 1) / 2 * kappa_inv),
    Y_l^m(xyz) = (x + i y)^m * N_lm * (-1)^m d^m P_l / dz^m (z),
    N_lm = sqrt((2l + 1) / (4 pi) * (l - m)! / (l + m)!),

real parts of every (l, m) first, then the imaginary parts.  The polynomial
form is evaluated as written also for vectors that are not unit length (the
reference feeds (r + 1) / 2 of the reflected direction r)."""
from __future__ import annotations

import math

import numpy as np
import torch
from numpy.polynomial import legendre as npl
from numpy.polynomial import polynomial as npp


def ml_pairs(deg):
    """(m, l) of the encoding, in output order."""
    return [(m, 2 ** i) for i in range(deg) for m in range(2 ** i + 1)]


def _poly_coefficients(deg):
    """Coefficients (n_pairs, l_max + 1) of N_lm (-1)^m d^m P_l / dz^m in
    powers of z."""
    pairs = ml_pairs(deg)
    l_max = 2 ** (deg - 1)
    C = np.zeros((len(pairs), l_max + 1))
    for i, (m, l) in enumerate(pairs):
        p = npl.leg2poly(np.eye(l + 1)[l])          # P_l in powers of z
        if m:
            p = npp.polyder(p, m)
        norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - m) / math.factorial(l + m))
        C[i, :len(p)] = (-1) ** m * norm * p
    return C


class IntegratedDirEncoding(torch.nn.Module):
    """IDE of degree `deg` (2 * sum(2^i + 1) outputs: 38 for deg 4)."""

    def __init__(self, deg=4):
        super().__init__()
        pairs = ml_pairs(deg)
        self.deg = int(deg)
        self.register_buffer("coef", torch.tensor(_poly_coefficients(deg), dtype=torch.float32),
                             persistent=False)
        self.register_buffer("m", torch.tensor([m for m, _ in pairs], dtype=torch.int64),
                             persistent=False)
        self.register_buffer("sigma", torch.tensor([0.5 * l * (l + 1) for _, l in pairs],
                                                   dtype=torch.float32), persistent=False)
        self.n_output_dims = 2 * len(pairs)

    def forward(self, xyz, kappa_inv):
        dt = xyz.dtype
        x, y, z = xyz[..., 0:1], xyz[..., 1:2], xyz[..., 2:3]
        k = self.coef.shape[1]
        zp = torch.cat([z ** i for i in range(k)], dim=-1)                  # (..., k)
        poly = zp @ self.coef.to(dt).T                                       # (..., pairs)
        # (x + i y)^m by repeated complex multiplication, m = 0 .. max
        m_max = int(self.m.max())
        re, im = [torch.ones_like(x)], [torch.zeros_like(x)]
        for _ in range(m_max):
            r0, i0 = re[-1], im[-1]
            re.append(r0 * x - i0 * y)
            im.append(r0 * y + i0 * x)
        re, im = torch.cat(re, -1)[..., self.m], torch.cat(im, -1)[..., self.m]
        att = torch.exp(-self.sigma.to(dt) * kappa_inv)
        return torch.cat([re * poly * att, im * poly * att], dim=-1)
