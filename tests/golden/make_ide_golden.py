"""Generate tests/golden/ide_deg4.npz: the reference's own integrated
directional encoding (models/utils.py:209-273, generate_ide_fn) of degree 4
on seeded inputs, imported through ``oracle.ref_harness``.

Run from the repository root, in a container that has the reference tree:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_ide_golden.py /root/reference

Inputs: 64 unit directions, 32 vectors (r + 1) / 2 of unit directions r (the
form the reference's reflection texture feeds, models/texture.py:91-95) and
roughness values in (0, 1), all float32 as the reference evaluates them.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref_harness as H  # noqa: E402


def main(reference_root):
    H.install(reference_root)
    import models.utils as U
    if not hasattr(np, "math"):
        import math
        np.math = math           # the reference calls np.math.factorial
    g = np.random.default_rng(17)
    d = g.normal(size=(64, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = g.normal(size=(32, 3))
    r /= np.linalg.norm(r, axis=1, keepdims=True)
    xyz = np.concatenate([d, (r + 1.0) / 2.0])
    kappa = g.uniform(0.0, 1.0, size=(96, 1))
    fn = U.generate_ide_fn(4)
    xyz, kappa = xyz.astype(np.float32), kappa.astype(np.float32)   # the reference keeps its
    out = fn(torch.from_numpy(xyz), torch.from_numpy(kappa)).numpy()  # coefficients in float32
    np.savez(os.path.join(HERE, "ide_deg4.npz"), xyz=xyz, kappa_inv=kappa, ide=out.astype(np.float64))
    print("ide_deg4.npz", out.shape)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_ide_golden.py <path of the Instant-angelo source tree>")
    main(sys.argv[1])
