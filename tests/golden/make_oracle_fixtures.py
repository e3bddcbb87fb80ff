"""Fixtures made with the oracle at sizes the reference itself cannot run here.

The large-grid configuration (n = 64 on [-10, 10]^3, 48 Gauss-Legendre radial
nodes x the 70-point symmetric design, hard spheres, e = e0 = 0.7) needs
(n_r, n_sigma, n^3) complex128 tables of 14 GB each in the reference's
broadcast form (``src/collision/inelastic_collisions.py:57-137``), beyond this
machine.  The oracle evaluates the same arithmetic one radial node at a time
(``oracle/fs_inelastic.py``, itself pinned to fixtures produced by the
reference at n = 8 / 16 / 32), so its output is the parity target here:

* ``c5_n64.npz`` -- one cell of a seeded 3-component Maxwellian mixture
  (means in [-3, 3]^3, temperatures in [0.5, 3], unit mass); the mixture's
  parameters (f is rebuilt from them), checksums of f, and
  Q = collide(f, with_loss=True), FP64.

Run from the repository root:  ``python tests/golden/make_oracle_fixtures.py``
(a few minutes on 8 cores).  GPU test runs never execute this script.
"""
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import fs_inelastic as fo  # noqa: E402

L10_S = 20.0 / (3.0 + math.sqrt(2.0))  # velocity-mesh "s" giving L = 10


def mixture_params(seed=64, k=3):
    """(weights, means, temperatures) of the seeded mixture."""
    rng = np.random.default_rng(seed)
    w = rng.uniform(0.5, 1.5, k)
    u = rng.uniform(-3.0, 3.0, (k, 3))
    T = rng.uniform(0.5, 3.0, k)
    return w, u, T


def mixture(v, w, u, T):
    """sum_i w_i M(v; u_i, T_i), normalised to unit mass on the grid."""
    V = np.meshgrid(v, v, v, indexing="ij")
    f = 0.0
    for wi, ui, Ti in zip(w, u, T):
        d2 = (V[0] - ui[0]) ** 2 + (V[1] - ui[1]) ** 2 + (V[2] - ui[2]) ** 2
        f = f + wi / (2 * math.pi * Ti) ** 1.5 * np.exp(-d2 / (2 * Ti))
    dv = (v[1] - v[0]) ** 3
    return f / (f.sum() * dv)


def make_c5():
    mesh = fo.Mesh(64, L10_S, 48, 70)
    op = fo.FSInelasticVHS(mesh, 0.7, 0.7, 1.0)
    w, u, T = mixture_params()
    f = mixture(mesh.v, w, u, T)
    t0 = time.time()
    q = op.collide_cell(f, with_loss=True)
    print(f"c5_n64: oracle Q in {time.time() - t0:.0f} s")
    np.savez_compressed(
        os.path.join(HERE, "c5_n64.npz"),
        params=np.array([64, L10_S, 48, 70, 0.7, 0.7, 1.0]),
        w=w, u=u, T=T, f_sum=np.array(f.sum()), f_max=np.array(f.max()),
        q=q,
    )


if __name__ == "__main__":
    make_c5()
