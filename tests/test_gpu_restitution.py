"""Per-cell restitution (one plan, one restitution law per cell) against the oracle.

An ensemble of homogeneous problems that share a velocity grid but not e runs
as one batched plan whose gain tables hold one set per cell
(pii_plan_set_restitution).  Each cell's Q must equal the operator built for
that cell's (e, e0) alone (src/collision/inelastic_collisions.py:30-52,77-103):
checked against the oracle for the pipeline (FP64 and mixed), the fused n = 32
packed kernel with its Nyquist correction, the fused cluster kernel of the
other sizes (the mixed default at n = 16, 24, 48, 64) and the n = 64
tensor-core column path.
"""
import math

import numpy as np
import pytest

from conftest import L8_S, maxwellian, op_config, rel_linf

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

E_SETS = [(0.3, 0.3), (0.85, 0.85), (0.6, 1.0)]  # the last one r-dependent: e(r) between 0.6 and 1


def _cells(v, k):
    rng = np.random.default_rng(17 + k)
    out = []
    for c in range(k):
        f = maxwellian(v, 1.0, rng.uniform(-1.5, 1.5, 3), rng.uniform(0.6, 1.4))
        f += maxwellian(v, 0.5, rng.uniform(-1.5, 1.5, 3), rng.uniform(0.6, 1.4))
        out.append(f)
    return np.stack(out)


CASES = [  # (n, s, n_r, n_sigma, precision, path, tolerance)
    (16, L8_S, 8, 12, "double", None, 1e-12),
    (16, L8_S, 8, 12, "mixed", None, 1e-5),
    (16, L8_S, 8, 12, "mixed", "packed", 1e-5),
    (48, L8_S, 3, 6, "mixed", "fused", 1e-5),
    (64, 20.0 / (3.0 + math.sqrt(2.0)), 4, 6, "mixed", "fused", 1e-5),
    (32, L8_S, 8, 32, "mixed", "packed", 1e-5),
    (32, L8_S, 8, 32, "mixed", "parity", 1e-5),
    (64, 20.0 / (3.0 + math.sqrt(2.0)), 4, 6, "mixed", "tensor", 1e-5),
]


@pytest.mark.parametrize("n,s,nr,ns,precision,path,tol", CASES)
def test_per_cell_restitution_matches_oracle(n, s, nr, ns, precision, path, tol):
    import proj_int_inelastic_gb300 as pkg
    from oracle import fs_inelastic as fo

    cfg = op_config(n, s, nr, ns, 0.9, 0.9, 1.0)  # the plan's own (e, e0): replaced per cell below
    sm = pkg.SpectralMesh(cfg)
    f = _cells(sm.v_center, len(E_SETS))
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision=precision, batch_max=len(E_SETS))
    if path == "tensor":
        col.plan.set_tuning("packed", 6, 131072, dft_path="tensor")
    elif path is not None:
        col.plan.set_tuning(path, 6, 131072)
    col.plan.set_restitution([e for e, _ in E_SETS], [e0 for _, e0 in E_SETS])
    q = col.collide(torch.as_tensor(f, device="cuda:0"), with_loss=True).cpu().numpy()
    mesh = fo.Mesh(n, s, nr, ns)
    for c, (e, e0) in enumerate(E_SETS):
        ref = fo.FSInelasticVHS(mesh, e, e0, 1.0).collide_cell(f[c], with_loss=True)
        err = rel_linf(q[c], ref)
        print(f"n={n} {precision} {path}: cell {c} (e={e}, e0={e0}) rel Linf vs oracle {err:.2e}")
        assert err < tol, c
    if path == "tensor":
        assert not col.plan.dft_stalled
    # more cells than restitution sets is an error; restoring one set takes any count again
    with pytest.raises(ValueError):
        col.collide(torch.as_tensor(np.concatenate([f, f[:1]]), device="cuda:0"), with_loss=True)
    col.plan.set_restitution([], [])
    q1 = col.collide(torch.as_tensor(f[:1], device="cuda:0"), with_loss=True).cpu().numpy()
    ref = fo.FSInelasticVHS(mesh, 0.9, 0.9, 1.0).collide_cell(f[0], with_loss=True)
    assert rel_linf(q1[0], ref) < tol


def test_per_cell_restitution_rejects_cluster_path_and_excess_sets():
    import proj_int_inelastic_gb300 as pkg

    cfg = op_config(32, L8_S, 4, 6, 0.9, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=2)
    col.plan.set_restitution([0.5, 0.7], [0.5, 0.7])
    with pytest.raises(ValueError):
        col.plan.set_tuning("cluster", 6, 131072)
    with pytest.raises(ValueError):
        col.plan.set_restitution([0.5, 0.6, 0.7], [0.5, 0.6, 0.7])  # beyond batch_max
