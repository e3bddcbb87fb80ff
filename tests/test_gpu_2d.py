"""GPU parity of the 2D-velocity operator (J_0 kernel, circle quadrature), the
2D solver runs (PFE, Euler, CONSP_M) and the fast sweep, against fixtures made
by the reference itself (tests/golden/make_golden.py)."""
import math

import numpy as np
import pytest

from conftest import rel_linf

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _pkg():
    import proj_int_inelastic_gb300 as pkg

    return pkg


def config_2d(nv, s, nr, nphi, e, e0, gamma):
    return {
        "velocity-mesh": {"nv": int(nv), "s": float(s), "nr": int(nr)},
        "circle-quad-rule": {"nphi": int(nphi)},
        "collision-model": {"dim": 2, "type": "vhs", "e": float(e), "e0": float(e0), "gamma": float(gamma)},
    }


@pytest.mark.parametrize("precision,tol", [("double", 1e-12), ("mixed", 1e-5)])
@pytest.mark.parametrize("case", range(4))
def test_operator_2d_golden(golden, case, precision, tol):
    pkg = _pkg()
    d = golden("op2d.npz")
    nv, nr, nphi, e, e0, g, s = d[f"case{case}_params"]
    cfg = config_2d(nv, s, nr, nphi, e, e0, g)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision=precision)
    f = d[f"case{case}_f"]
    assert rel_linf(col(f), d[f"case{case}_gain"]) < tol  # numpy in -> numpy out, gain only
    assert rel_linf(col.collide(f, with_loss=True), d[f"case{case}_full"]) < tol
    assert rel_linf(col(f, heat_bath=0.3), d[f"case{case}_heat"]) < tol
    # a single cell without the batch axis, and torch in -> torch out
    q0 = col(torch.as_tensor(f[0], device="cuda:0"))
    assert isinstance(q0, torch.Tensor) and q0.shape == f[0].shape
    assert rel_linf(q0.cpu().numpy(), d[f"case{case}_gain"][0]) < tol


@pytest.mark.parametrize("precision,tol", [("double", 1e-12), ("mixed", 1e-5)])
def test_laplacian_2d_vs_oracle(precision, tol):
    """``laplacian`` (src/collision/inelastic_collisions.py:229-230) of a 2D
    plan through pii_laplacian against the oracle's FP64 spectral Laplacian."""
    from oracle import fs_inelastic as fo

    pkg = _pkg()
    nv, s = 32, 16.0 / (3.0 + math.sqrt(2.0))
    m = fo.Mesh(nv, s, 4, dim=2, nphi=8)
    op = fo.FSInelasticVHS(m, 0.8, 0.8, 0.0)
    x, y = np.meshgrid(m.v, m.v, indexing="ij")
    f = np.stack([np.exp(-((x - 0.5) ** 2 + y**2) / 2.0), 0.5 * np.exp(-(x**2 + (y + 1.0) ** 2) / 1.5)])
    ref = op.laplacian(f)
    cfg = config_2d(nv, s, 4, 8, 0.8, 0.8, 0.0)
    col = pkg.FSInelasticVHSCollision(cfg, pkg.SpectralMesh(cfg), precision=precision)
    assert rel_linf(col.laplacian(f), ref) < tol


def test_cooling_law_2d_maxwell_molecules():
    """-dT/dt = (1 - e^2) rho T / 4 in 2D as well (the law CONSP_M integrates,
    src/boltzmann.py:103-105), on the GPU FP64 path."""
    pkg = _pkg()
    s = 16.0 / (3 + math.sqrt(2))
    for e in (0.9, 0.5):
        cfg = config_2d(32, s, 16, 32, e, e, 0.0)
        sm = pkg.SpectralMesh(cfg)
        col = pkg.FSInelasticVHSCollision(cfg, sm, precision="double")
        V = np.meshgrid(sm.v_center, sm.v_center, indexing="ij")
        f = 1 / (2 * math.pi) * np.exp(-((V[0] - 0.3) ** 2 + V[1] ** 2) / 2)
        q = col.collide(f, with_loss=True)
        dv = sm.delta**2
        rho = f.sum() * dv
        E = 0.5 * (f * (V[0] ** 2 + V[1] ** 2)).sum() * dv
        u = np.array([(f * V[k]).sum() * dv / rho for k in range(2)])
        T = E / rho - 0.5 * (u**2).sum()
        dE = 0.5 * (q * (V[0] ** 2 + V[1] ** 2)).sum() * dv
        dmom = np.array([(q * V[k]).sum() * dv for k in range(2)])
        drho = q.sum() * dv
        dT = dE / rho - E * drho / rho**2 - (u * (dmom - u * drho)).sum() / rho
        assert abs(-dT / (rho * T * (1 - e**2)) - 0.25) < 5e-3, e


@pytest.mark.parametrize("use_graph", [False, True])
@pytest.mark.parametrize("precision,tol", [("double", 1e-11), ("mixed", 1e-5)])
@pytest.mark.parametrize("name", ["pfe", "euler", "consp_m"])
def test_solver2d_golden(golden, name, precision, tol, use_graph):
    pkg = _pkg()
    d = golden("solver2d.npz")
    nv, nr, nphi, e, e0, g, s, nx = d["params"]
    cfg = config_2d(nv, s, nr, nphi, e, e0, g)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision=precision, with_loss=(name != "euler"))
    dt, tend, kn, dx = d[f"{name}_meta"]
    sol = pkg.Solution({"dim_x": 1, "dim_v": 2, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": int(nx), "nv": int(nv)})
    assert abs(sol.state.delta[0] - dx) < 1e-15 and tuple(sol.f.shape) == (int(nx), int(nv), int(nv))
    sol.state.f.copy_(torch.as_tensor(d[f"{name}_f0"]))
    solver = pkg.BoltzmannSolver1D(float(kn), collision_operator=col)
    solver.all_bcs = pkg.BC.extrap if name == "pfe" else pkg.BC.periodic
    solver.time_integrator = {"pfe": "PFE", "euler": "Euler", "consp_m": "CONSP_M"}[name]
    solver.inner_steps = [int(k) for k in d[f"{name}_K"]]
    solver.inner_dt = [float(h) for h in d[f"{name}_h"]]
    solver.dt = float(dt)
    solver.penalty, solver.e, solver.tau = (float(x) for x in d["consp_m_coeffs"])
    solver.use_graph = use_graph
    solver.evolve_to_time(sol, float(tend))
    assert rel_linf(sol.f.cpu().numpy(), d[f"{name}_f"]) < tol


def test_moments_2d_match_reference_form():
    """State.rho / u / T in 2D (src/state.py:31-52): sums over the two velocity
    axes times delta^2, T = E / rho - |u|^2 / 2."""
    pkg = _pkg()
    from oracle import integrators as it

    sol = pkg.Solution({"dim_x": 1, "dim_v": 2, "xmin": 0.0, "xmax": 1.0, "l": 8.0, "nx": 5, "nv": 16})
    v = sol.state.v
    V = np.meshgrid(v, v, indexing="ij")
    f = np.stack([(1 + 0.1 * i) / (2 * math.pi * (1 + 0.2 * i)) *
                  np.exp(-((V[0] - 0.2 * i) ** 2 + (V[1] + 0.1) ** 2) / (2 * (1 + 0.2 * i))) for i in range(5)])
    sol.state.f.copy_(torch.as_tensor(f))
    rho, u, T = sol.state.moments()
    mo = it.moments(f, v, v[1] - v[0], dim=2)
    assert np.abs(rho - mo["rho"]).max() < 1e-13 and np.abs(u - mo["u"]).max() < 1e-13
    assert np.abs(T - mo["T"]).max() < 1e-13


def test_fast_sweep_2d_golden(golden):
    """Three BoltzmannFastSweep iterations (src/iter_solver.py:38-62) with the
    FP64 operator: states and returned errors as the reference's."""
    pkg = _pkg()
    d = golden("sweep2d.npz")
    nv, nr, nphi, e, e0, g, s, nx = d["params"]
    cfg = config_2d(nv, s, nr, nphi, e, e0, g)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="double")
    sol = pkg.Solution({"dim_x": 1, "dim_v": 2, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": int(nx), "nv": int(nv)})
    sol.state.f.copy_(torch.as_tensor(d["f0"]))
    sweep = pkg.BoltzmannFastSweep(None, collision=col, kn=float(d["kn"]), tol=1e-12)
    for k in range(3):
        err = sweep.step(sol.state)
        assert rel_linf(sol.f.cpu().numpy(), d["f"][k]) < 1e-12, k
        assert abs(err - d["err"][k]) <= 1e-12 * abs(d["err"][k]), k
    # solve(): iterate until the error is below tol or n_iter is reached
    err, steps = sweep.solve(sol, n_iter=4)
    assert steps == 4 and err > 0


def test_fast_sweep_3d_vs_oracle():
    """The sweep generalised to 3D velocity (every (v2, v3) swept the same way),
    against the oracle's restatement (FP64 collision term)."""
    pkg = _pkg()
    from conftest import L8_S, maxwellian, op_config
    from oracle import fs_inelastic as fo
    from oracle import integrators as it

    cfg = op_config(16, L8_S, 8, 12, 0.8, 0.8, 0.0)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", batch_max=8)
    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": 8, "nv": 16})
    v = sol.state.v
    f0 = np.stack([maxwellian(v, 1 + 0.1 * math.sin(i), (0.2, 0, 0), 1 + 0.05 * i) for i in range(8)])
    sol.state.f.copy_(torch.as_tensor(f0))
    m = fo.Mesh(16, L8_S, 8, 12)
    op = fo.FSInelasticVHS(m, 0.8, 0.8, 0.0)
    f = f0.copy()
    sweep = pkg.BoltzmannFastSweep(None, collision=col, kn=0.3)
    for _ in range(2):
        err_gpu = sweep.step(sol.state)
        err_cpu = it.fast_sweep_step(f, v, sol.state.delta[0], 0.3, op, m.delta, dim=3)
        assert rel_linf(sol.f.cpu().numpy(), f) < 1e-12
        assert abs(err_gpu - err_cpu) <= 1e-10 * err_cpu
