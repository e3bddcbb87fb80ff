"""Generate the golden fixtures by running the reference solver itself.

The reference (Mayuyu/proj-int-inelastic) ships no tests, fixtures or golden
vectors, so parity is pinned by executing its own code under the shims in
``ref_shim.py`` on seeded inputs and storing inputs + outputs here:

* ``op_small.npz``   -- ``FSInelasticVHSCollision`` (``__call__`` = gain only,
  ``collide(with_loss=True)``, heat-bath Laplacian) at n = 8 / 16 for several
  (e, e0, gamma, n_r, n_sigma), batched over cells;
* ``op_c32.npz``     -- the same operator at n = 32, n_r = n_sigma = 32,
  e = e0 = 0.9, hard spheres, on the normalised two-beam Maxwellian;
* ``euler_c32.npz``  -- 100 forward-Euler steps of that problem (dt = 0.01):
  density / temperature history and the final f;
* ``transport.npz``  -- ``BoltzmannSolver1D.df_advection`` increments
  (extrapolation and periodic ghost cells);
* ``solver1d.npz``   -- short PFE / TPI2 / TPI3 runs of ``BoltzmannSolver1D``
  (reference default collision call = gain only, plus a gain - loss run).
* ``op2d.npz``       -- the 2D-velocity operator (``J_0`` kernel, circle
  quadrature) at n = 8 / 16 / 32: gain, gain - loss, heat bath;
* ``solver2d.npz``   -- ``BoltzmannSolver1D`` on 2D velocity (its native
  setting): PFE, Euler and CONSP_M runs (the convex splitting with the
  Maxwellian penalty exists only in 2D in the reference);
* ``sweep2d.npz``    -- ``BoltzmannFastSweep`` iterations (state after each
  step and the returned errors).

Run from the repository root:  ``python tests/golden/make_golden.py [stem ...]``
(all fixtures, or only the named ones; the full set reproduces the committed
files, the transport fixture drawing from the same generator after op_small).
Needs the reference checkout: set ``PII_REFERENCE_ROOT`` to it (required, no
default); GPU test runs never execute this script.
"""
import math
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from ref_shim import load_reference  # noqa: E402

L8_S = 16.0 / (3.0 + math.sqrt(2.0))  # s such that L = 8


def op_config(nv, s, nr, nsphr, e, e0, gamma):
    return {
        "velocity-mesh": {"nv": nv, "s": s, "nr": nr},
        "spherical-design-rule": {"ssrule": "womersley", "nsphr": nsphr},
        "collision-model": {"dim": 3, "type": "vhs", "e": e, "e0": e0, "gamma": gamma},
    }


def maxwellian(v, rho, u, T):
    V = np.meshgrid(v, v, v, indexing="ij")
    d2 = (V[0] - u[0]) ** 2 + (V[1] - u[1]) ** 2 + (V[2] - u[2]) ** 2
    return rho / (2 * math.pi * T) ** 1.5 * np.exp(-d2 / (2 * T))


def two_beam(v, delta):
    f = 0.5 * (maxwellian(v, 1.0, (2.0, 0.0, 0.0), 1.0) + maxwellian(v, 1.0, (-2.0, 0.0, 0.0), 1.0))
    return f / (f.sum() * delta**3)


def moments(f, v, delta):
    V = np.meshgrid(v, v, v, indexing="ij")
    dv = delta**3
    rho = f.sum(axis=(-3, -2, -1)) * dv
    mom = np.stack([(f * V[d]).sum(axis=(-3, -2, -1)) * dv for d in range(3)], -1)
    E = 0.5 * (f * (V[0] ** 2 + V[1] ** 2 + V[2] ** 2)).sum(axis=(-3, -2, -1)) * dv
    u = mom / rho[..., None]
    T = (2.0 / 3.0) * (E / rho - 0.5 * (u**2).sum(-1))
    return rho, u, T


OP_CASES = [
    # nv, nr, nsphr, e, e0, gamma, cells
    (8, 4, 6, 0.9, 0.9, 1.0, 3),
    (8, 3, 12, 0.5, 1.0, 0.0, 2),
    (16, 8, 12, 0.8, 0.8, 1.0, 2),
    (16, 5, 32, 0.2, 0.7, 0.0, 1),
]


def make_op_small(ref, rng):
    out = {}
    for i, (nv, nr, ns, e, e0, g, cells) in enumerate(OP_CASES):
        cfg = op_config(nv, L8_S, nr, ns, e, e0, g)
        sm = ref.spectral_mesh.SpectralMesh(cfg)
        col = ref.inelastic.FSInelasticVHSCollision(cfg, sm)
        f = rng.random((cells, nv, nv, nv)) + 0.1
        out[f"case{i}_params"] = np.array([nv, nr, ns, e, e0, g, L8_S])
        out[f"case{i}_f"] = f
        out[f"case{i}_gain"] = col(f)
        out[f"case{i}_full"] = col.collide(f, with_loss=True)
        out[f"case{i}_heat"] = col(f, heat_bath=0.3)
        # single-cell (no leading batch axis) call
        out[f"case{i}_gain_cell0"] = col(f[0])
    np.savez_compressed(os.path.join(HERE, "op_small.npz"), **out)


def make_op_c32(ref):
    cfg = op_config(32, L8_S, 32, 32, 0.9, 0.9, 1.0)
    sm = ref.spectral_mesh.SpectralMesh(cfg)
    col = ref.inelastic.FSInelasticVHSCollision(cfg, sm)
    f = two_beam(sm.v_center, sm.delta)
    gain = col(f)
    full = col.collide(f, with_loss=True)
    np.savez_compressed(os.path.join(HERE, "op_c32.npz"), params=np.array([32, 32, 32, 0.9, 0.9, 1.0, L8_S]),
                        f=f, gain=gain, full=full)
    return cfg, sm, col, f


def make_euler_c32(ref, cfg, sm, col, f0):
    f = f0.copy()
    dt, nsteps = 0.01, 100
    hist = [moments(f, sm.v_center, sm.delta)]
    col(f)  # build
    for _ in range(nsteps):
        f += dt * col.collide(f, with_loss=True)  # homogeneous Euler step, kn = 1 (src/boltzmann.py:82-84,160-164)
        hist.append(moments(f, sm.v_center, sm.delta))
    rho = np.array([h[0] for h in hist])
    T = np.array([h[2] for h in hist])
    np.savez_compressed(os.path.join(HERE, "euler_c32.npz"), dt=dt, nsteps=nsteps, rho=rho, T=T, f_final=f)


def _solution(ref, nx, nv, L, xmin=0.0, xmax=1.0):
    Solution = __import__("src.solution", fromlist=["Solution"]).Solution
    cfg = types.SimpleNamespace(dim_x=1, dim_v=3, xmin=xmin, xmax=xmax, l=L, nx=nx, nv=nv)
    return Solution(cfg)


def sod_f0(v, nx):
    x = (np.arange(nx) + 0.5) / nx
    f = np.empty((nx, len(v), len(v), len(v)))
    left = maxwellian(v, 1.0, (0.0, 0.0, 0.0), 1.0)
    right = maxwellian(v, 0.125, (0.0, 0.0, 0.0), 0.8)
    for i in range(nx):
        f[i] = left if x[i] < 0.5 else right
    return f


def periodic_f0(v, nx):
    x = (np.arange(nx) + 0.5) / nx
    return np.stack([maxwellian(v, 1 + 0.2 * math.sin(2 * math.pi * xi), (0.0, 0.0, 0.0),
                                1 + 0.1 * math.cos(2 * math.pi * xi)) for xi in x])


def make_transport(ref, rng):
    out = {}
    nx, nv = 12, 8
    L = 8.0
    for bcname, bc in (("extrap", ref.solver.BC.extrap), ("periodic", ref.solver.BC.periodic)):
        sol = _solution(ref, nx, nv, L)
        f = rng.random((nx, nv, nv, nv))
        f[3] = f[4]  # a zero wave, exercises the masked limiter ratio
        sol.state.f[:] = f
        solver = ref.boltzmann.BoltzmannSolver1D(1.0, riemann_solver=ref.advection_1D.advection_1D,
                                                 collision_operator=None)
        solver.all_bcs = bc
        solver.setup(sol)
        for j, dt in enumerate((1e-3, 4e-3)):
            out[f"{bcname}_f"] = f
            out[f"{bcname}_dt{j}"] = dt
            out[f"{bcname}_df{j}"] = solver.df_advection(sol.state, dt)
        out[f"{bcname}_dx"] = sol.state.grid.delta[0]
        out["v"] = sol.state.grid.dimensions[1].centers
    np.savez_compressed(os.path.join(HERE, "transport.npz"), **out)


def make_solver1d(ref):
    out = {}
    nv, nr, ns, nx = 8, 4, 6, 16
    kn = 1e-2
    cfg = op_config(nv, L8_S, nr, ns, 0.8, 0.8, 1.0)
    sm = ref.spectral_mesh.SpectralMesh(cfg)
    col = ref.inelastic.FSInelasticVHSCollision(cfg, sm)
    runs = [
        # name, integrator, bc, f0, inner_steps, inner_dt, dt, tend, collision
        ("pfe", "PFE", ref.solver.BC.extrap, "sod", [2], [1e-3], 4e-3, 8e-3, "gain"),
        ("pfe_full", "PFE", ref.solver.BC.extrap, "sod", [2], [1e-3], 4e-3, 8e-3, "full"),
        ("tpi2", "TPI2", ref.solver.BC.periodic, "per", [2, 2], [5e-4, 2e-3], 6e-3, 6e-3, "gain"),
        ("tpi3", "TPI3", ref.solver.BC.periodic, "per", [2, 2, 2], [2e-4, 6e-4, 2e-3], 6e-3, 1.2e-2, "full"),
        ("euler", "Euler", ref.solver.BC.extrap, "sod", [3], [1e-3], 5e-4, 2e-3, "gain"),
        ("consp", "CONSP", ref.solver.BC.periodic, "per", [3], [1e-3], 1e-3, 3e-3, "full"),
    ]
    for name, integ, bc, init, K, h, dt, tend, which in runs:
        sol = _solution(ref, nx, nv, sm.L)
        v = sol.state.grid.dimensions[1].centers
        f0 = sod_f0(v, nx) if init == "sod" else periodic_f0(v, nx)
        sol.state.f[:] = f0
        if which == "gain":
            operator = col
        else:
            def operator(f, _c=col):
                _c(f)
                return _c.collide(f, with_loss=True)
        solver = ref.boltzmann.BoltzmannSolver1D(kn, riemann_solver=ref.advection_1D.advection_1D,
                                                 collision_operator=operator)
        solver.all_bcs = bc
        solver.time_integrator = integ
        solver.inner_steps = list(K)
        solver.inner_dt = list(h)
        solver.dt = dt
        solver.penalty = 5.0
        solver.evolve_to_time(sol, tend)
        out[f"{name}_f0"] = f0
        out[f"{name}_f"] = sol.state.f.copy()
        out[f"{name}_meta"] = np.array([dt, tend, kn, sol.state.grid.delta[0]])
        out[f"{name}_K"] = np.array(K)
        out[f"{name}_h"] = np.array(h)
    out["params"] = np.array([nv, nr, ns, 0.8, 0.8, 1.0, L8_S, nx])
    np.savez_compressed(os.path.join(HERE, "solver1d.npz"), **out)


def op_config_2d(nv, s, nr, nphi, e, e0, gamma):
    return {
        "velocity-mesh": {"nv": nv, "s": s, "nr": nr},
        "circle-quad-rule": {"nphi": nphi},
        "collision-model": {"dim": 2, "type": "vhs", "e": e, "e0": e0, "gamma": gamma},
    }


def maxwellian_2d(v, rho, u, T):
    V = np.meshgrid(v, v, indexing="ij")
    return rho / (2 * math.pi * T) * np.exp(-((V[0] - u[0]) ** 2 + (V[1] - u[1]) ** 2) / (2 * T))


OP2D_CASES = [
    # nv, nr, nphi, e, e0, gamma, cells
    (8, 4, 8, 0.9, 0.9, 0.0, 3),
    (16, 8, 16, 0.5, 1.0, 1.0, 2),
    (16, 5, 12, 0.7, 0.7, 0.0, 2),
    (32, 16, 16, 0.8, 0.8, 1.0, 2),
]


def make_op2d(ref, rng):
    out = {}
    for i, (nv, nr, nphi, e, e0, g, cells) in enumerate(OP2D_CASES):
        cfg = op_config_2d(nv, L8_S, nr, nphi, e, e0, g)
        sm = ref.spectral_mesh.SpectralMesh(cfg)
        col = ref.inelastic.FSInelasticVHSCollision(cfg, sm)
        if i == 3:
            v = sm.v_center
            f = np.stack([maxwellian_2d(v, 1.0 + 0.1 * c, (0.5 * c, -0.3), 1.0 + 0.2 * c)
                          + 0.5 * maxwellian_2d(v, 1.0, (-1.5, 1.0), 0.7) for c in range(cells)])
        else:
            f = rng.random((cells, nv, nv)) + 0.1
        out[f"case{i}_params"] = np.array([nv, nr, nphi, e, e0, g, L8_S])
        out[f"case{i}_f"] = f
        out[f"case{i}_gain"] = col(f)
        out[f"case{i}_full"] = col.collide(f, with_loss=True)
        out[f"case{i}_heat"] = col(f, heat_bath=0.3)
    np.savez_compressed(os.path.join(HERE, "op2d.npz"), **out)


def _solution_2d(ref, nx, nv, L, xmin=0.0, xmax=1.0):
    Solution = __import__("src.solution", fromlist=["Solution"]).Solution
    cfg = types.SimpleNamespace(dim_x=1, dim_v=2, xmin=xmin, xmax=xmax, l=L, nx=nx, nv=nv)
    return Solution(cfg)


def sod_f0_2d(v, nx):
    x = (np.arange(nx) + 0.5) / nx
    left = maxwellian_2d(v, 1.0, (0.0, 0.0), 1.0)
    right = maxwellian_2d(v, 0.125, (0.0, 0.0), 0.8)
    return np.stack([left if xi < 0.5 else right for xi in x])


def periodic_f0_2d(v, nx):
    x = (np.arange(nx) + 0.5) / nx
    return np.stack([maxwellian_2d(v, 1 + 0.2 * math.sin(2 * math.pi * xi), (0.3 * math.cos(2 * math.pi * xi), 0.0),
                                   1 + 0.1 * math.cos(2 * math.pi * xi)) for xi in x])


def make_solver2d(ref):
    out = {}
    # n_x + 2 >= n_v: the reference's transport slices its speed array on the
    # velocity axis (src/boltzmann.py:200) and fails to broadcast otherwise
    nv, nr, nphi, nx = 16, 8, 16, 16
    kn, e, tau, penalty = 1e-2, 0.8, 0.05, 5.0
    cfg = op_config_2d(nv, L8_S, nr, nphi, e, e, 0.0)
    sm = ref.spectral_mesh.SpectralMesh(cfg)
    col = ref.inelastic.FSInelasticVHSCollision(cfg, sm)
    runs = [
        # name, integrator, bc, f0, inner_steps, inner_dt, dt, tend, collision
        ("pfe", "PFE", ref.solver.BC.extrap, "sod", [2], [5e-4], 2e-3, 4e-3, "full"),
        ("euler", "Euler", ref.solver.BC.periodic, "per", [3], [1e-3], 5e-4, 1.5e-3, "gain"),
        ("consp_m", "CONSP_M", ref.solver.BC.periodic, "per", [3], [1e-3], 1e-3, 3e-3, "full"),
    ]
    for name, integ, bc, init, K, h, dt, tend, which in runs:
        sol = _solution_2d(ref, nx, nv, sm.L)
        v = sol.state.grid.dimensions[1].centers
        f0 = sod_f0_2d(v, nx) if init == "sod" else periodic_f0_2d(v, nx)
        sol.state.f[:] = f0
        if which == "gain":
            operator = col
        else:
            def operator(f, _c=col):
                _c(f)
                return _c.collide(f, with_loss=True)
        solver = ref.boltzmann.BoltzmannSolver1D(kn, riemann_solver=ref.advection_1D.advection_1D,
                                                 collision_operator=operator)
        solver.all_bcs = bc
        solver.time_integrator = integ
        solver.inner_steps = list(K)
        solver.inner_dt = list(h)
        solver.dt = dt
        solver.penalty = penalty
        solver.e = e
        solver.tau = tau
        solver.evolve_to_time(sol, tend)
        out[f"{name}_f0"] = f0
        out[f"{name}_f"] = sol.state.f.copy()
        out[f"{name}_meta"] = np.array([dt, tend, kn, sol.state.grid.delta[0]])
        out[f"{name}_K"] = np.array(K)
        out[f"{name}_h"] = np.array(h)
    out["params"] = np.array([nv, nr, nphi, e, e, 0.0, L8_S, nx])
    out["consp_m_coeffs"] = np.array([penalty, e, tau])
    np.savez_compressed(os.path.join(HERE, "solver2d.npz"), **out)


def make_sweep2d(ref):
    import tempfile

    nv, nr, nphi, nx = 16, 8, 16, 10
    kn = 0.5
    cfg = op_config_2d(nv, L8_S, nr, nphi, 0.9, 0.9, 0.0)
    sm = ref.spectral_mesh.SpectralMesh(cfg)
    col = ref.inelastic.FSInelasticVHSCollision(cfg, sm)
    sol = _solution_2d(ref, nx, nv, sm.L)
    v = sol.state.grid.dimensions[1].centers
    f0 = periodic_f0_2d(v, nx)
    sol.state.f[:] = f0
    log = os.path.join(tempfile.mkdtemp(), "sweep.log")
    sweep = ref.iter_solver.BoltzmannFastSweep(log, collision=col, kn=kn, tol=1e-12)
    fs, errs = [], []
    for _ in range(3):
        errs.append(sweep.step(sol.state))
        fs.append(sol.state.f.copy())
    np.savez_compressed(os.path.join(HERE, "sweep2d.npz"), params=np.array([nv, nr, nphi, 0.9, 0.9, 0.0, L8_S, nx]),
                        kn=kn, dx=sol.state.grid.delta[0], v=v, f0=f0, f=np.stack(fs), err=np.array(errs))


def main(which=None):
    """Write every fixture, or only those named in ``which`` (file stems)."""
    ref = load_reference()
    want = set(which or ["op_small", "op_c32", "euler_c32", "transport", "solver1d", "op2d", "solver2d", "sweep2d"])
    rng = np.random.default_rng(20261203)
    if "op_small" in want:
        make_op_small(ref, rng)
    if want & {"op_c32", "euler_c32"}:
        cfg, sm, col, f = make_op_c32(ref)
        make_euler_c32(ref, cfg, sm, col, f)
    if "transport" in want:
        make_transport(ref, np.random.default_rng(1) if "op_small" not in want else rng)
    if "solver1d" in want:
        make_solver1d(ref)
    if "op2d" in want:
        make_op2d(ref, np.random.default_rng(20261204))
    if "solver2d" in want:
        make_solver2d(ref)
    if "sweep2d" in want:
        make_sweep2d(ref)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1:])
