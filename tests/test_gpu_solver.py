"""GPU parity of the transport step and the Euler / PFE / TPI2 / TPI3 integrators."""
import math

import numpy as np
import pytest

from conftest import L8_S, maxwellian, op_config, rel_linf

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _pkg():
    import proj_int_inelastic_gb300 as pkg

    return pkg


def test_transport_golden(golden):
    pkg = _pkg()
    d = golden("transport.npz")
    v = d["v"]
    for bc, code in (("extrap", pkg.BC.extrap), ("periodic", pkg.BC.periodic)):
        solver = pkg.BoltzmannSolver1D(1.0)
        solver.all_bcs = code
        sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": 8.0, "nx": 12, "nv": 8})
        sol.state.f.copy_(torch.as_tensor(d[f"{bc}_f"]))
        assert abs(sol.state.delta[0] - float(d[f"{bc}_dx"])) < 1e-15
        assert np.array_equal(sol.state.v, v)
        for j in range(2):
            df = solver.df_advection(sol.state, float(d[f"{bc}_dt{j}"]))
            assert rel_linf(df.cpu().numpy(), d[f"{bc}_df{j}"]) < 1e-12, (bc, j)


RUNS = [("pfe", "PFE", "extrap"), ("pfe_full", "PFE", "extrap"), ("tpi2", "TPI2", "periodic"),
        ("tpi3", "TPI3", "periodic"), ("euler", "Euler", "extrap")]


@pytest.mark.parametrize("use_graph", [False, True])
@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("name,integ,bc", RUNS)
def test_solver1d_golden(golden, name, integ, bc, precision, use_graph):
    pkg = _pkg()
    d = golden("solver1d.npz")
    nv, nr, ns, e, e0, g, s, nx = d["params"]
    cfg = op_config(nv, s, nr, ns, e, e0, g)
    sm = pkg.SpectralMesh(cfg)
    with_loss = name.endswith("_full") or name == "tpi3"
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision=precision, with_loss=with_loss)
    dt, tend, kn, dx = d[f"{name}_meta"]
    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": int(nx), "nv": int(nv)})
    sol.state.f.copy_(torch.as_tensor(d[f"{name}_f0"]))
    solver = pkg.BoltzmannSolver1D(float(kn), collision_operator=col)
    solver.all_bcs = pkg.BC.extrap if bc == "extrap" else pkg.BC.periodic
    solver.time_integrator = integ
    solver.inner_steps = [int(k) for k in d[f"{name}_K"]]
    solver.inner_dt = [float(h) for h in d[f"{name}_h"]]
    solver.dt = float(dt)
    solver.use_graph = use_graph
    solver.evolve_to_time(sol, float(tend))
    torch.cuda.synchronize()
    tol = 1e-11 if precision == "double" else 1e-5
    assert rel_linf(sol.f.cpu().numpy(), d[f"{name}_f"]) < tol
    assert abs(sol.t - float(tend)) < 1e-12


def test_generic_collision_callable_path(golden):
    """A plain callable as collision_operator steps through the Python nesting."""
    pkg = _pkg()
    d = golden("solver1d.npz")
    nv, nr, ns, e, e0, g, s, nx = d["params"]
    cfg = op_config(nv, s, nr, ns, e, e0, g)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="double")
    dt, tend, kn, dx = d["tpi3_meta"]
    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": int(nx), "nv": int(nv)})
    sol.state.f.copy_(torch.as_tensor(d["tpi3_f0"]))
    solver = pkg.BoltzmannSolver1D(float(kn), collision_operator=lambda f: col.collide(f, with_loss=True))
    solver.all_bcs = pkg.BC.periodic
    solver.time_integrator = "TPI3"
    solver.inner_steps = [int(k) for k in d["tpi3_K"]]
    solver.inner_dt = [float(h) for h in d["tpi3_h"]]
    solver.dt = float(dt)
    solver.evolve_to_time(sol, float(tend))
    assert rel_linf(sol.f.cpu().numpy(), d["tpi3_f"]) < 1e-11


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_euler_c32_temperature_history(golden, precision):
    """100 forward-Euler steps of the homogeneous two-beam problem (n = 32, 32 x 32
    quadrature, e = 0.9, hard spheres): T(t) and final f against the reference."""
    pkg = _pkg()
    c = golden("op_c32.npz")
    d = golden("euler_c32.npz")
    nv, nr, ns, e, e0, g, s = c["params"]
    cfg = op_config(nv, s, nr, ns, e, e0, g)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision=precision, with_loss=True)
    sol = pkg.Solution({"dim_x": 0, "dim_v": 3, "l": sm.L, "nv": 32})
    sol.state.f.copy_(torch.as_tensor(c["f"]))
    solver = pkg.BoltzmannSolver0D(1.0, collision_operator=col)
    solver.dt = float(d["dt"])
    T = [float(sol.state.T)]
    for _ in range(int(d["nsteps"])):
        solver.evolve_to_time(sol)  # one step
        T.append(float(sol.state.T))
    T = np.array(T)
    tol = 1e-11 if precision == "double" else 1e-5
    assert np.abs(T - d["T"]).max() / d["T"].max() < tol
    assert rel_linf(sol.f.cpu().numpy(), d["f_final"]) < (1e-10 if precision == "double" else 1e-5)


def test_moments_vs_oracle():
    pkg = _pkg()
    from oracle import integrators as it

    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": 8.0, "nx": 3, "nv": 16})
    v = sol.state.v
    f = np.stack([maxwellian(v, r, u, T) for r, u, T in ((1, (0, 0, 0), 1), (0.5, (1, -1, 0.5), 2), (2, (0, 2, 0), 0.7))])
    sol.state.f.copy_(torch.as_tensor(f))
    rho, u, T = sol.state.moments()
    ref = it.moments(f, v, sol.state.dv)
    assert np.abs(rho - ref["rho"]).max() < 1e-13
    assert np.abs(u - ref["u"]).max() < 1e-12
    assert np.abs(T - ref["T"]).max() < 1e-12


def test_pfe_c2_full_size_mass_and_parity():
    """The 1D Riemann workload at full size (128 cells x 32^3, e = 0.8, kn = 1e-2,
    PFE K = 2): one macro-step in mixed precision vs FP64 on the GPU, and mass
    conservation of the mass-fixed operator with outflow data (cells far from the
    boundary)."""
    pkg = _pkg()
    cfg = op_config(32, L8_S, 32, 32, 0.8, 0.8, 1.0)
    sm = pkg.SpectralMesh(cfg)
    nx = 128
    x = (np.arange(nx) + 0.5) / nx
    v = sm.v_center
    left, right = maxwellian(v, 1.0, (0, 0, 0), 1.0), maxwellian(v, 0.125, (0, 0, 0), 0.8)
    f0 = torch.as_tensor(np.stack([left if xi < 0.5 else right for xi in x]), device="cuda:0")
    out = {}
    for prec in ("mixed", "double"):
        col = pkg.FSInelasticVHSCollision(cfg, sm, precision=prec, with_loss=True, mass_fix=True, batch_max=nx)
        sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": nx, "nv": 32})
        sol.state.f.copy_(f0)
        solver = pkg.BoltzmannSolver1D(1e-2, collision_operator=col)
        solver.all_bcs = pkg.BC.extrap
        solver.time_integrator = "PFE"
        solver.inner_steps = [2]
        h = 4.0e-4  # CFL 0.5 bound: 0.5 dx / v_max
        solver.inner_dt = [h]
        solver.dt = 4 * h
        rho0 = sol.state.rho
        solver.evolve_to_time(sol, 4 * h)
        out[prec] = (sol.f.clone(), rho0, sol.state.rho)
    fm, fd = out["mixed"][0], out["double"][0]
    assert float((fm - fd).abs().max() / fd.abs().max()) < 1e-5
    rho0, rho1 = out["mixed"][1], out["mixed"][2]
    # total mass changes only by the boundary fluxes; interior cells far from x = 0.5 keep rho
    assert abs(rho1[:20].mean() - rho0[:20].mean()) / rho0[:20].mean() < 1e-6


@pytest.mark.parametrize("use_graph", [False, True])
@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_consp_golden(golden, precision, use_graph):
    """Convex splitting (src/boltzmann.py:86-94) against the reference run."""
    pkg = _pkg()
    d = golden("solver1d.npz")
    nv, nr, ns, e, e0, g, s, nx = d["params"]
    cfg = op_config(nv, s, nr, ns, e, e0, g)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision=precision, with_loss=True)
    dt, tend, kn, dx = d["consp_meta"]
    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": int(nx), "nv": int(nv)})
    sol.state.f.copy_(torch.as_tensor(d["consp_f0"]))
    solver = pkg.BoltzmannSolver1D(float(kn), collision_operator=col)
    solver.all_bcs = pkg.BC.periodic
    solver.time_integrator = "CONSP"
    solver.penalty = 5.0
    solver.dt = float(dt)
    solver.use_graph = use_graph
    solver.evolve_to_time(sol, float(tend))
    tol = 1e-11 if precision == "double" else 1e-5
    assert rel_linf(sol.f.cpu().numpy(), d["consp_f"]) < tol


def test_consp_maxwellian_3d_vs_oracle():
    """CONSP_M in its 3D-velocity form against the oracle restatement."""
    pkg = _pkg()
    from oracle import fs_inelastic as fo
    from oracle import integrators as it
    from oracle import transport as tr

    nv, nr, ns, e = 8, 4, 6, 0.6
    cfg = op_config(nv, L8_S, nr, ns, e, e, 0.0)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", with_loss=True)
    nx = 6
    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": nx, "nv": nv})
    v = sol.state.v
    f0 = np.stack([maxwellian(v, 1 + 0.1 * i, (0.3 * i - 0.5, 0.2, 0.0), 1 + 0.05 * i) for i in range(nx)])
    sol.state.f.copy_(torch.as_tensor(f0))
    solver = pkg.BoltzmannSolver1D(0.5, collision_operator=col)
    solver.all_bcs = pkg.BC.extrap
    solver.time_integrator = "CONSP_M"
    solver.penalty, solver.e, solver.tau, solver.dt = 3.0, e, 0.05, 1e-3
    solver.evolve_to_time(sol, 3e-3)
    m = fo.Mesh(nv, L8_S, nr, ns)
    op = fo.FSInelasticVHS(m, e, e, 0.0)
    f = f0.copy()
    dx = 1.0 / nx
    for _ in range(3):
        it.convex_splitting_maxwellian_step(f, 1e-3, lambda x: op.collide(x, with_loss=True), 0.5, 3.0, e, 0.05,
                                            m.v, m.delta, lambda x, h: tr.df_advection(x, m.v, h, dx))
    assert rel_linf(sol.f.cpu().numpy(), f) < 1e-11


def test_state_guard_detects_nonfinite_and_mass_drift():
    """Failures injected on the host: a NaN written into f, and a mass change."""
    pkg = _pkg()
    cfg = op_config(8, L8_S, 4, 6, 0.9, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", with_loss=True, mass_fix=True)
    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": 4, "nv": 8})
    v = sol.state.v
    sol.state.f.copy_(torch.as_tensor(np.stack([maxwellian(v, 1.0, (0, 0, 0), 1.0)] * 4)))
    solver = pkg.BoltzmannSolver1D(1.0, collision_operator=col)
    solver.all_bcs = pkg.BC.periodic
    solver.time_integrator = "PFE"
    solver.inner_steps, solver.inner_dt, solver.dt = [2], [1e-3], 4e-3
    solver.check_every, solver.mass_drift_tol = 1, 1e-9
    solver.evolve_to_time(sol, 8e-3)  # healthy: periodic transport + mass-fixed collisions conserve mass
    rho, u, T = solver.check_state(sol.state)
    assert np.all(np.isfinite(T))
    sol.state.f[2, 3, 4, 5] += 1.0  # host-side injection: mass changes
    with pytest.raises(RuntimeError, match="mass drifted"):
        solver.check_state(sol.state)
    sol.state.f[1, 0, 0, 0] = float("nan")  # host-side injection: a NaN
    with pytest.raises(FloatingPointError):
        solver.check_state(sol.state)
    # the library and the plan stay usable after the guard fired
    sol.state.f.copy_(torch.as_tensor(np.stack([maxwellian(v, 1.0, (0, 0, 0), 1.0)] * 4)))
    solver._mass0 = None
    solver.evolve_to_time(sol, sol.t + 4e-3)
    assert torch.isfinite(sol.f).all()


@pytest.mark.parametrize("name,integ,method", [("pfe", "PFE", "proj_euler_step"), ("tpi2", "TPI2", "tel_proj_step2"),
                                               ("euler", "Euler", "euler_step")])
def test_per_integrator_methods_fused(golden, name, integ, method):
    """The reference's per-integrator methods (src/boltzmann.py:82-158) on the
    GB300 operator: one call of e.g. ``proj_euler_step`` is the macro-step
    ``step`` runs for that ``time_integrator`` (the same native call), and
    matches the reference's run over its time span."""
    pkg = _pkg()
    d = golden("solver1d.npz")
    nv, nr, ns, e, e0, g, s, nx = d["params"]
    cfg = op_config(nv, s, nr, ns, e, e0, g)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="double")
    dt, tend, kn, dx = d[f"{name}_meta"]
    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": int(nx), "nv": int(nv)})
    sol.state.f.copy_(torch.as_tensor(d[f"{name}_f0"]))
    solver = pkg.BoltzmannSolver1D(float(kn), collision_operator=col)
    solver.all_bcs = pkg.BC.extrap if name != "tpi2" else pkg.BC.periodic
    solver.time_integrator = "Euler" if integ != "Euler" else "PFE"  # the method runs its own integrator
    solver.inner_steps = [int(k) for k in d[f"{name}_K"]]
    solver.inner_dt = [float(h) for h in d[f"{name}_h"]]
    solver.dt = float(dt)
    solver.setup(sol)
    steps = int(round((float(tend)) / float(dt)))
    for _ in range(steps):
        getattr(solver, method)(sol, False, 0.0, float(tend))
    torch.cuda.synchronize()
    assert rel_linf(sol.f.cpu().numpy(), d[f"{name}_f"]) < 1e-11


def test_state_helpers_and_grid():
    """State / Solution helpers of the reference (src/state.py:31-120,
    src/solution.py:36-46, src/geometry.py): grid attributes, sum_f against the
    FP64 moments, get_f_global and deepcopy as copies, ghost-array copies."""
    import copy

    pkg = _pkg()
    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": 8.0, "nx": 4, "nv": 8})
    st = sol.state
    assert sol.grid is st.grid and st.num_dim == 4 and st.num_dim_x == 1 and sol.num_cells == [4, 8, 8, 8]
    _, vx, vy, vz = st.c_centers
    f0 = np.exp(-((vx - 0.3) ** 2 + vy**2 + vz**2) / 2.0) * (1.0 + st.c_centers[0])
    st.f.copy_(torch.as_tensor(f0))
    rho = st.sum_f(st.f)
    assert isinstance(rho, torch.Tensor) and rho.shape == (4,)
    assert np.abs(rho.cpu().numpy() - st.rho).max() < 1e-12 * np.abs(st.rho).max()
    assert np.allclose(st.sum_f(f0), st.rho, rtol=1e-12, atol=0)
    g = st.get_f_global()
    g += 1.0
    assert torch.equal(st.f, torch.as_tensor(f0, device=st.f.device))
    st2 = copy.deepcopy(st)
    st2.f += 1.0
    assert torch.equal(st.f, torch.as_tensor(f0, device=st.f.device)) and st2.grid is not st.grid
    fbc = torch.zeros((8, 8, 8, 8), dtype=torch.float64, device=st.f.device)
    st.get_fbc_from_f(2, fbc)
    assert torch.equal(fbc[2:-2], st.f) and float(fbc[:2].abs().max()) == 0.0
    st.set_f_from_fbc(2, fbc)
    assert torch.equal(st.f, fbc[2:-2])
    sol.set_all_states("t", 0.25)
    assert sol.t == 0.25 and st.t == 0.25
    assert st.new_array().shape == (4, 8, 8, 8)
