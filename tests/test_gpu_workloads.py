"""The remaining benchmark configurations as GPU parity cases (mixed precision vs FP64).

* ensemble: 64 independent homogeneous problems, n in {16, 24, 32, 48},
  e ~ U[0.2, 1], 2-4 Maxwellian mixtures, one CUDA graph per PFE macro-step;
* stiff telescopic: TPI3 at kn = 1e-4, periodic, rho = 1 + 0.2 sin(2 pi x),
  T = 1 + 0.1 cos(2 pi x), n = 32, 32 x 32, 512 cells for one macro-step
  against FP64 (the state error against its measured bound, mass to 1e-10),
  and one homogeneous cell stepped to the end time t = 0.05 in both
  precisions;
* large grid: n = 64, L = 10, e = 0.7, 48 radial nodes x the 70-point design
  (no 64-point symmetric design exists), 3-component mixtures; against the
  oracle's fixture (tests/golden/c5_n64.npz) and the FP64 path.
Tolerance: 1e-5 relative L-inf against the FP64 GPU path unless stated.
"""
import math

import numpy as np
import pytest

from conftest import L8_S, maxwellian, op_config, rel_linf

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _pkg():
    import proj_int_inelastic_gb300 as pkg

    return pkg


def _mixture(v, rng, k, mean_box, t_range):
    f = sum(maxwellian(v, rng.uniform(0.5, 1.5), rng.uniform(-mean_box, mean_box, 3), rng.uniform(*t_range))
            for _ in range(k))
    dv = (v[1] - v[0]) ** 3
    return f / (f.sum() * dv)


def test_ensemble_uneven_sizes_graph_vs_fp64():
    pkg = _pkg()
    rng = np.random.default_rng(2026)
    sizes = [16, 24, 32, 48]
    configs, f0s = [], []
    for i in range(64):
        n = sizes[i % 4]
        e = float(rng.uniform(0.2, 1.0))
        cfg = op_config(n, L8_S, n // 2, 32, e, e, 1.0)
        sm = pkg.SpectralMesh(cfg)
        configs.append(cfg)
        f0s.append(_mixture(sm.v_center, rng, int(rng.integers(2, 5)), 2.0, (0.5, 2.0)))
    kw = dict(dt=0.02, kn=1.0, integrator="PFE", inner_steps=[2], inner_dt=[0.005], with_loss=True)
    mixed = pkg.Ensemble(configs, f0s, precision="mixed", **kw)
    eager = pkg.Ensemble(configs, f0s, precision="mixed", **kw)
    dbl = pkg.Ensemble(configs, f0s, precision="double", **kw)
    for _ in range(2):
        mixed.step()  # graph: captured on the first call, replayed on the second
        eager.step(use_graph=False)
        dbl.step(use_graph=False)
    torch.cuda.synchronize()
    for i in range(64):
        assert torch.equal(mixed.f[i], eager.f[i]), i
        assert rel_linf(mixed.f[i].cpu().numpy(), dbl.f[i].cpu().numpy()) < 1e-5, i
    for (r1, u1, T1), (r2, u2, T2) in zip(mixed.moments(), dbl.moments()):
        assert abs(T1 - T2) < 1e-5 * T2


# the stiff telescopic configuration: TPI3, kn = 1e-4, e = e0 = 0.9, periodic,
# rho = 1 + 0.2 sin(2 pi x), T = 1 + 0.1 cos(2 pi x).  Levels dt = (1e-5,
# 2.5e-5, 6.25e-5), K = 2 each, macro-step 2e-4: M = (0.5, 0.5, 1.2), advection
# CFL 0.79 at 512 cells, and an inner step inside the collision term's explicit
# bound (nu dt0 / kn <= 0.62).  The reference defaults (K = [3, 3, 3],
# dt_l = [kn, 5 kn, 10 kn]) give M_1 = -1 and an inner Euler step of kn,
# outside that bound: both FP64 and mixed runs diverge there.
C4_LEVELS = dict(inner_steps=[2, 2, 2], inner_dt=[1e-5, 2.5e-5, 6.25e-5], dt=2e-4)


def _c4_run(pkg, precision, nx, steps, f0=None, record=None):
    kn = 1e-4
    cfg = op_config(32, L8_S, 32, 32, 0.9, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    if f0 is None:
        x = (np.arange(nx) + 0.5) / nx
        f0 = np.stack([maxwellian(sm.v_center, 1 + 0.2 * math.sin(2 * math.pi * xi), (0, 0, 0),
                                  1 + 0.1 * math.cos(2 * math.pi * xi)) for xi in x])
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision=precision, with_loss=True, mass_fix=True, batch_max=nx)
    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": nx, "nv": 32})
    sol.state.f.copy_(torch.as_tensor(f0))
    solver = pkg.BoltzmannSolver1D(kn, collision_operator=col)
    solver.all_bcs = pkg.BC.periodic
    solver.time_integrator = "TPI3"
    solver.inner_steps = C4_LEVELS["inner_steps"]
    solver.inner_dt = C4_LEVELS["inner_dt"]
    solver.dt = C4_LEVELS["dt"]
    solver.check_every = 1  # FP64 NaN / Inf guard after every macro-step
    rho0, _, _ = sol.state.moments()
    for k in range(steps):
        solver.step(sol, False, k * solver.dt, (k + 1) * solver.dt)
        if record is not None:
            record.append((sol.f.clone(), sol.state.moments()))
    torch.cuda.synchronize()
    return sol.f.clone(), rho0


def test_c4_full_size_macro_step_mixed_vs_fp64():
    """512 cells, one macro-step (8 operator calls) in both precisions.  Near
    equilibrium Q = gain - loss cancels, so the FP32 rounding of each term
    (~1e-7 of |gain|) reaches f multiplied by dt / kn and the extrapolation
    factors: measured 6.9e-6 after one macro-step, growing by ~1.8e-5 per
    macro-step over the next two (2.8e-5, 5.5e-5), although every Q call is
    within 3e-6 of FP64.  Bound: 2e-5 after one macro-step."""
    pkg = _pkg()
    fm, rho0 = _c4_run(pkg, "mixed", 512, 1)
    fd, _ = _c4_run(pkg, "double", 512, 1)
    err = float((fm - fd).abs().max() / fd.abs().max())
    print(f"C4 512 cells: mixed vs FP64 rel Linf after 1 macro-step = {err:.3e}")
    assert err < 2e-5
    dv = (2 * 8.0 / 32) ** 3  # velocity cell volume of the 32^3 grid on [-8, 8]^3
    for f in (fm, fd):  # periodic transport + mass-fixed Q conserve the total mass
        assert abs(float(f.sum()) * dv / float(rho0.sum()) - 1) < 1e-10


def _tpi3_time_per_macro_step(K, h, dt):
    """Time one macro-step advances under the reference's telescopic
    recurrence (src/boltzmann.py:142-158): the level-l extrapolation adds
    M_l d_l with d_{l+1} = M_l d_l, i.e. M_l ... M_0 inner increments of h_0,
    so a macro-step advances K2 (K1 h1 + M1 M0 h0) + M2 M1 M0 h0 (h1 = (K0 + M0) h0)."""
    M0, M1, M2 = h[1] / h[0] - K[0], h[2] / h[1] - K[1], dt / h[2] - K[2]
    return K[2] * (K[1] * h[1] + M1 * M0 * h[0]) + M2 * M1 * M0 * h[0]


def test_c4_homogeneous_cell_full_horizon_mixed_vs_fp64():
    """The stiff configuration's cooling on one homogeneous cell (rho = T = 1),
    250 macro-steps to its nominal end time t = 0.05, in both precisions and
    next to forward Euler at a step that divides the macro-step's true advance.

    Measured: with these levels a macro-step advances 1.08e-4, not 2e-4 (the
    reference's recurrence extrapolates the last inner increment only).  The
    inelastic cooling takes T below ~0.15 by t ~ 0.003, where the 32^3 grid on
    [-8, 8]^3 no longer resolves f (f < 0 appears); without the mass fix the
    reference method then loses mass and blows up (NaN by t ~ 0.007 in forward
    Euler at dt = 2e-6 and 1e-5, 0.013 in TPI3), with the fix it spreads the
    mass defect uniformly over the box and heats the gas (T = 1.98 at the end
    in FP64 too), and that growth amplifies the rounding differences between
    the precisions (5e-3 by macro-step 100, 0.5 at the end).  Asserted: over
    the first 25 macro-steps (T >= 0.1) mixed agrees with FP64 to 1e-4 in f
    and 1e-2 in T, and the TPI3 temperature follows the fine explicit run's at
    the same time to 2e-2."""
    pkg = _pkg()
    cfg = op_config(32, L8_S, 32, 32, 0.9, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    f0 = maxwellian(sm.v_center, 1.0, (0, 0, 0), 1.0)[None]
    hist = {}
    for prec in ("mixed", "double"):
        rec = []
        _c4_run(pkg, prec, 1, 250, f0=f0, record=rec)
        hist[prec] = rec
    tau = _tpi3_time_per_macro_step(C4_LEVELS["inner_steps"], C4_LEVELS["inner_dt"], C4_LEVELS["dt"])
    assert abs(tau - 1.08e-4) < 1e-12
    # forward Euler (mixed, mass fix) at dt = tau / 54 = 2e-6, T after every tau
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", with_loss=True, mass_fix=True, batch_max=1)
    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": 1, "nv": 32})
    sol.state.f.copy_(torch.as_tensor(f0))
    eul = pkg.BoltzmannSolver1D(1e-4, collision_operator=col)
    eul.all_bcs = pkg.BC.periodic
    eul.time_integrator = "Euler"
    eul.dt = tau / 54
    resolved = 25
    T_euler = []
    for k in range(54 * resolved):
        eul.step(sol, False, k * eul.dt, (k + 1) * eul.dt)
        if (k + 1) % 54 == 0:
            T_euler.append(float(sol.state.moments()[2][0]))
    errs, dT = [], []
    for (fm, (_, _, Tm)), (fd, (_, _, Td)) in zip(hist["mixed"], hist["double"]):
        errs.append(float((fm - fd).abs().max() / fd.abs().max()))
        dT.append(float(abs(Tm[0] / Td[0] - 1)))
    Td = [float(m[2][0]) for _, m in hist["double"]]
    print("C4 homogeneous cell: macro-step, time, T (TPI3 FP64), T (Euler), mixed-vs-FP64 rel Linf of f, of T")
    for k in list(range(0, 250, 25)) + [249]:
        te = f"{T_euler[k]:.5f}" if k < resolved else "   -   "
        print(f"  {k + 1:4d} t={(k + 1) * tau:.5f} T={Td[k]:.5f} T_euler={te} err={errs[k]:.3e} dT={dT[k]:.3e}")
    assert max(errs[:resolved]) < 1e-4
    assert max(dT[:resolved]) < 1e-2
    assert max(abs(Td[k] / T_euler[k] - 1) for k in range(resolved)) < 2e-2


def _mixture_from(v, w, u, T):
    """The seeded mixture of tests/golden/make_oracle_fixtures.py, rebuilt from its parameters."""
    V = np.meshgrid(v, v, v, indexing="ij")
    f = 0.0
    for wi, ui, Ti in zip(w, u, T):
        d2 = (V[0] - ui[0]) ** 2 + (V[1] - ui[1]) ** 2 + (V[2] - ui[2]) ** 2
        f = f + wi / (2 * math.pi * Ti) ** 1.5 * np.exp(-d2 / (2 * Ti))
    return f / (f.sum() * (v[1] - v[0]) ** 3)


def test_large_grid_n64_full_quadrature_vs_oracle_fixture(golden):
    """The large-grid configuration at its full quadrature (n = 64, L = 10,
    48 radial nodes x the 70-point design, e = e0 = 0.7, hard spheres) against
    the oracle's Q on one seeded 3-Maxwellian cell: the FP64 path to 1e-12 and
    the mixed path with both first-axis column transforms (CUDA-core FFT and
    tensor-core split-FP16 DFT) to 1e-5."""
    pkg = _pkg()
    d = golden("c5_n64.npz")
    n, s, nr, ns, e, e0, g = (float(x) for x in d["params"])
    cfg = op_config(int(n), s, int(nr), int(ns), e, e0, g)
    sm = pkg.SpectralMesh(cfg)
    assert abs(sm.L - 10.0) < 1e-12
    f = _mixture_from(sm.v_center, d["w"], d["u"], d["T"])
    assert abs(f.sum() - float(d["f_sum"])) < 1e-12 * float(d["f_sum"])
    assert abs(f.max() - float(d["f_max"])) < 1e-12 * float(d["f_max"])
    ref = d["q"][None]
    ft = torch.as_tensor(f[None], device="cuda:0")
    qd = pkg.FSInelasticVHSCollision(cfg, sm, precision="double").collide(ft, with_loss=True)
    err = rel_linf(qd.cpu().numpy(), ref)
    print(f"n=64 full quadrature, FP64 path vs oracle: rel Linf {err:.3e}")
    assert err < 1e-12
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed")
    for gain, path in (("fused", None), ("packed", "fft"), ("packed", "tensor")):
        col.plan.set_tuning(gain, 6, 131072, dft_path=path)
        qm = col.collide(ft, with_loss=True)
        err = rel_linf(qm.cpu().numpy(), ref)
        print(f"n=64 full quadrature, mixed path ({gain}, {path} columns) vs oracle: rel Linf {err:.3e}")
        assert err < 1e-5, (gain, path)
    assert not col.plan.dft_stalled


def test_large_grid_n64_full_quadrature():
    pkg = _pkg()
    s = 20.0 / (3.0 + math.sqrt(2.0))  # L = 10
    cfg = op_config(64, s, 48, 70, 0.7, 0.7, 1.0)
    sm = pkg.SpectralMesh(cfg)
    assert abs(sm.L - 10.0) < 1e-12
    rng = np.random.default_rng(5)
    f = np.stack([_mixture(sm.v_center, rng, 3, 3.0, (0.5, 3.0)) for _ in range(2)])
    f = torch.as_tensor(f, device="cuda:0")
    qm = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=2).collide(f, with_loss=True)
    qd = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", batch_max=2).collide(f, with_loss=True)
    for c in range(2):
        assert rel_linf(qm[c].cpu().numpy(), qd[c].cpu().numpy()) < 1e-5, c


def test_large_grid_n64_tensor_core_dft():
    """The first-axis column transforms of the n = 64 pipeline on the tensor
    cores (split-FP16 DFT, FP32 accumulation) against the FP64 path, next to
    the CUDA-core FFT path; the full 48 x 70 quadrature on two cells."""
    pkg = _pkg()
    s = 20.0 / (3.0 + math.sqrt(2.0))  # L = 10
    cfg = op_config(64, s, 48, 70, 0.7, 0.7, 1.0)
    sm = pkg.SpectralMesh(cfg)
    rng = np.random.default_rng(11)
    f = np.stack([_mixture(sm.v_center, rng, 3, 3.0, (0.5, 3.0)) for _ in range(2)])
    f = torch.as_tensor(f, device="cuda:0")
    qd = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", batch_max=2).collide(f, with_loss=True)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=2)
    col.plan.set_tuning("packed", 6, 131072, dft_path="fft")
    qf = col.collide(f, with_loss=True)
    col.plan.set_dft_path("tensor")
    assert col.plan.tuning["dft_path"] == "tensor"
    qt = col.collide(f, with_loss=True)
    assert not col.plan.dft_stalled
    for c in range(2):
        et = rel_linf(qt[c].cpu().numpy(), qd[c].cpu().numpy())
        ef = rel_linf(qf[c].cpu().numpy(), qd[c].cpu().numpy())
        print(f"n=64 cell {c}: rel Linf vs FP64: tensor-core DFT {et:.3e}, CUDA-core FFT {ef:.3e}")
        assert et < 1e-5, c
    # mass defect of Q relative to the mass of f: no worse than the FFT path's
    dv = sm.delta**3
    mass = f.sum(dim=(1, 2, 3)) * dv
    mt = float((qt.sum(dim=(1, 2, 3)) * dv / mass).abs().max())
    mf = float((qf.sum(dim=(1, 2, 3)) * dv / mass).abs().max())
    print(f"n=64 mass defect: tensor-core {mt:.3e}, CUDA-core {mf:.3e}")
    assert mt < max(1e-6, 2 * mf)


def test_tensor_core_dft_path_rules():
    """The tensor-core DFT exists for n = 64 FP32 3D plans only; other plans
    refuse it with ValueError."""
    pkg = _pkg()
    cfg = op_config(32, L8_S, 8, 12, 0.9, 0.9, 1.0)
    col = pkg.FSInelasticVHSCollision(cfg, pkg.SpectralMesh(cfg), precision="mixed", batch_max=1)
    with pytest.raises(ValueError):
        col.plan.set_dft_path("tensor")
    assert col.plan.tuning["dft_path"] == "fft"


def test_tensor_core_dft_ragged_chunks():
    """Tensor-core column passes on ragged chunks: 3 cells with 2 cells per
    chunk (chunk_points = 2 x 64^3) and 24 pairs split 19 + 5, so items of one
    launch span two cells and the last chunk holds one cell; against the
    CUDA-core FFT columns and the FP64 path."""
    pkg = _pkg()
    s = 20.0 / (3.0 + math.sqrt(2.0))
    cfg = op_config(64, s, 4, 6, 0.6, 0.8, 1.0)
    sm = pkg.SpectralMesh(cfg)
    rng = np.random.default_rng(3)
    f = torch.as_tensor(np.stack([_mixture(sm.v_center, rng, 2, 2.0, (0.6, 2.0)) for _ in range(3)]),
                        device="cuda:0")
    qd = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", batch_max=3).collide(f, with_loss=True)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=3)
    out = {}
    for path in ("fft", "tensor"):
        col.plan.set_tuning("pipeline", 6, 2 * 64**3, dft_path=path)
        out[path] = col.collide(f, with_loss=True)
    assert not col.plan.dft_stalled
    for c in range(3):
        et = rel_linf(out["tensor"][c].cpu().numpy(), qd[c].cpu().numpy())
        ef = rel_linf(out["fft"][c].cpu().numpy(), qd[c].cpu().numpy())
        etf = rel_linf(out["tensor"][c].cpu().numpy(), out["fft"][c].cpu().numpy())
        print(f"ragged n=64 cell {c}: tensor {et:.3e}, fft {ef:.3e}, tensor vs fft {etf:.3e}")
    for c in range(3):
        assert rel_linf(out["tensor"][c].cpu().numpy(), qd[c].cpu().numpy()) < 1e-5, c
