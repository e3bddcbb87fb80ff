"""GPU parity of the collision operator against the golden fixtures and the oracle.

Tolerances: <= 1e-12 relative L-inf for the FP64 GPU path, <= 1e-5 for the
mixed-precision (FP32 FFT / quadrature) path, both against FP64 references.
"""
import ctypes
import math

import numpy as np
import pytest

from conftest import L8_S, maxwellian, op_config, rel_linf

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {"double": 1e-12, "mixed": 1e-5}


def _pkg():
    import proj_int_inelastic_gb300 as pkg

    return pkg


def _op(params, precision, **kw):
    nv, nr, ns, e, e0, g, s = params
    cfg = op_config(nv, s, nr, ns, e, e0, g)
    pkg = _pkg()
    sm = pkg.SpectralMesh(cfg)
    return sm, pkg.FSInelasticVHSCollision(cfg, sm, precision=precision, **kw)


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("case", range(4))
def test_operator_small_golden(golden, case, precision):
    d = golden("op_small.npz")
    sm, col = _op(d[f"case{case}_params"], precision)
    f = d[f"case{case}_f"]
    tol = TOL[precision]
    assert rel_linf(col(f), d[f"case{case}_gain"]) < tol  # __call__ = gain only (reference default)
    assert rel_linf(col.collide(f, with_loss=True), d[f"case{case}_full"]) < tol
    assert rel_linf(col(f, heat_bath=0.3), d[f"case{case}_heat"]) < tol
    assert rel_linf(col(f[0]), d[f"case{case}_gain_cell0"]) < tol  # (n, n, n) input


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("nv", [16, 32])
def test_laplacian_vs_oracle(nv, precision):
    """``laplacian`` (src/collision/inelastic_collisions.py:229-230) through
    pii_laplacian against the oracle's FP64 spectral Laplacian: two cells,
    NumPy in / out and torch in / out."""
    from oracle import fs_inelastic as fo

    m = fo.Mesh(nv, L8_S, 4, 6)
    op = fo.FSInelasticVHS(m, 0.8, 0.8, 1.0)
    f = np.stack([maxwellian(m.v, 1.0, (0.5, -0.3, 0.2), 1.2), maxwellian(m.v, 0.7, (-1.0, 1.0, 0.0), 0.6)])
    ref = op.laplacian(f)
    sm, col = _op((nv, 4, 6, 0.8, 0.8, 1.0, L8_S), precision)
    assert rel_linf(col.laplacian(f), ref) < TOL[precision]
    ft = torch.as_tensor(f, device="cuda:0")
    lt = col.laplacian(ft)
    assert isinstance(lt, torch.Tensor) and lt.is_cuda and lt.shape == ft.shape
    assert rel_linf(lt.cpu().numpy(), ref) < TOL[precision]
    assert rel_linf(col.laplacian(f[1]), ref[1]) < TOL[precision]  # (n, n, n) input


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_conservation_and_dissipation(precision):
    """Moments of Q = Q+ - Q- on a two-beam state at n = 32: mass and momentum
    are conserved to spectral accuracy for any e, energy for e = 1, and e < 1
    dissipates energy.  (The oracle gives, as fractions of the scale
    sum |Q| (1 + |v|^2) dv: mass 2e-5, momentum 1.5e-5, energy 7e-5 at e = 1,
    and an energy moment of -0.17 at e = 0.8.)"""
    for e in (1.0, 0.8):
        sm, col = _op((32, 16, 32, e, e, 1.0, L8_S), precision)
        v = sm.v_center
        f = maxwellian(v, 1.0, (0.8, 0.0, 0.0), 0.8) + maxwellian(v, 1.0, (-0.8, 0.2, 0.0), 1.0)
        q = col.collide(f, with_loss=True)
        V = np.meshgrid(v, v, v, indexing="ij")
        dv = sm.delta**3
        v2 = V[0] ** 2 + V[1] ** 2 + V[2] ** 2
        scale = (np.abs(q) * (1 + v2)).sum() * dv
        mass = q.sum() * dv / scale
        mom = [(q * V[i]).sum() * dv / scale for i in range(3)]
        energy = (q * v2 / 2).sum() * dv / scale
        assert abs(mass) < 1e-4 and max(abs(x) for x in mom) < 1e-4, (e, mass, mom)
        if e == 1.0:
            assert abs(energy) < 2e-4, energy
        else:
            assert energy < -0.1, energy


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_operator_c32_two_beam_golden(golden, precision):
    d = golden("op_c32.npz")
    sm, col = _op(d["params"], precision)
    tol = TOL[precision]
    assert rel_linf(col.collide(d["f"], with_loss=True), d["full"]) < tol
    assert rel_linf(col.collide(d["f"]), d["gain"]) < tol


def test_torch_in_torch_out_and_input_untouched(golden):
    d = golden("op_small.npz")
    sm, col = _op(d["case2_params"], "mixed")
    f = torch.as_tensor(d["case2_f"], device="cuda:0")
    f0 = f.clone()
    q = col.collide(f, with_loss=True)
    assert isinstance(q, torch.Tensor) and q.is_cuda and q.dtype == torch.float64 and q.shape == f.shape
    assert torch.equal(f, f0)
    assert rel_linf(q.cpu().numpy(), d["case2_full"]) < 1e-5


@pytest.mark.parametrize("nv", [24, 48])
def test_radix3_sizes_vs_oracle(nv):
    """n = 24 / 48 (radix-3 stages) against the oracle, FP64 and mixed."""
    from oracle import fs_inelastic as fo

    nr, ns = (6, 6) if nv == 48 else (8, 12)
    m = fo.Mesh(nv, L8_S, nr, ns)
    op = fo.FSInelasticVHS(m, 0.6, 0.9, 1.0)
    f = maxwellian(m.v, 1.0, (0.5, -0.3, 0.2), 1.2) + 0.3 * maxwellian(m.v, 1.0, (-2, 1, 0), 0.6)
    ref = op.collide(f, with_loss=True)
    for prec in ("double", "mixed"):
        sm, col = _op((nv, nr, ns, 0.6, 0.9, 1.0, L8_S), prec)
        assert rel_linf(col.collide(f, with_loss=True), ref) < TOL[prec], prec


def test_n64_vs_oracle():
    from oracle import fs_inelastic as fo

    m = fo.Mesh(64, L8_S * 1.25, 4, 6)
    op = fo.FSInelasticVHS(m, 0.7, 0.7, 1.0)
    f = maxwellian(m.v, 1.0, (1.0, 0.0, -1.0), 1.5)
    ref = op.collide(f, with_loss=True)
    sm, col = _op((64, 4, 6, 0.7, 0.7, 1.0, L8_S * 1.25), "mixed")
    assert rel_linf(col.collide(f, with_loss=True), ref) < 1e-5


def test_full_size_properties_c2():
    """128 cells x 32^3 (the 1D Riemann workload): quadratic scaling Q(2f) = 4 Q(f),
    batch-order independence, single-cell equality, mixed vs FP64 agreement."""
    pkg = _pkg()
    cfg = op_config(32, L8_S, 32, 32, 0.8, 0.8, 1.0)
    sm = pkg.SpectralMesh(cfg)
    v = sm.v_center
    nx = 128
    x = (np.arange(nx) + 0.5) / nx
    left = maxwellian(v, 1.0, (0, 0, 0), 1.0)
    right = maxwellian(v, 0.125, (0, 0, 0), 0.8)
    f = torch.as_tensor(np.stack([left if xi < 0.5 else right for xi in x]), device="cuda:0")
    gen = torch.Generator(device="cuda:0").manual_seed(7)
    f += 1e-3 * torch.rand(f.shape, generator=gen, device="cuda:0", dtype=f.dtype) * f
    mixed = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=nx)
    dbl = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", batch_max=nx)
    q = mixed.collide(f, with_loss=True)
    q64 = dbl.collide(f, with_loss=True)
    err = (q - q64).abs().amax(dim=(1, 2, 3)) / q64.abs().amax(dim=(1, 2, 3))
    assert float(err.max()) < 1e-5
    q2 = mixed.collide(2 * f, with_loss=True)
    assert float((q2 - 4 * q).abs().max() / (4 * q).abs().max()) < 1e-6
    # batch order: the fused kernel splits the (cell, pair) work evenly over the
    # SMs, so a cell's FP32 partial sums are grouped by its batch position; each
    # grouping is an FP32 evaluation inside the mixed-precision tolerance
    # (measured 1.5e-6 of max |Q| on this near-equilibrium data)
    perm = torch.randperm(nx, device="cuda:0")
    qp = mixed.collide(f[perm].contiguous(), with_loss=True)
    assert float((qp - q[perm]).abs().max() / q.abs().max()) < 1e-5
    assert torch.equal(mixed.collide(f[perm].contiguous(), with_loss=True), qp)  # deterministic
    # one cell alone: other groupings of the FP32 partial sums (work split and
    # correction blocks), rounding only; near equilibrium Q is a small difference
    # of large gain and loss terms, so the bound is the mixed-precision one
    q7 = mixed.collide(f[7:8].contiguous(), with_loss=True)
    assert float((q7[0] - q[7]).abs().max() / q[7].abs().max()) < 1e-5


@pytest.mark.parametrize("path", ["cluster", "parity", "packed"])
@pytest.mark.parametrize("cells", [1, 3, 128])
def test_fused_kernel_matches_pipeline_and_fp64(cells, path):
    """n = 32 mixed precision: the fused gain kernels (2-CTA cluster, a-parity)
    against the column / plane pipeline and against the FP64 path, gain and
    gain - loss."""
    pkg = _pkg()
    cfg = op_config(32, L8_S, 32, 32, 0.7, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    v = sm.v_center
    rng = np.random.default_rng(cells)
    f = np.stack([maxwellian(v, 1.0 + 0.2 * rng.random(), rng.uniform(-2, 2, 3), rng.uniform(0.5, 2.0))
                  + 0.3 * maxwellian(v, 1.0, rng.uniform(-2, 2, 3), rng.uniform(0.5, 2.0)) for _ in range(cells)])
    f = torch.as_tensor(f, device="cuda:0")
    clus = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=cells, gain_path=path)
    pipe = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=cells, gain_path="pipeline")
    dbl = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", batch_max=cells)
    for wl in (False, True):
        qc, qp, qd = clus.collide(f, with_loss=wl), pipe.collide(f, with_loss=wl), dbl.collide(f, with_loss=wl)
        for c in range(cells):
            assert rel_linf(qc[c].cpu().numpy(), qd[c].cpu().numpy()) < 1e-5, (wl, c)
            assert rel_linf(qc[c].cpu().numpy(), qp[c].cpu().numpy()) < 1e-5, (wl, c)


@pytest.mark.parametrize("path", ["cluster", "parity", "packed", "packed-direct"])
def test_fused_kernel_rough_input(path):
    """Uniform random f (spectrum up to the Nyquist planes, where exp_rs f^ is
    not Hermitian): fused kernels against the FP64 path, with and without loss,
    with heat bath, and with pair ranges of every length; the packed kernel
    with both Nyquist corrections (the quadratic form, the default, and the
    direct kernel)."""
    pkg = _pkg()
    cfg = op_config(32, L8_S, 3, 12, 0.5, 0.8, 1.0)
    sm = pkg.SpectralMesh(cfg)
    f = torch.as_tensor(np.random.default_rng(11).random((5, 32, 32, 32)), device="cuda:0")
    fused = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=5, gain_path=path.split("-")[0])
    if path == "packed-direct":
        fused.plan.set_nyquist_path("direct")
    dbl = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", batch_max=5)
    for wl in (False, True):
        qf, qd = fused.collide(f, with_loss=wl), dbl.collide(f, with_loss=wl)
        assert rel_linf(qf.cpu().numpy(), qd.cpu().numpy()) < 1e-5, wl
    qf, qd = fused(f, heat_bath=0.2), dbl(f, heat_bath=0.2)
    assert rel_linf(np.asarray(qf.cpu()), np.asarray(qd.cpu())) < 1e-5


def test_autotuner_keeps_results():
    """pii_plan_autotune picks a kernel configuration; results stay within tolerance."""
    pkg = _pkg()
    cfg = op_config(32, L8_S, 16, 32, 0.8, 0.8, 1.0)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=8)
    best, choice = col.plan.autotune(8)
    assert best > 0 and choice["gain_path"] in ("packed", "parity", "cluster", "pipeline")
    assert choice["items_per_cluster"] in (2, 4, 6, 8)
    v = sm.v_center
    f = torch.as_tensor(np.stack([maxwellian(v, 1.0, (0.3 * c, 0, 0), 1.0) for c in range(8)]), device="cuda:0")
    ref = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", batch_max=8).collide(f, with_loss=True)
    q = col.collide(f, with_loss=True)
    for c in range(8):
        assert rel_linf(q[c].cpu().numpy(), ref[c].cpu().numpy()) < 1e-5


def test_mass_fix_conserves_mass_fp32():
    pkg = _pkg()
    cfg = op_config(32, L8_S, 32, 32, 0.9, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", mass_fix=True)
    f = 0.5 * (maxwellian(sm.v_center, 1, (2, 0, 0), 1) + maxwellian(sm.v_center, 1, (-2, 0, 0), 1))
    q = col.collide(f, with_loss=True)
    dv = sm.delta**3
    assert abs(q.sum() * dv) / (f.sum() * dv) < 1e-6
    # and the uncorrected operator, checked against the oracle's correction
    from oracle import fs_inelastic as fo

    raw = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed").collide(f, with_loss=True)
    assert rel_linf(q, fo.mass_mode_correction(raw)) < 1e-6


def test_cooling_law_gpu():
    """Maxwell molecules: -dT/dt / (rho T (1 - e^2)) = 1/4."""
    pkg = _pkg()
    for e in (0.9, 0.5):
        cfg = op_config(32, L8_S, 16, 32, e, e, 0.0)
        sm = pkg.SpectralMesh(cfg)
        col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed")
        v = sm.v_center
        f = maxwellian(v, 1.0, (0.0, 0.0, 0.0), 1.0)
        q = col.collide(f, with_loss=True)
        V = np.meshgrid(v, v, v, indexing="ij")
        dv = sm.delta**3
        rho = f.sum() * dv
        dE = 0.5 * (q * (V[0] ** 2 + V[1] ** 2 + V[2] ** 2)).sum() * dv
        E = 0.5 * (f * (V[0] ** 2 + V[1] ** 2 + V[2] ** 2)).sum() * dv
        T = (2 / 3) * E / rho
        drho = q.sum() * dv
        dT = (2 / 3) * (dE / rho - E * drho / rho**2)
        k = -dT / (rho * T * (1 - e**2))
        assert abs(k - 0.25) < 5e-3, (e, k)


def test_c_abi_errors_on_gpu():
    pkg = _pkg()
    lib = pkg._lib.load()
    sm, col = _op((8, 4, 6, 0.9, 0.9, 1.0, L8_S), "mixed", batch_max=2)
    plan = col.plan
    f = torch.zeros((3, 8, 8, 8), dtype=torch.float64, device="cuda:0")
    q = torch.empty_like(f)
    st = lib.pii_collide(plan.handle, f.data_ptr(), q.data_ptr(), 3, 1, 0.0, 0, None)
    assert st == pkg._lib.PII_ERR_SIZE
    st = lib.pii_collide(plan.handle, f.data_ptr(), f.data_ptr(), 1, 1, 0.0, 0, None)
    assert st == pkg._lib.PII_ERR_ARG
    v = np.ascontiguousarray(sm.v_center)
    st = lib.pii_transport_df(plan.handle, f.data_ptr(), q.data_ptr(), 2, 1e-3, 0.1, pkg._lib.dptr(v), 7, 1, None)
    assert st == pkg._lib.PII_ERR_ARG and "Boundary condition" in pkg._lib.last_error()
    # the plan keeps working after rejected calls
    st = lib.pii_collide(plan.handle, f.data_ptr(), q.data_ptr(), 2, 1, 0.0, 0, None)
    assert st == pkg._lib.PII_OK
    torch.cuda.synchronize()
    assert float(q[:2].abs().max()) == 0.0  # Q(0) = 0; cell 2 was not part of the call
