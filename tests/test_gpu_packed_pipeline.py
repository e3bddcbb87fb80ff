"""The packed passes (antipodal pairs + the Nyquist correction) against the oracle.

For every n other than 32 the FP32 plans of an antipodally symmetric design
evaluate each direction pair (sigma, -sigma) in one pass with a real phase,
in the fused cluster kernel (n = 16, 24, 48, 64) or the column / plane
pipeline, and add what the pass leaves out on the three Nyquist planes.  Checked against the oracle's Q
(src/collision/inelastic_collisions.py:208-227) on smooth and on rough input
(uniform random f: a full spectrum, where the Nyquist planes carry weight),
next to the unpacked pipeline, with an r-dependent restitution (e != e0).
"""
import numpy as np
import pytest

from conftest import L8_S, maxwellian, op_config, rel_linf

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5  # mixed precision against FP64
CASES = [(8, 4, 6), (16, 8, 12), (24, 4, 12), (48, 3, 6), (64, 2, 6)]


@pytest.mark.parametrize("gain", ["fused", "packed"])
@pytest.mark.parametrize("nyq", ["quadratic", "direct"])
@pytest.mark.parametrize("n,nr,ns", CASES)
def test_packed_pipeline_matches_oracle(n, nr, ns, nyq, gain):
    import proj_int_inelastic_gb300 as pkg
    from oracle import fs_inelastic as fo

    cfg = op_config(n, L8_S, nr, ns, 0.6, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    v = sm.v_center
    smooth = maxwellian(v, 1.0, (0.7, -0.4, 0.2), 1.1) + maxwellian(v, 0.6, (-1.2, 0.5, 0.3), 0.7)
    rough = np.random.default_rng(n).uniform(0.1, 1.0, (n, n, n)) * 0.05
    f = np.stack([smooth, rough])
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=2)
    # the defaults: the fused kernel at n = 16, 24, 48, else the packed pipeline
    assert col.plan.tuning["gain_path"] == ("packed" if n in (8, 64) else "fused")
    assert col.plan.nyquist_path == "quadratic"  # the default correction where its kernels fit
    if gain == "fused" and n == 8:
        pytest.skip("no fused kernel at n = 8")
    col.plan.set_tuning(gain, 6, 131072)
    col.plan.set_nyquist_path(nyq)
    assert col.plan.nyquist_path == nyq
    ft = torch.as_tensor(f, device="cuda:0")
    qp = col.collide(ft, with_loss=True).cpu().numpy()
    gp = col.collide(ft, with_loss=False).cpu().numpy()
    col.plan.set_tuning("pipeline", 6, 131072)
    qu = col.collide(ft, with_loss=True).cpu().numpy()
    op = fo.FSInelasticVHS(fo.Mesh(n, L8_S, nr, ns), 0.6, 0.9, 1.0)
    for c in range(2):
        ref = op.collide_cell(f[c], with_loss=True)
        refg = op.collide_cell(f[c], with_loss=False)
        ep, eu, eg = rel_linf(qp[c], ref), rel_linf(qu[c], ref), rel_linf(gp[c], refg)
        print(f"n={n} {gain} {nyq} cell {c}: packed {ep:.2e} (gain only {eg:.2e}), unpacked {eu:.2e}")
        assert ep < TOL and eg < TOL and eu < TOL, c


@pytest.mark.parametrize("nyq", ["quadratic", "direct"])
def test_packed_pipeline_per_cell_restitution_and_chunks(nyq):
    """Three cells with their own restitution laws and chunks of one cell
    (n = 16, 8 x 12 quadrature: 48 antipodal passes)."""
    import proj_int_inelastic_gb300 as pkg
    from oracle import fs_inelastic as fo

    cfg = op_config(16, L8_S, 8, 12, 0.9, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    rng = np.random.default_rng(5)
    f = rng.uniform(0.1, 1.0, (3, 16, 16, 16)) * 0.05
    sets = [(0.3, 0.3), (0.8, 1.0), (1.0, 1.0)]
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=3)
    col.plan.set_restitution([e for e, _ in sets], [e0 for _, e0 in sets])
    col.plan.set_tuning("packed", 6, 4096)  # one cell per chunk
    col.plan.set_nyquist_path(nyq)
    q = col.collide(torch.as_tensor(f, device="cuda:0"), with_loss=True).cpu().numpy()
    mesh = fo.Mesh(16, L8_S, 8, 12)
    for c, (e, e0) in enumerate(sets):
        ref = fo.FSInelasticVHS(mesh, e, e0, 1.0).collide_cell(f[c], with_loss=True)
        assert rel_linf(q[c], ref) < TOL, c


@pytest.mark.parametrize("n,nr,cells", [(32, 32, 37), (48, 6, 9)])
def test_quadratic_correction_many_cells(n, nr, cells):
    """Cell counts that split into several groups (the last one partial) and
    several input-point ranges: both Nyquist corrections against the FP64 plan."""
    import proj_int_inelastic_gb300 as pkg

    cfg = op_config(n, L8_S, nr, 32, 0.8, 0.8, 1.0)
    sm = pkg.SpectralMesh(cfg)
    v = sm.v_center
    rng = np.random.default_rng(cells)
    f = np.stack([maxwellian(v, 1.0, tuple(rng.uniform(-1, 1, 3)), rng.uniform(0.6, 1.4)) *
                  (1 + 0.05 * rng.random((n, n, n))) for _ in range(cells)])
    ft = torch.as_tensor(f, device="cuda:0")
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=cells)
    ref = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", batch_max=cells).collide(ft, with_loss=True)
    ref = ref.cpu().numpy()
    out = {}
    for nyq in ("direct", "quadratic"):
        col.plan.set_nyquist_path(nyq)
        out[nyq] = col.collide(ft, with_loss=True).cpu().numpy()
        for c in range(cells):
            assert rel_linf(out[nyq][c], ref[c]) < TOL, (nyq, c)
    assert rel_linf(out["quadratic"], out["direct"]) < 2e-6


@pytest.mark.parametrize("n", [16, 24, 48])
def test_fused_kernel_unpacked_design(n):
    """A direction set without antipodal pairs: the fused kernel runs every
    (r, sigma) pair unpacked, with no Nyquist correction; against the
    pipeline and the FP64 plan."""
    import proj_int_inelastic_gb300 as pkg

    rng = np.random.default_rng(n)
    pts = rng.standard_normal((7, 3))
    pts /= np.linalg.norm(pts, axis=1, keepdims=True)
    cfg = op_config(n, L8_S, 3, 7, 0.7, 0.9, 1.0)
    cfg["spherical-design-rule"]["points"] = pts
    sm = pkg.SpectralMesh(cfg)
    v = sm.v_center
    f = np.stack([maxwellian(v, 1.0, (0.5, -0.2, 0.1), 1.1), rng.uniform(0.1, 1.0, (n, n, n)) * 0.05])
    ft = torch.as_tensor(f, device="cuda:0")
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=2)
    assert col.plan.tuning["gain_path"] == "fused"
    qf = col.collide(ft, with_loss=True).cpu().numpy()
    col.plan.set_tuning("pipeline", 6, 131072)
    qp = col.collide(ft, with_loss=True).cpu().numpy()
    qd = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", batch_max=2).collide(ft, with_loss=True)
    qd = qd.cpu().numpy()
    for c in range(2):
        assert rel_linf(qf[c], qd[c]) < TOL and rel_linf(qp[c], qd[c]) < TOL, c


def test_fused_path_rules():
    """The fused kernel exists for FP32 3D plans of n = 16, 24, 48, 64; other
    plans refuse it with ValueError and keep their kernel choice."""
    import proj_int_inelastic_gb300 as pkg

    for n, precision in ((32, "mixed"), (8, "mixed"), (16, "double")):
        cfg = op_config(n, L8_S, 2, 6, 0.9, 0.9, 1.0)
        col = pkg.FSInelasticVHSCollision(cfg, pkg.SpectralMesh(cfg), precision=precision, batch_max=1)
        before = col.plan.tuning["gain_path"]
        with pytest.raises(ValueError):
            col.plan.set_tuning("fused", 6, 131072)
        assert col.plan.tuning["gain_path"] == before
    cfg = op_config(64, L8_S, 2, 6, 0.9, 0.9, 1.0)
    col = pkg.FSInelasticVHSCollision(cfg, pkg.SpectralMesh(cfg), precision="mixed", batch_max=2)
    assert col.plan.tuning["gain_path"] == "packed"  # the 64^3 default; the fused kernel on request
    col.plan.set_tuning("fused", 6, 131072)
    assert col.plan.tuning["gain_path"] == "fused"


@pytest.mark.parametrize("nyq", ["quadratic", "direct"])
@pytest.mark.parametrize("n,nr", [(48, 3), (64, 2)])
def test_fused_split_with_pipeline(n, nr, nyq):
    """The fused path with a share of the cells on the packed pipeline (side
    stream, on the SMs the fused kernel's clusters leave idle; the
    quadratic-form correction's partial sums on that stream too): every cell
    against the FP64 plan, and against the unsplit fused kernel."""
    import proj_int_inelastic_gb300 as pkg

    cfg = op_config(n, L8_S, nr, 6, 0.6, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    v = sm.v_center
    rng = np.random.default_rng(n + 1)
    f = np.stack([maxwellian(v, 1.0, rng.uniform(-1, 1, 3), rng.uniform(0.6, 1.4)) for _ in range(4)]
                 + [rng.uniform(0.1, 1.0, (n, n, n)) * 0.05])
    ft = torch.as_tensor(f, device="cuda:0")
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=5)
    col.plan.set_tuning("fused", 6, 65536)
    col.plan.set_nyquist_path(nyq)
    assert col.plan.tuning["fused_split"] == 0.0
    q0 = col.collide(ft, with_loss=True).cpu().numpy()
    col.plan.set_tuning("fused", 6, 65536, fused_split=0.4)  # the last 2 of 5 cells on the pipeline
    assert col.plan.tuning["fused_split"] == 0.4
    q1 = col.collide(ft, with_loss=True).cpu().numpy()
    qd = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", batch_max=5).collide(ft, with_loss=True)
    qd = qd.cpu().numpy()
    for c in range(5):
        assert rel_linf(q1[c], qd[c]) < TOL and rel_linf(q0[c], qd[c]) < TOL, c
        assert rel_linf(q1[c], q0[c]) < 2e-6, c
    with pytest.raises(ValueError):
        col.plan.set_fused_split(1.0)


def test_fused_split_in_captured_graph():
    """The split's fork onto the plan's side stream and join back are captured
    into the macro-step graph: graph replay and eager steps agree bit for bit,
    and with one restitution set per instance both match the FP64 ensemble."""
    import proj_int_inelastic_gb300 as pkg

    rng = np.random.default_rng(48)
    configs, f0s = [], []
    for i in range(4):
        cfg = op_config(48, L8_S, 3, 6, float(rng.uniform(0.3, 1.0)), 0.9, 1.0)
        v = pkg.SpectralMesh(cfg).v_center
        configs.append(cfg)
        f0s.append(maxwellian(v, 1.0, rng.uniform(-1, 1, 3), rng.uniform(0.7, 1.3)))
    kw = dict(dt=0.02, kn=1.0, integrator="PFE", inner_steps=[2], inner_dt=[0.005], with_loss=True)
    graph = pkg.Ensemble(configs, f0s, precision="mixed", **kw)
    eager = pkg.Ensemble(configs, f0s, precision="mixed", **kw)
    dbl = pkg.Ensemble(configs, f0s, precision="double", **kw)
    for ens in (graph, eager):
        for op, _, _ in ens._classes:
            op.plan.set_tuning("fused", 6, 65536, fused_split=0.25)  # the last instance on the pipeline
    for _ in range(2):
        graph.step()
        eager.step(use_graph=False)
        dbl.step(use_graph=False)
    torch.cuda.synchronize()
    for i in range(4):
        assert torch.equal(graph.f[i], eager.f[i]), i
        # one restitution set per instance, on both sides of the split
        assert rel_linf(graph.f[i].cpu().numpy(), dbl.f[i].cpu().numpy()) < 1e-5, i


@pytest.mark.parametrize("n,nr,ns", [(8, 4, 6), (16, 4, 12), (32, 3, 6), (48, 2, 6)])
def test_fp64_packed_pipeline(n, nr, ns):
    """FP64 plans on a symmetric design default to the packed pipeline with
    the FP64 quadratic-form Nyquist correction: against the unpacked FP64
    pipeline and the oracle at 1e-12, with one restitution set per cell."""
    import proj_int_inelastic_gb300 as pkg
    from oracle import fs_inelastic as fo

    cfg = op_config(n, L8_S, nr, ns, 0.6, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    v = sm.v_center
    rng = np.random.default_rng(n + 7)
    f = np.stack([maxwellian(v, 1.0, (0.7, -0.4, 0.2), 1.1) + maxwellian(v, 0.6, (-1.2, 0.5, 0.3), 0.7),
                  rng.uniform(0.1, 1.0, (n, n, n)) * 0.05])
    ft = torch.as_tensor(f, device="cuda:0")
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", batch_max=2)
    assert col.plan.tuning["gain_path"] == "packed"
    assert col.plan.nyquist_path == "quadratic"
    with pytest.raises(ValueError):
        col.plan.set_nyquist_path("direct")  # FP32 kernels only
    qp = col.collide(ft, with_loss=True).cpu().numpy()
    col.plan.set_tuning("pipeline", 6, 131072)
    qu = col.collide(ft, with_loss=True).cpu().numpy()
    op = fo.FSInelasticVHS(fo.Mesh(n, L8_S, nr, ns), 0.6, 0.9, 1.0)
    for c in range(2):
        ref = op.collide_cell(f[c], with_loss=True)
        assert rel_linf(qp[c], qu[c]) < 1e-12 and rel_linf(qp[c], ref) < 1e-12, c
    # one restitution set per cell: the correction's kernels are rebuilt per set
    es, e0s = [0.5, 0.95], [0.8, 0.7]
    col.plan.set_tuning("packed", 6, 131072)
    col.plan.set_restitution(es, e0s)
    qs = col.collide(ft, with_loss=True).cpu().numpy()
    for c in range(2):
        ref = fo.FSInelasticVHS(fo.Mesh(n, L8_S, nr, ns), es[c], e0s[c], 1.0).collide_cell(f[c], with_loss=True)
        assert rel_linf(qs[c], ref) < 1e-12, c
