"""Failure detection on the GPU without a GPU fault, and bounded host state.

* The tensor-core DFT kernel (n = 64, FP32) bounds every mbarrier wait.  The
  test hook makes its TMA thread withhold every copy, so the other roles wait
  on barriers that nothing completes and give up, with no copy or MMA in
  flight; the launch reports the stall through a mapped host word, the next
  call on the plan raises, and the plan works normally afterwards.
* The macro-step graph cache keeps at most 8 instantiated graphs per plan,
  however many distinct step arguments a caller uses.
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


def test_tensor_core_dft_stall_is_reported_and_recovers():
    pkg = _pkg()
    s = 20.0 / (3.0 + math.sqrt(2.0))  # L = 10
    cfg = op_config(64, s, 2, 6, 0.7, 0.7, 1.0)
    sm = pkg.SpectralMesh(cfg)
    f = torch.as_tensor(maxwellian(sm.v_center, 1.0, (0.5, -0.3, 0.2), 1.3)[None], device="cuda:0")
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=1)
    col.plan.set_tuning("packed", 6, 131072, dft_path="tensor")
    good = col.collide(f, with_loss=True).clone()
    assert not col.plan.dft_stalled
    # every copy withheld: the roles give up after 1024 polls each
    col.plan.dft_test_hooks(wait_limit=1024, withhold=True)
    col.collide(f, with_loss=True)  # enqueued; the stall surfaces on the next call
    torch.cuda.synchronize()
    assert col.plan.dft_stalled
    with pytest.raises(RuntimeError, match="gave up waiting"):
        col.collide(f, with_loss=True)
    assert not col.plan.dft_stalled  # reported once, then cleared
    col.plan.dft_test_hooks()  # defaults: copies issued, 2^22 polls
    again = col.collide(f, with_loss=True)
    torch.cuda.synchronize()
    assert not col.plan.dft_stalled
    assert rel_linf(again.cpu().numpy(), good.cpu().numpy()) < 1e-12


def test_fused_cluster_exchange_stall_is_reported_and_recovers():
    """The fused kernel's exchange waits (n = 48: 6-CTA clusters) give up when
    no CTA delivers its elements (withheld: no remote store and no expected
    byte count is issued, so nothing is in flight when the waits run out);
    the stall is reported once by the next call, and the plan then works."""
    pkg = _pkg()
    cfg = op_config(48, L8_S, 2, 6, 0.7, 0.7, 1.0)
    sm = pkg.SpectralMesh(cfg)
    f = torch.as_tensor(maxwellian(sm.v_center, 1.0, (0.5, -0.3, 0.2), 1.3)[None], device="cuda:0")
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=1)
    assert col.plan.tuning["gain_path"] == "fused"
    good = col.collide(f, with_loss=True).clone()
    assert not col.plan.dft_stalled
    col.plan.dft_test_hooks(wait_limit=1024, withhold=True)
    col.collide(f, with_loss=True)  # enqueued; the stall surfaces on the next call
    torch.cuda.synchronize()
    assert col.plan.dft_stalled
    with pytest.raises(RuntimeError, match="gave up waiting"):
        col.collide(f, with_loss=True)
    assert not col.plan.dft_stalled  # reported once, then cleared
    col.plan.dft_test_hooks()  # defaults: exchanges issued, 2^22 polls
    again = col.collide(f, with_loss=True)
    torch.cuda.synchronize()
    assert not col.plan.dft_stalled
    assert rel_linf(again.cpu().numpy(), good.cpu().numpy()) < 1e-12


def test_step_graph_cache_is_bounded():
    pkg = _pkg()
    cfg = op_config(8, L8_S, 4, 6, 0.9, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", with_loss=True, batch_max=4)
    v = sm.v_center
    f0 = np.stack([maxwellian(v, 1.0 + 0.1 * i, (0.2 * i, 0, 0), 1.0) for i in range(4)])
    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": 4, "nv": 8})
    sol.state.f.copy_(torch.as_tensor(f0))
    ref = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": 4, "nv": 8})
    ref.state.f.copy_(torch.as_tensor(f0))
    solvers = []
    for use_graph in (True, False):
        sv = pkg.BoltzmannSolver1D(1.0, collision_operator=col)
        sv.all_bcs = pkg.BC.periodic
        sv.time_integrator = "PFE"
        sv.inner_steps = [2]
        sv.use_graph = use_graph
        solvers.append(sv)
    for k in range(20):  # 20 distinct macro-step sizes: 20 distinct graph keys
        dt = 1e-3 * (1 + 0.05 * k)
        for sv, so in zip(solvers, (sol, ref)):
            sv.inner_dt = [dt / 4]
            sv.dt = dt
            sv.step(so, True, 0.0, dt)
        assert col.plan.graph_count <= 8
    torch.cuda.synchronize()
    assert col.plan.graph_count == 8
    # replayed graphs (with evictions along the way) give the eager result
    assert rel_linf(sol.state.f.cpu().numpy(), ref.state.f.cpu().numpy()) < 1e-13
