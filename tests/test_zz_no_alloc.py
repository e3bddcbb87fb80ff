"""The allocation-free Q(f,f) entry point, against the oracle and the planned one.

pii_collide_noalloc serves callers that may not call cudaMalloc where they
need a collision evaluation: a host framework that hands out device memory
only through its own pool, a time loop with a fixed memory budget set at
start-up, or code that must not stall the device (cudaMalloc / cudaFree may
synchronise it).  Its tables and workspace sit in a static device array
inside the library, so it can only take small grids (n in {8, 16}, <= 8
cells, n_r * n_sigma <= 1024).  This file is collected last so that a
failure here never hides the results of the other tests; it also passes on
its own in a fresh process.
"""
import numpy as np
import pytest

from conftest import L8_S, maxwellian, op_config, rel_linf

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5  # the mixed-precision tolerance used by every FP32-path test


def _call_noalloc(lib, sm, f, q, e, e0, gamma, with_loss):
    from proj_int_inelastic_gb300 import _lib

    r, wr = (np.ascontiguousarray(a, np.float64) for a in sm.rquad())
    sig, wsig = sm.circ_or_sphr_quad()
    sig = np.ascontiguousarray(sig, np.float64)
    cells = f.numel() // sm.nv**3
    return lib.pii_collide_noalloc(f.data_ptr(), q.data_ptr(), cells, sm.nv, len(r), len(sig), _lib.dptr(r),
                                   _lib.dptr(wr), _lib.dptr(sig), float(wsig), float(sm.L), float(sm.R), float(e),
                                   float(e0), float(gamma), int(with_loss), torch.cuda.current_stream().cuda_stream)


# (n, n_r, n_sigma, cells): two small cases and the documented limit
# (n = 16 with 8 cells and n_r * n_sigma = 1024, where the chunk buffer is
# smallest and the pair loop splits into the most chunks)
CASES = [(16, 8, 12, 3), (8, 4, 6, 8), (16, 32, 32, 8)]


@pytest.mark.parametrize("nv,nr,ns,cells", CASES)
def test_noalloc_matches_oracle_and_planned_operator_twice(nv, nr, ns, cells):
    import proj_int_inelastic_gb300 as pkg
    from oracle import fs_inelastic as fo

    lib = pkg._lib.load()
    e, e0, g = 0.7, 0.9, 1.0
    cfg = op_config(nv, L8_S, nr, ns, e, e0, g)
    sm = pkg.SpectralMesh(cfg)
    planned = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=cells)
    oracle = fo.FSInelasticVHS(fo.Mesh(nv, L8_S, nr, ns), e, e0, g)
    v = sm.v_center
    rng = np.random.default_rng(7)
    inputs = []
    for k in range(2):  # two calls in a row, different data and cell counts
        cc = cells - k
        f = np.stack([maxwellian(v, 1.0 + 0.1 * c, (0.4 * c - 1, 0.2, -0.3 * k), 0.8 + 0.1 * c) for c in range(cc)])
        f *= 1 + 0.02 * rng.random(f.shape)
        inputs.append(f)
    for k, f in enumerate(inputs):
        with_loss = k == 0
        fd = torch.as_tensor(f, device="cuda:0")
        q = torch.full_like(fd, float("nan"))
        st = _call_noalloc(lib, sm, fd, q, e, e0, g, with_loss=with_loss)
        assert st == 0, pkg._lib.last_error()
        torch.cuda.synchronize()
        assert torch.isfinite(q).all()
        qh = q.cpu().numpy()
        ref = oracle.collide(f, with_loss=with_loss)
        assert rel_linf(qh, ref) < TOL, (k, rel_linf(qh, ref))
        mine = planned.collide(fd, with_loss=with_loss).cpu().numpy()
        assert rel_linf(qh, mine) < TOL, (k, rel_linf(qh, mine))


def test_noalloc_rejects_oversized_requests():
    import proj_int_inelastic_gb300 as pkg

    lib = pkg._lib.load()
    cfg = op_config(32, L8_S, 4, 6, 0.9, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    f = torch.zeros((1, 32, 32, 32), dtype=torch.float64, device="cuda:0")
    q = torch.empty_like(f)
    st = _call_noalloc(lib, sm, f, q, 0.9, 0.9, 1.0, True)
    assert st == pkg._lib.PII_ERR_SIZE
    assert "static-scratch limits" in pkg._lib.last_error()
    cfg = op_config(8, L8_S, 4, 6, 0.9, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    f = torch.zeros((9, 8, 8, 8), dtype=torch.float64, device="cuda:0")
    q = torch.empty_like(f)
    assert _call_noalloc(lib, sm, f, q, 0.9, 0.9, 1.0, True) == pkg._lib.PII_ERR_SIZE
