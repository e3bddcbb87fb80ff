"""The allocation-free Q(f,f) entry point against the planned one.

pii_collide_noalloc serves callers that cannot call cudaMalloc when they need
a collision evaluation (for instance while they record a CUDA graph, or when a
host framework owns all device memory): its tables and workspace sit in a
static device array inside the library.  This file is collected last so that a
failure here never hides the results of the other tests; it also passes on its
own in a fresh process.
"""
import ctypes

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


@pytest.mark.parametrize("nv,nr,ns,cells", [(16, 8, 12, 3), (8, 4, 6, 8)])
def test_noalloc_matches_planned_operator_twice(nv, nr, ns, cells):
    import proj_int_inelastic_gb300 as pkg

    lib = pkg._lib.load()
    e, e0, g = 0.7, 0.9, 1.0
    cfg = op_config(nv, L8_S, nr, ns, e, e0, g)
    sm = pkg.SpectralMesh(cfg)
    planned = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", batch_max=cells)
    v = sm.v_center
    rng = np.random.default_rng(7)
    inputs = []
    for k in range(2):  # two calls in a row, different data and cell counts
        cc = cells - k
        f = np.stack([maxwellian(v, 1.0 + 0.1 * c, (0.4 * c - 1, 0.2, -0.3 * k), 0.8 + 0.1 * c) for c in range(cc)])
        f *= 1 + 0.02 * rng.random(f.shape)
        inputs.append(torch.as_tensor(f, device="cuda:0"))
    for k, f in enumerate(inputs):
        q = torch.full_like(f, float("nan"))
        st = _call_noalloc(lib, sm, f, q, e, e0, g, with_loss=(k == 0))
        assert st == 0, pkg._lib.last_error()
        torch.cuda.synchronize()
        ref = planned.collide(f, with_loss=(k == 0))
        assert torch.isfinite(q).all()
        assert rel_linf(q.cpu().numpy(), ref.cpu().numpy()) < TOL, k


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
