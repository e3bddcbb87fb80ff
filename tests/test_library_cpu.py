"""CPU-side checks of the C-ABI library and the host layer (no GPU compute)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import L8_S, ROOT, op_config

HEADER = os.path.join(ROOT, "include", "pii_gb300.h")


def _declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pii_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    import proj_int_inelastic_gb300 as pkg

    lib = pkg._lib.load()
    names = _declared()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    # the ctypes table binds exactly the declared entry points
    assert sorted(pkg._lib.SIGNATURES) == names


def test_library_is_in_tree_and_built_for_sm103a():
    import proj_int_inelastic_gb300 as pkg

    path = pkg._lib.LIB_PATH
    assert os.path.dirname(path).endswith("proj-int-inelastic_gb300")
    blob = open(path, "rb").read()
    assert b"sm_103a" in blob or b"sm_103" in blob


def test_version_and_error_paths_without_gpu():
    import proj_int_inelastic_gb300 as pkg

    lib = pkg._lib.load()
    assert lib.pii_version().startswith(b"pii_gb300")
    h = ctypes.c_void_p()
    r = np.zeros(4)
    st = lib.pii_plan_create(ctypes.byref(h), 20, 4, 6, pkg._lib.dptr(r), pkg._lib.dptr(r), pkg._lib.dptr(r), 1.0,
                             8.0, 7.0, 0.9, 0.9, 1.0, 0, 4, 0)
    assert st == pkg._lib.PII_ERR_ARG
    assert "n = 20" in pkg._lib.last_error()
    with pytest.raises(ValueError):
        pkg._lib.check(st, "pii_plan_create")
    assert lib.pii_plan_destroy(None) == pkg._lib.PII_ERR_ARG
    assert lib.pii_axpby(None, None, 1.0, 1.0, 4, None) == pkg._lib.PII_ERR_ARG
    # tuning entry points validate before touching a plan
    assert lib.pii_plan_set_dft_path(None, 1) == pkg._lib.PII_ERR_ARG
    assert "path must be 0" in pkg._lib.last_error()
    path, stalled = ctypes.c_int(-1), ctypes.c_int(-1)
    assert lib.pii_plan_get_dft_path(None, ctypes.byref(path), ctypes.byref(stalled)) == pkg._lib.PII_ERR_ARG
    assert lib.pii_plan_set_gain_path(None, 3) == pkg._lib.PII_ERR_ARG


def test_spectral_mesh_matches_oracle():
    import proj_int_inelastic_gb300 as pkg
    from oracle import fs_inelastic as fo

    for nv, nr, ns in ((32, 32, 32), (16, None, 12), (24, 12, 48)):
        cfg = op_config(nv, L8_S, nr if nr else nv // 2, ns, 0.9, 0.9, 1.0)
        if nr is None:
            del cfg["velocity-mesh"]["nr"]
        sm = pkg.SpectralMesh(cfg)
        m = fo.Mesh(nv, L8_S, nr, ns)
        assert sm.nr == m.nr
        assert np.array_equal(sm.v_center, m.v)
        assert np.array_equal(sm.rquad()[0], m.r) and np.array_equal(sm.rquad()[1], m.wr)
        assert np.array_equal(sm.circ_or_sphr_quad()[0], m.sigma)
        assert sm.circ_or_sphr_quad()[1] == m.wsigma
        assert abs(sm.L - 8.0) < 1e-12 and sm.delta == m.delta


def test_sphere_design_selection():
    import proj_int_inelastic_gb300 as pkg

    assert pkg.get_sphrquadrule("symmetric", "womersley", npts=32).shape == (32, 3)
    # smallest design of strength >= 8 is the 48-point strength-9 design
    assert pkg.get_sphrquadrule("symmetric", "womersley", qdeg=8).shape == (48, 3)
    with pytest.raises(ValueError):
        pkg.get_sphrquadrule("symmetric", "womersley", npts=64)  # no 64-point rule exists
    pts = np.eye(3)
    assert np.array_equal(pkg.get_sphrquadrule("symmetric", pts, npts=3), pts)


def test_config_errors():
    import proj_int_inelastic_gb300 as pkg

    cfg = op_config(16, L8_S, 8, 12, 0.9, 0.9, 1.0)
    cfg["collision-model"]["dim"] = 4
    with pytest.raises(ValueError):
        pkg.SpectralMesh(cfg)
    cfg["collision-model"]["dim"] = 2
    with pytest.raises(KeyError):  # 2D needs config["circle-quad-rule"] (src/collision/spectral_mesh.py:52)
        pkg.SpectralMesh(cfg)
    cfg = op_config(16, L8_S, 8, 12, 0.9, 0.9, 1.0)
    sm = pkg.SpectralMesh(cfg)
    with pytest.raises(ValueError):
        pkg.FSInelasticVHSCollision(cfg, sm, precision="half")
    col = pkg.FSInelasticVHSCollision(cfg, sm)
    assert col.precision == "mixed" and col.default_with_loss is False
    cfg2 = dict(cfg, config={"precision": "double"})
    assert pkg.FSInelasticVHSCollision(cfg2, sm).precision == "double"


def test_solver_host_logic():
    import proj_int_inelastic_gb300 as pkg

    s = pkg.BoltzmannSolver1D(1e-2)
    s.all_bcs = pkg.BC.periodic
    assert s.bc_lower == [pkg.BC.periodic] and s.bc_upper == [pkg.BC.periodic]
    assert s.inner_dt == [1e-2, 5e-2, 1e-1] and s.inner_steps == [3, 3, 3]
    s.time_integrator = "RK4"

    class _Sol:
        t = 0.0
        state = None

    with pytest.raises(NotImplementedError):
        s.step(_Sol(), False, 0, 1)
    s.dt = 0.3
    with pytest.raises(Exception, match="does not divide"):
        s._is_set_up = True
        s.evolve_to_time(_Sol(), 1.0)


def test_mesh_2d_matches_oracle():
    """2D-velocity mesh: circle quadrature and radial nodes as the reference's
    SpectralMesh (src/collision/spectral_mesh.py:51-56,94-97)."""
    import proj_int_inelastic_gb300 as pkg
    from oracle import fs_inelastic as fo

    cfg = {"velocity-mesh": {"nv": 32, "s": L8_S, "nr": 16}, "circle-quad-rule": {"nphi": 16},
           "collision-model": {"dim": 2, "type": "vhs", "e": 0.8, "gamma": 0.0}}
    sm = pkg.SpectralMesh(cfg)
    m = fo.Mesh(32, L8_S, 16, dim=2, nphi=16)
    sig, w = sm.circ_or_sphr_quad()
    assert sm.ndim == 2 and sm.ncirc_or_nsphr == 16 and sig.shape == (16, 2)
    assert np.array_equal(sig, m.sigma) and w == m.wsigma
    assert np.array_equal(sm.rquad()[0], m.r) and np.array_equal(sm.v_center, m.v)
    assert len(sm.v_centers) == 2 and sm.v_centers[0].shape == (32, 32)


def test_python_tuning_maps():
    """The Python tuning names map onto the C ABI's path codes."""
    import proj_int_inelastic_gb300 as pkg
    from proj_int_inelastic_gb300 import collision

    assert collision.GAIN_PATHS == {"pipeline": 0, "cluster": 1, "parity": 2, "packed": 3}
    assert collision.DFT_PATHS == {"fft": 0, "tensor": 1}
    assert set(pkg._lib.SIGNATURES) >= {"pii_plan_set_dft_path", "pii_plan_get_dft_path"}

