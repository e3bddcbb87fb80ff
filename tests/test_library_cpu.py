"""CPU-side checks of the C-ABI library and the host layer (no GPU compute)."""
import ctypes
import math
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

    r32 = pkg.get_sphrquadrule("symmetric", "womersley", npts=32)
    assert r32.pts.shape == (32, 3) and r32.wts.shape == (0,)
    # smallest design of strength >= 8 is the 48-point strength-9 design
    assert pkg.get_sphrquadrule("symmetric", "womersley", qdeg=8).pts.shape == (48, 3)
    with pytest.raises(ValueError):
        pkg.get_sphrquadrule("symmetric", "womersley", npts=64)  # no 64-point rule exists
    with pytest.raises(ValueError, match="Must specify"):
        pkg.get_sphrquadrule("symmetric", "womersley")
    pts = np.eye(3)
    assert np.array_equal(pkg.get_sphrquadrule("symmetric", pts, npts=3).pts, pts)


def test_tabulated_sphere_rules():
    """Tabulated rules given as text (src/collision/spherical_design/__init__.py:
    8-40,94-109): records per line or per parenthesised group, optional weights;
    the reference's checks on counts and weights."""
    import proj_int_inelastic_gb300 as pkg

    pts = np.array([[1.0, 0.0, 0.0], [-1.0, 0.0, 0.0], [0.0, 0.6, 0.8], [0.0, -0.6, -0.8]])
    lines = "\n".join(" ".join(repr(float(x)) for x in p) for p in pts)
    for text in (lines, "\n" + lines + "\n\n",
                 ", ".join("(" + ", ".join(repr(float(x)) for x in p) + ")" for p in pts),
                 "[" + ", ".join("(" + ", ".join(repr(float(x)) for x in p) + ")" for p in pts) + "]"):
        r = pkg.get_sphrquadrule("symmetric", text, npts=4)
        assert np.array_equal(r.pts, pts) and r.wts.shape == (0,), text
    w = "\n".join(" ".join(repr(float(x)) for x in p) + " 3.14159" for p in pts)
    r = pkg.get_sphrquadrule("symmetric", w, qdeg=1)
    assert np.array_equal(r.pts, pts) and np.all(r.wts == 3.14159)
    with pytest.raises(ValueError, match="Invalid number of points"):
        pkg.get_sphrquadrule("symmetric", lines, npts=6)
    with pytest.raises(ValueError, match="no quadrature weights"):
        pkg.get_sphrquadrule("symmetric", lines, qdeg=2)
    with pytest.raises(ValueError, match="Invalid points"):
        pkg.get_sphrquadrule("symmetric", "1 0\n0 1")
    with pytest.raises(ValueError, match="Invalid number of weights"):
        pkg.get_sphrquadrule("symmetric", "1 0 0 0.5\n0 1 0")
    # a tabulated rule in the config drives the mesh (a 4-direction design)
    cfg = op_config(16, L8_S, 4, 4, 0.9, 0.9, 1.0)
    cfg["spherical-design-rule"]["ssrule"] = lines
    sig, wsig = pkg.SpectralMesh(cfg).circ_or_sphr_quad()
    assert np.array_equal(sig, pts) and wsig == math.pi


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
    # the drop-in default is the reference's FP64 arithmetic; mixed precision is opt-in
    assert col.precision == "double" and col.default_with_loss is False
    cfg2 = dict(cfg, config={"precision": "mixed"})
    assert pkg.FSInelasticVHSCollision(cfg2, sm).precision == "mixed"
    # an empty batch gives an empty result without touching a GPU; wrong trailing axes raise
    for shape in ((0, 16, 16, 16), (3, 0, 16, 16, 16)):
        out = col(np.empty(shape))
        assert isinstance(out, np.ndarray) and out.shape == shape and out.dtype == np.float64
        assert col.collide(np.empty(shape), with_loss=True).shape == shape
        assert col.laplacian(np.empty(shape)).shape == shape
    with pytest.raises(ValueError):
        col(np.empty((0, 8, 8, 8)))


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


def test_solver_setup_and_config_errors_match_reference():
    """Boundary-condition errors of the ghost fill (src/solver.py:67-105) and
    the velocity-dimension check, raised before any GPU work."""
    import proj_int_inelastic_gb300 as pkg

    assert (pkg.BC.extrap, pkg.BC.periodic) == (1, 2)  # src/solver.py:5-7
    s = pkg.BoltzmannSolver1D(1.0)
    with pytest.raises(Exception, match="Lower boundary condition not specified."):
        s.setup(None)
    s.bc_lower = [pkg.BC.extrap]
    with pytest.raises(Exception, match="Upper boundary condition not specified."):
        s.setup(None)
    s.bc_upper = [3]
    with pytest.raises(NotImplementedError, match="Boundary condition 3 not implemented"):
        s.setup(None)
    s.bc_upper = [pkg.BC.periodic]
    s.setup(None)
    assert s._is_set_up
    # step-time checks of src/boltzmann.py:46-80 (before any device work)
    class _Sol:
        t = 0.0
        state = None

    s.time_integrator = "CONSP"
    with pytest.raises(ValueError, match="The penalty parameter is not given"):
        s.step(_Sol(), False, 0.0, 1.0)
    s.time_integrator, s.penalty = "CONSP_M", 1.0
    with pytest.raises(ValueError, match="The penalty parameter, e or tau are not given"):
        s.step(_Sol(), False, 0.0, 1.0)
    with pytest.raises(NotImplementedError, match="No stepping routine has been defined!"):
        pkg.Solver().step(_Sol(), False, 0.0, 1.0)
    with pytest.raises(NotImplementedError, match="No stepping routine has been defined!"):
        pkg.IterativeBoltzmannSolver().step(_Sol())
    with pytest.raises(ValueError, match="Dimension must be 2 or 3."):
        pkg.Solution({"dim_x": 1, "dim_v": 4, "xmin": 0.0, "xmax": 1.0, "l": 8.0, "nx": 4, "nv": 8})


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

    assert collision.GAIN_PATHS == {"pipeline": 0, "cluster": 1, "parity": 2, "packed": 3, "fused": 4}
    assert collision.DFT_PATHS == {"fft": 0, "tensor": 1}
    assert collision._code(collision.GAIN_PATHS, "packed", "gain_path") == 3
    with pytest.raises(ValueError, match="gain_path must be one of"):
        collision._code(collision.GAIN_PATHS, "fast", "gain_path")
    assert set(pkg._lib.SIGNATURES) >= {"pii_plan_set_dft_path", "pii_plan_get_dft_path"}



def test_grid_geometry_matches_reference_arithmetic():
    """``state.grid`` attributes (src/geometry.py:45-194): per-axis delta,
    centers and nodes by the reference's arithmetic (the velocity centres equal
    the oracle mesh's bit for bit), c_centers / c_nodes broadcast over the grid."""
    import proj_int_inelastic_gb300 as pkg
    from oracle import fs_inelastic as fo

    m = fo.Mesh(16, L8_S, 4, 6)
    g = pkg.Grid([8, 16, 16, 16], [0.0, -m.L, -m.L, -m.L], [1.0, m.L, m.L, m.L], 1)
    assert g.num_dim == 4 and g.num_dim_x == 1 and g.num_cells == [8, 16, 16, 16]
    assert g.delta[0] == 1.0 / 8 and g.delta[1] == m.delta
    for ax in (1, 2, 3):
        assert np.array_equal(g.centers[ax], m.v)
    assert np.array_equal(g.centers[0], (np.arange(8) + 0.5) / 8)
    assert len(g.nodes[0]) == 9 and g.nodes[0][-1] == 1.0 and g.nodes[1][0] == -m.L
    cc = g.c_centers
    assert len(cc) == 4 and all(c.shape == (8, 16, 16, 16) for c in cc)
    assert cc[0][3, 1, 2, 5] == g.centers[0][3] and cc[2][3, 1, 2, 5] == m.v[2] and cc[3][0, 0, 0, 5] == m.v[5]
    assert all(c.shape == (9, 17, 17, 17) for c in g.c_nodes)


def test_maxwellian_helper_matches_oracle():
    """``maxwellian`` (src/boltzmann.py:9-13) against the oracle's restatement."""
    import proj_int_inelastic_gb300 as pkg
    from oracle import integrators as it

    v = np.linspace(-5, 5, 12)
    vx, vy = np.meshgrid(v, v, indexing="ij")
    rho, u, T = np.array([1.0, 0.5]), np.array([0.2, -0.4]), np.array([1.1, 0.7])
    assert np.array_equal(pkg.maxwellian(vx, vy, rho, u, T), it.maxwellian_2d(vx, vy, rho, u, T))


@pytest.mark.parametrize("ti", ["Euler", "PFE", "TPI2", "TPI3", "CONSP"])
def test_per_integrator_methods_match_oracle(ti):
    """The reference's per-integrator methods (src/boltzmann.py:82-158) on the
    generic path (a Python collision callable, a homogeneous CPU state), and
    ``step`` dispatching to them by ``time_integrator``."""
    torch = pytest.importorskip("torch")
    import proj_int_inelastic_gb300 as pkg
    from oracle import integrators as it

    rng = np.random.default_rng(3)
    A = rng.uniform(-1.0, 1.0, (6, 6))

    def collision(f):  # a linear "collision" term, torch in -> torch out
        return f @ torch.as_tensor(A)

    kn, dt, K, h = 0.5, 0.2, [2, 2, 3], [0.01, 0.03, 0.1]
    f0 = rng.uniform(0.5, 1.5, (4, 6))

    class _State:
        pass

    class _Sol:
        pass

    s = pkg.BoltzmannSolver0D(kn, collision_operator=collision)
    s.dt, s.inner_steps, s.inner_dt, s.penalty = dt, K, h, 2.0
    method = {"Euler": s.euler_step, "PFE": s.proj_euler_step, "TPI2": s.tel_proj_step2,
              "TPI3": s.tel_proj_step3, "CONSP": s.convex_splitting_step}[ti]
    sol = _Sol()
    sol.state = _State()
    sol.state.f = torch.as_tensor(f0.copy())
    method(sol, False, 0.0, dt)
    ref = f0.copy()
    df = lambda f, hh: it.boltzmann_df(f, hh, lambda x: x @ A, kn)
    if ti == "Euler":
        it.euler_step(ref, dt, df)
    elif ti == "PFE":
        it.proj_euler_step(ref, dt, df, K, h)
    elif ti == "TPI2":
        it.tel_proj_step2(ref, dt, df, K, h)
    elif ti == "TPI3":
        it.tel_proj_step3(ref, dt, df, K, h)
    else:
        it.convex_splitting_step(ref, dt, lambda x: x @ A, kn, s.penalty)
    assert np.abs(sol.state.f.numpy() - ref).max() <= 1e-14 * np.abs(ref).max()
    # step() runs the same method
    s.time_integrator = ti
    sol.state.f = torch.as_tensor(f0.copy())
    s.step(sol, False, 0.0, dt)
    assert np.abs(sol.state.f.numpy() - ref).max() <= 1e-14 * np.abs(ref).max()


def test_header_is_plain_c_and_links():
    """include/pii_gb300.h is a C-ABI header: it compiles as C99 and C++11 on
    its own (no CUDA or torch types), and a C program built against it links
    with the library and calls the entry points that need no GPU."""
    import shutil
    import subprocess
    import tempfile

    import proj_int_inelastic_gb300 as pkg

    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    inc = os.path.join(ROOT, "include")
    for std, lang in (("c99", "c"), ("c++11", "c++")):
        r = subprocess.run([gcc if lang == "c" else (shutil.which("g++") or gcc), f"-std={std}", "-Wall",
                            "-Werror", "-fsyntax-only", "-x", lang, HEADER], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    prog = (
        '#include <stdio.h>\n#include <string.h>\n#include "pii_gb300.h"\n'
        "int main(void) {\n"
        "  int st = pii_plan_destroy(NULL);\n"
        '  printf("%s|%d|%s\\n", pii_version(), st, pii_last_error());\n'
        "  return strlen(pii_version()) > 0 ? 0 : 1;\n}\n")
    libdir = os.path.dirname(pkg._lib.LIB_PATH)
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "t.c"), os.path.join(d, "t")
        open(src, "w").write(prog)
        r = subprocess.run([gcc, "-std=c99", "-I", inc, src, "-o", exe, "-L", libdir, "-lpii_gb300",
                            f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        version, status, _ = r.stdout.strip().split("|", 2)
        assert version and int(status) != 0  # NULL plan: an error status, not a crash
