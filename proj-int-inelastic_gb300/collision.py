"""Drop-in GB300 collision operator with the reference's call signatures.

* ``SpectralMesh(config)`` -- velocity mesh and quadratures
  (src/collision/spectral_mesh.py:8-132);
* ``FSInelasticVHSCollision(config, spectral_mesh)`` -- the fast
  Fourier-spectral inelastic VHS operator (3D velocity: sinc kernel on a
  spherical design; 2D velocity: J_0 kernel on the circle quadrature) with ``__call__(input_f,
  heat_bath=None, device=...)``, ``collide(input_f, with_loss=False)`` and
  ``laplacian(input_f)`` (src/collision/base.py:7-58,
  src/collision/inelastic_collisions.py:116-230).

Both take the reference's nested-dict config (``config["velocity-mesh"]["nv"]``
...).  The operator evaluates on the GPU through ``libpii_gb300.so``; it
accepts NumPy arrays (returned as NumPy, as the reference returns) or torch
CUDA tensors (returned as torch CUDA tensors, no host copy).  There is no CPU
path: ``device`` is accepted for signature compatibility only.
"""
import math
import os
import re

import numpy as np
import torch

from . import _lib

_DESIGNS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "sphere_designs.npz")


class SphericalQuadRule:
    """A spherical quadrature rule: ``pts`` (m x 3 unit vectors) and ``wts``
    (one weight per point, or empty when the rule carries none), the two
    attributes of the reference's rule objects
    (src/collision/spherical_design/__init__.py:7-40)."""

    def __init__(self, pts, wts=()):
        self.pts = np.asarray(pts, np.float64).reshape(-1, 3)
        self.wts = np.asarray(wts, np.float64).reshape(-1)


def _parse_tabulated(text):
    """Points (and optional weights) of a tabulated rule: one record ``x y z``
    or ``x y z w`` per line or per parenthesised group, numbers separated by
    blanks or commas, optionally enclosed in [ ] (the text format read at
    src/collision/spherical_design/__init__.py:8-40)."""
    body = text.strip()
    if body.startswith("[") and body.endswith("]"):
        body = body[1:-1]
    records = re.findall(r"\(([^()]*)\)", body) if "(" in body else body.splitlines()
    pts, wts = [], []
    for rec in records:
        vals = [float(x) for x in rec.replace(",", " ").split()]
        if not vals:
            continue
        if len(vals) == 3:
            pts.append(vals)
        elif len(vals) == 4:
            pts.append(vals[:3])
            wts.append(vals[3])
        else:
            raise ValueError("Invalid points in quadrature rule")
    if wts and len(wts) != len(pts):
        raise ValueError("Invalid number of weights")
    return SphericalQuadRule(pts, wts)


def get_sphrquadrule(sstype, rule=None, npts=None, qdeg=None, flags=None):
    """Symmetric spherical design, as ``get_sphrquadrule``
    (src/collision/spherical_design/__init__.py:91-116): returns a rule with
    ``pts`` / ``wts``.

    * ``rule`` a name (``"womersley"``, or None): the stored Womersley
      symmetric design with exactly ``npts`` points (the strongest if several),
      or the one with the fewest points of strength >= ``qdeg``;
    * ``rule`` a tabulated rule (text of ``x y z [w]`` records), or an (m, 3)
      array of unit vectors: that point set, checked against ``npts``.
    """
    if sstype != "symmetric":
        raise ValueError(f"unknown spherical design type {sstype!r}")
    tabulated = None
    if rule is not None and not isinstance(rule, str):
        tabulated = SphericalQuadRule(rule)
    elif rule and not re.fullmatch(r"[A-Za-z0-9_\-~+]+", rule):
        tabulated = _parse_tabulated(rule)
    if tabulated is not None:
        if npts and npts != len(tabulated.pts):
            raise ValueError("Invalid number of points in provided rule")
        if qdeg and not len(tabulated.wts):
            raise ValueError("Provided rule has no quadrature weights")
        return tabulated
    if not npts and not qdeg:
        raise ValueError("Must specify either npts or qdeg")
    if rule not in (None, "", "womersley"):
        raise ValueError("No suitable spherical quadrature rule found")
    d = np.load(_DESIGNS)
    best = None
    for key in d.files:
        if not key.startswith("m"):
            continue
        m = int(key[1:])
        q = int(d[f"qdeg_{key}"])
        if (not npts or npts == m) and (not qdeg or qdeg <= q):
            if best is None or (npts and q > best[2]) or (qdeg and m < best[1]):
                best = (key, m, q)
    if best is None:
        raise ValueError("No suitable spherical quadrature rule found")
    return SphericalQuadRule(d[best[0]].copy())


class SpectralMesh:
    """Velocity mesh and quadratures (src/collision/spectral_mesh.py:8-132)."""

    def __init__(self, config, *args, **kwargs):
        self.config = config
        vm = config["velocity-mesh"]
        self._nv = int(vm["nv"])
        self._nr = int(vm.get("nr", int(self._nv / 2)))
        self._S = float(vm["s"])
        self._R = 2 * self._S
        self._L = 0.5 * (3.0 + math.sqrt(2)) * self._S
        quad_rule = vm.get("quad-rule", "legendre")
        if quad_rule != "legendre":
            raise KeyError(quad_rule)
        x, w = np.polynomial.legendre.leggauss(self._nr)
        self._r = 0.5 * (x + 1) * self._R
        self._wr = 0.5 * self._R * w
        self._ndim = int(config["collision-model"]["dim"])
        if self._ndim == 2:
            # circle quadrature (src/collision/spectral_mesh.py:51-56)
            self._nphi = int(config["circle-quad-rule"]["nphi"])
            self._wphi = 2 * math.pi / self._nphi
            self._phi = np.arange(0, 2 * math.pi, self._wphi)
        elif self._ndim == 3:
            sp = config["spherical-design-rule"]
            self._ssrule = sp.get("ssrule", "womersley")
            self._nsphr = int(sp["nsphr"])
            self._spts = get_sphrquadrule("symmetric", rule=sp.get("points", self._ssrule), npts=self._nsphr).pts
            self._wspts = 4 * math.pi / self._nsphr
        else:
            raise ValueError("Dimension must be 2 or 3.")
        self._v_center = None
        self._v_centers = None

    @property
    def v_center(self):
        if self._v_center is None:
            self._v_center = np.array([-self.L + (i + 0.5) * self.delta for i in range(self.nv)])
        return self._v_center

    @property
    def v_centers(self):
        if self._v_centers is None:
            index = np.indices(self.nv_s)
            self._v_centers = [self.v_center[index[i, ...]] for i in range(self.ndim)]
        return self._v_centers

    @property
    def ncirc_or_nsphr(self):
        return self._nphi if self._ndim == 2 else self._nsphr

    def circ_or_sphr_quad(self):
        """(directions, weight): (cos phi, sin phi) and 2 pi / n_phi in 2D, the
        spherical design and 4 pi / n_sigma in 3D (src/collision/spectral_mesh.py:94-101)."""
        if self._ndim == 2:
            return np.stack((np.cos(self._phi), np.sin(self._phi)), axis=-1), self._wphi
        return self._spts, self._wspts

    @property
    def ndim(self):
        return self._ndim

    @property
    def nv(self):
        return self._nv

    @property
    def nv_s(self):
        return [self.nv] * self.ndim

    @property
    def L(self):
        return self._L

    @property
    def R(self):
        return self._R

    @property
    def delta(self):
        return 2 * self.L / self.nv

    @property
    def nr(self):
        return self._nr

    def rquad(self):
        return self._r, self._wr


def _precision_of(config, precision):
    if precision is None:
        precision = str(config.get("config", {}).get("precision", "double")).lower()
    if precision in ("double", "fp64", "float64"):
        return _lib.PREC_FP64
    if precision in ("mixed", "single", "fp32", "float32"):
        return _lib.PREC_FP32
    raise ValueError(f"precision must be 'mixed'/'fp32' or 'double'/'fp64', got {precision!r}")


GAIN_PATHS = {"pipeline": 0, "cluster": 1, "parity": 2, "packed": 3, "fused": 4}
# first-axis column transforms of the n = 64 FP32 pipeline
DFT_PATHS = {"fft": 0, "tensor": 1}


def _code(table, name, what):
    if name not in table:
        raise ValueError(f"{what} must be one of {sorted(table)}, got {name!r}")
    return table[name]


class Plan:
    """Owner of one ``pii_plan`` (device tables + workspace for batch_max cells)."""

    def __init__(self, mesh, e, e0, gamma, precision, batch_max, device, gain_path=None):
        lib = _lib.load()
        self.n = mesh.nv
        self.batch_max = int(batch_max)
        self.device = int(device)
        self.precision = precision
        r, wr = mesh.rquad()
        sigma, wsigma = mesh.circ_or_sphr_quad()
        self._r = np.ascontiguousarray(r, np.float64)
        self._wr = np.ascontiguousarray(wr, np.float64)
        self._sigma = np.ascontiguousarray(sigma, np.float64)
        self.dim = int(mesh.ndim)
        h = _lib._vp()
        torch.cuda.init()
        st = lib.pii_plan_create_nd(
            _lib.ctypes.byref(h), self.dim, int(mesh.nv), int(len(self._r)), int(len(self._sigma)),
            _lib.dptr(self._r), _lib.dptr(self._wr), _lib.dptr(self._sigma), float(wsigma), float(mesh.L),
            float(mesh.R), float(e), float(e0), float(gamma), int(precision), self.batch_max, self.device)
        _lib.check(st, "pii_plan_create_nd")
        self.handle = h.value
        self._lib = lib
        if gain_path is not None:
            _lib.check(lib.pii_plan_set_gain_path(self.handle, _code(GAIN_PATHS, gain_path, "gain_path")),
                       "pii_plan_set_gain_path")

    def autotune(self, cells):
        """Time the kernel choices for `cells` cells and keep the fastest
        (``pii_plan_autotune``); returns (best ms, choices)."""
        best = _lib.ctypes.c_double()
        _lib.check(self._lib.pii_plan_autotune(self.handle, int(cells), _lib.ctypes.byref(best),
                                               torch.cuda.current_stream().cuda_stream), "pii_plan_autotune")
        return best.value, self.tuning

    def set_tuning(self, gain_path, items_per_cluster, chunk_points, dft_path=None, fused_split=None, **_):
        """Restore choices (as returned by :attr:`tuning`), ``pii_plan_set_tuning``
        (and ``pii_plan_set_dft_path`` / ``pii_plan_set_fused_split`` when
        `dft_path` / `fused_split` is given)."""
        _lib.check(self._lib.pii_plan_set_tuning(self.handle, _code(GAIN_PATHS, gain_path, "gain_path"),
                                                 int(items_per_cluster), int(chunk_points)), "pii_plan_set_tuning")
        if dft_path is not None:
            self.set_dft_path(dft_path)
        if fused_split is not None:
            self.set_fused_split(fused_split)

    def set_fused_split(self, fraction):
        """Share of a call's cells that the packed pipeline takes on a side
        stream while the fused kernel runs (gain path "fused" at n = 48, 64,
        whose clusters leave SMs idle; 0 turns it off),
        ``pii_plan_set_fused_split``."""
        _lib.check(self._lib.pii_plan_set_fused_split(self.handle, float(fraction)), "pii_plan_set_fused_split")

    def set_dft_path(self, dft_path):
        """'fft' (CUDA-core FFT) or 'tensor' (tensor-core split-FP16 DFT; n = 64
        FP32 plans) for the first-axis column transforms, ``pii_plan_set_dft_path``."""
        _lib.check(self._lib.pii_plan_set_dft_path(self.handle, _code(DFT_PATHS, dft_path, "dft_path")),
                   "pii_plan_set_dft_path")

    NYQUIST_PATHS = {"quadratic": 0, "direct": 1}

    def set_nyquist_path(self, path):
        """Nyquist-plane correction of the packed paths: "quadratic" (the
        precomputed quadratic form in f^, the default where its kernels fit
        the memory budget) or "direct" (the per-pass kernels),
        ``pii_plan_set_nyquist_path``."""
        _lib.check(self._lib.pii_plan_set_nyquist_path(self.handle, _code(self.NYQUIST_PATHS, path, "nyquist_path")),
                   "pii_plan_set_nyquist_path")

    @property
    def nyquist_path(self):
        return {0: "quadratic", 1: "direct"}.get(int(self._lib.pii_plan_get_nyquist_path(self.handle)))

    def set_restitution(self, e, e0):
        """Per-cell restitution: cell c of later calls uses (e[c], e0[c])
        (``pii_plan_set_restitution``); empty sequences restore the plan's own."""
        e = np.ascontiguousarray(e, np.float64)
        e0 = np.ascontiguousarray(e0, np.float64)
        if e.shape != e0.shape or e.ndim != 1:
            raise ValueError("e and e0 must be 1D sequences of the same length")
        _lib.check(self._lib.pii_plan_set_restitution(self.handle, _lib.dptr(e), _lib.dptr(e0), len(e)),
                   "pii_plan_set_restitution")
        self.restitution_sets = len(e)

    def dft_test_hooks(self, wait_limit=1 << 22, withhold=False):
        """Test hooks of the bounded waits of the tensor-core DFT and the fused
        cluster kernel (``pii_plan_dft_test_hooks``): polls before a wait gives
        up, and whether the copies / exchange stores are withheld (so the waits
        run out with nothing in flight)."""
        _lib.check(self._lib.pii_plan_dft_test_hooks(self.handle, int(wait_limit), int(bool(withhold))),
                   "pii_plan_dft_test_hooks")

    @property
    def graph_count(self):
        """Instantiated macro-step graphs held by the plan (bounded)."""
        return int(self._lib.pii_plan_graph_count(self.handle))

    @property
    def dft_stalled(self):
        """True if a tensor-core DFT or fused-kernel launch gave up waiting and
        the stall has not been reported by a later call yet
        (``pii_plan_get_dft_path``; synchronises)."""
        path, stalled = _lib.ctypes.c_int(), _lib.ctypes.c_int()
        _lib.check(self._lib.pii_plan_get_dft_path(self.handle, _lib.ctypes.byref(path), _lib.ctypes.byref(stalled)),
                   "pii_plan_get_dft_path")
        return bool(stalled.value)

    @property
    def tuning(self):
        path, items, pts = _lib.ctypes.c_int(), _lib.ctypes.c_int(), _lib.ctypes.c_int64()
        _lib.check(self._lib.pii_plan_get_tuning(self.handle, _lib.ctypes.byref(path), _lib.ctypes.byref(items),
                                                 _lib.ctypes.byref(pts)), "pii_plan_get_tuning")
        dft = _lib.ctypes.c_int()
        _lib.check(self._lib.pii_plan_get_dft_path(self.handle, _lib.ctypes.byref(dft), None), "pii_plan_get_dft_path")
        return {"gain_path": {v: k for k, v in GAIN_PATHS.items()}[path.value], "items_per_cluster": items.value,
                "chunk_points": pts.value, "dft_path": {v: k for k, v in DFT_PATHS.items()}[dft.value],
                "fused_split": float(self._lib.pii_plan_get_fused_split(self.handle))}

    @property
    def workspace_bytes(self):
        return int(self._lib.pii_plan_workspace_bytes(self.handle))

    def close(self):
        if getattr(self, "handle", None):
            self._lib.pii_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _stream_handle():
    return torch.cuda.current_stream().cuda_stream


class FSInelasticVHSCollision:
    """GB300 fast-spectral inelastic VHS collision operator.

    Same constructor and methods as the reference class
    (src/collision/inelastic_collisions.py:116-230, src/collision/base.py:6-58).
    Extra keyword arguments (not in the reference):

    * ``precision``  -- "double" (all FP64, the reference's arithmetic and the
      default) or "mixed" (FP32 FFTs and quadrature sums, FP64 state and
      output: ~1e-6 relative to FP64, tens of times faster); also read from
      ``config["config"]["precision"]``;
    * ``with_loss``  -- what ``__call__`` evaluates: the reference's ``__call__``
      never passes ``with_loss``, so it returns the gain term only (default
      False, kept); True returns Q+ - Q-;
    * ``mass_fix``   -- subtract the per-cell mean of Q in FP64 (k = 0 mode);
    * ``batch_max``  -- initial cell capacity of the plan (grown on demand);
    * ``device``     -- CUDA device index;
    * ``gain_path``  -- in mixed precision: "packed" (each antipodal direction
      pair (sigma, -sigma) in one real-phase pass, plus the Nyquist-plane
      correction; the default where the design is antipodally symmetric: the
      fused a-parity kernel for n = 32, the column / plane pipeline otherwise),
      for n = 32 also "parity" (fused a-parity kernel with a tensor-memory
      accumulator, the default otherwise) or "cluster" (fused 2-CTA-cluster
      kernel); "pipeline" (column / plane passes on every pair) in every case.
      All evaluate the same operator.
    """

    collision_model = "vhs"

    def __init__(self, config, spectral_mesh, precision=None, with_loss=False, mass_fix=False, batch_max=1,
                 device=0, gain_path=None, **kwargs):
        self.config = config
        self.sm = spectral_mesh
        self.ndim = int(config["collision-model"]["dim"])
        assert self.ndim == self.sm.ndim, (
            "'spectral_mesh' has different velocity dimensions from collision model! This may be caused by "
            "using different config files. Please check the consistency.")
        self.load_parameters()
        self._precision = _precision_of(config, precision)
        self.default_with_loss = bool(with_loss)
        self.mass_fix = bool(mass_fix)
        self._device = int(device)
        self._gain_path = gain_path
        self._plan = None
        self._batch_max = max(1, int(batch_max))
        self._pinned = {}
        self._input_shape = None

    # -- reference hooks -------------------------------------------------
    def load_parameters(self):
        """``load_parameters`` (src/collision/inelastic_collisions.py:30-52)."""
        cm = self.config["collision-model"]
        self._e = float(cm.get("e", 1.0))
        self._e0 = float(cm.get("e0", 1.0))
        self._gamma = float(cm.get("gamma", 0.0))
        if self.ndim not in (2, 3):
            raise ValueError("Dimension must be 2 or 3.")
        self._sphr_fac = 2 * math.pi ** (0.5 * self.ndim) / math.gamma(0.5 * self.ndim)

    def perform_precomputation(self):
        """Tables are built on the device by the plan (``pii_plan_create``)."""
        self._ensure_plan(self._batch_max)

    @property
    def precision(self):
        return "double" if self._precision == _lib.PREC_FP64 else "mixed"

    @property
    def plan(self):
        return self._ensure_plan(self._batch_max)

    def _ensure_plan(self, cells):
        sets = getattr(self._plan, "restitution_sets", 0)
        if sets > 1 and cells > sets:
            # a grown plan would drop the per-cell restitution: refuse like the C ABI does
            raise ValueError(f"{cells} cells for a plan with {sets} per-cell restitution sets")
        if self._plan is None or self._plan.batch_max < cells:
            if self._plan is not None:
                torch.cuda.synchronize(self._device)
                self._plan.close()
            self._batch_max = max(self._batch_max, int(cells))
            self._plan = Plan(self.sm, self._e, self._e0, self._gamma, self._precision, self._batch_max,
                              self._device, self._gain_path)
        return self._plan

    # -- evaluation --------------------------------------------------------
    def _as_device(self, input_f):
        """(device FP64 contiguous tensor, was_numpy)."""
        n, d = self.sm.nv, self.ndim
        if tuple(input_f.shape[-d:]) != (n,) * d or len(input_f.shape) < d:
            raise ValueError(f"input_f must end with {(n,) * d}, got {tuple(input_f.shape)}")
        if isinstance(input_f, torch.Tensor):
            t = input_f
            if not t.is_cuda:
                t = t.to(f"cuda:{self._device}")
            return t.to(torch.float64).contiguous(), False
        a = np.ascontiguousarray(input_f, dtype=np.float64)
        key = a.shape
        pin = self._pinned.get(key)
        if pin is None:
            pin = (torch.empty(key, dtype=torch.float64).pin_memory(),
                   torch.empty(key, dtype=torch.float64).pin_memory())
            self._pinned = {key: pin}
        pin[0].numpy()[...] = a
        return pin[0].to(f"cuda:{self._device}", non_blocking=True), True

    def _run(self, input_f, with_loss, heat_bath, laplacian=False):
        n, d = self.sm.nv, self.ndim
        if len(input_f.shape) >= d and tuple(input_f.shape[-d:]) == (n,) * d and int(np.prod(input_f.shape)) == 0:
            # an empty batch of cells: an empty result, as the reference's transforms give
            if isinstance(input_f, torch.Tensor):
                return torch.empty(tuple(input_f.shape), dtype=torch.float64, device=input_f.device)
            return np.empty(tuple(input_f.shape), dtype=np.float64)
        f, was_np = self._as_device(input_f)
        lead = f.shape[:-self.ndim]
        cells = int(np.prod(lead)) if len(lead) else 1
        plan = self._ensure_plan(cells)
        q = torch.empty_like(f)
        if laplacian:
            st = plan._lib.pii_laplacian(plan.handle, f.data_ptr(), q.data_ptr(), cells, _stream_handle())
            _lib.check(st, "pii_laplacian")
        else:
            st = plan._lib.pii_collide(plan.handle, f.data_ptr(), q.data_ptr(), cells, int(bool(with_loss)),
                                       float(heat_bath or 0.0), int(self.mass_fix), _stream_handle())
            _lib.check(st, "pii_collide")
        self._input_shape = tuple(f.shape)
        if was_np:
            out = self._pinned[tuple(f.shape)][1]
            out.copy_(q, non_blocking=True)
            torch.cuda.current_stream().synchronize()
            return out.numpy().copy()
        return q

    def __call__(self, input_f, heat_bath=None, device="gpu"):
        """``BaseCollision.__call__`` (src/collision/base.py:32-58): Q of each
        cell (gain only unless the operator was built with ``with_loss=True``),
        plus ``heat_bath * laplacian`` when ``heat_bath`` is truthy."""
        if device not in ("cpu", "gpu", "cuda"):
            raise ValueError(f"unknown device {device!r}")
        return self._run(input_f, self.default_with_loss, heat_bath if heat_bath else 0.0)

    def collide(self, input_f, with_loss=False):
        """``collide`` (src/collision/inelastic_collisions.py:208-227)."""
        return self._run(input_f, with_loss, 0.0)

    def laplacian(self, input_f):
        """Heat-bath Laplacian (src/collision/inelastic_collisions.py:229-230):
        one forward and one inverse transform in the plan's precision
        (``pii_laplacian``)."""
        return self._run(input_f, False, 0.0, laplacian=True)

    def close(self):
        if self._plan is not None:
            self._plan.close()
            self._plan = None
