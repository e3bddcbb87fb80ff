"""FP64 NumPy restatement of the fast Fourier-spectral inelastic VHS operator.

Test infrastructure (the oracle), not product code.  Follows the reference
(Mayuyu/proj-int-inelastic) line by line in its arithmetic, but evaluates the
quadrature one radial node at a time and loops over cells, so that it never
materialises the reference's ``(n_r, n_sigma, cells, n, n, n)`` broadcast.

Conventions kept from the reference:

* velocity grid ``v_i = -L + (i + 1/2) * delta`` with ``delta = 2L/n``,
  ``R = 2S`` and ``L = (3 + sqrt 2) S / 2``
  (``src/collision/spectral_mesh.py:36-49,69-74,124-125``);
* Gauss-Legendre radial nodes mapped to ``[0, R]``
  (``src/collision/spectral_mesh.py:28-34``); equal-weight spherical design,
  ``w_sigma = 4 pi / n_sigma`` (``src/collision/spectral_mesh.py:58-66``);
* spectral index order ``fftshift(arange(-n/2, n/2))``, unnormalised forward
  FFT and 1/N inverse (``src/collision/inelastic_collisions.py:62,139-162``);
* 2D velocity (``dim = 2``): circle quadrature ``phi = arange(0, 2 pi, 2 pi /
  n_phi)``, ``sigma = (cos phi, sin phi)``, ``w = 2 pi / n_phi``
  (``src/collision/spectral_mesh.py:51-56,94-97``), kernel ``J_0`` instead of
  ``sinc`` and the circle constant ``2 pi`` (``inelastic_collisions.py:42-52``).
"""
import math
import os

import numpy as np
import scipy.fft
from scipy import special

_DESIGNS = os.path.join(
    os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
    "proj-int-inelastic_gb300",
    "data",
    "sphere_designs.npz",
)


def _workers():
    return int(os.environ.get("PII_ORACLE_WORKERS", os.cpu_count() or 1))


def fftn(x, workers=None, dim=3):
    return scipy.fft.fftn(x, axes=tuple(range(-dim, 0)), workers=workers or _workers())


def ifftn(x, workers=None, dim=3):
    return scipy.fft.ifftn(x, axes=tuple(range(-dim, 0)), workers=workers or _workers())


def sphere_design(npts):
    """Symmetric Womersley design with ``npts`` points, as selected by
    ``get_sphrquadrule("symmetric", rule="womersley", npts=...)``
    (``src/collision/spherical_design/__init__.py:62-116``)."""
    d = np.load(_DESIGNS)
    key = f"m{int(npts):05d}"
    if key not in d.files:
        raise ValueError("No suitable spherical quadrature rule found")
    return d[key].copy()


class Mesh:
    """Velocity mesh + quadratures (``src/collision/spectral_mesh.py:8-132``)."""

    def __init__(self, nv, s, nr=None, nsphr=32, sigma=None, dim=3, nphi=None):
        self.dim = int(dim)
        if self.dim not in (2, 3):
            raise ValueError("Dimension must be 2 or 3.")  # :23
        self.nv = int(nv)
        self.nr = int(nr if nr is not None else int(self.nv / 2))  # :43
        self.S = float(s)
        self.R = 2 * self.S  # :46-48
        self.L = 0.5 * (3.0 + math.sqrt(2)) * self.S
        x, w = np.polynomial.legendre.leggauss(self.nr)  # :28-34
        self.r = 0.5 * (x + 1) * self.R
        self.wr = 0.5 * self.R * w
        if self.dim == 2:
            self.nphi = int(nphi)
            self.wsigma = 2 * math.pi / self.nphi  # :53-54
            phi = np.arange(0, 2 * math.pi, self.wsigma)  # :55
            self.sigma = np.stack((np.cos(phi), np.sin(phi)), axis=-1)  # :94-97
        else:
            self.sigma = sphere_design(nsphr) if sigma is None else np.asarray(sigma, np.float64)
            self.wsigma = 4 * math.pi / self.sigma.shape[0]  # :66
        self.nsphr = self.sigma.shape[0]
        self.delta = 2 * self.L / self.nv  # :124-125
        self.v = np.array([-self.L + (i + 0.5) * self.delta for i in range(self.nv)])  # :69-74

    def v_centers(self):
        return np.meshgrid(*([self.v] * self.dim), indexing="ij")


class FSInelasticVHS:
    """Tables and evaluation of Q(f,f) in 2D or 3D velocity (``mesh.dim``).

    Tables follow ``perform_precomputation``
    (``src/collision/inelastic_collisions.py:57-137``) with ``e``, ``e0`` and
    ``gamma`` as in ``load_parameters`` (``:30-52``); the gain and ``exp``
    tables are produced per radial node by :meth:`tables_r`.
    """

    def __init__(self, mesh, e=1.0, e0=1.0, gamma=0.0):
        self.m = mesh
        self.e_in, self.e0, self.gamma = float(e), float(e0), float(gamma)
        n = mesh.nv
        d = self.dim = mesh.dim
        self.sphr_fac = 2 * math.pi ** (0.5 * d) / math.gamma(0.5 * d)  # :50-52 (4 pi in 3D, 2 pi in 2D)
        idx = np.fft.fftshift(np.arange(-int(n / 2), int(n / 2)))  # :62
        self.idx = idx
        idx_norm, idx_square = 0, idx**2  # :63-67
        for i in range(d):
            idx_norm = idx_norm + idx_square[(...,) + (None,) * i]
        self.idx_norm = np.sqrt(idx_norm)
        self.lapl = -math.pi**2 / mesh.L**2 * self.idx_norm**2  # :69
        r = mesh.r
        # r-dependent restitution and exponential factor (:77-80)
        self.e_r = 0.5 * (self.e0 - self.e_in) * np.tanh(r - 0.5 * mesh.R) + 0.5 * (self.e0 + self.e_in)
        self.exp_fac = 0.25 * math.pi * (1 + self.e_r) / mesh.L
        # k . sigma mesh (n_sigma, n, ..., n), built in the reference's order (:86-90)
        sigma = mesh.sigma
        idx_mesh = 0
        for i in range(d):
            idx_mesh = np.expand_dims(idx_mesh, axis=-1) + idx * sigma[(slice(None), slice(i, i + 1)) + (None,) * i]
        self.kdotsig = idx_mesh
        # loss (:109-114)
        self.loss_kern = self.pre_fac(r) * mesh.wr
        # the reference precomputes every table once (:57-137); cache them up to ~4 GB
        self._cache = {}
        self._cache_ok = 2 * mesh.nr * mesh.nsphr * mesh.nv**d * 16 <= (4 << 30)

    def pre_fac(self, r):
        return self.sphr_fac * r ** (self.gamma + self.dim - 1)  # :54-55

    def sinc(self, x):
        """sp_func (:42-45): J_0 in 2D, sin(x)/x in 3D."""
        if self.dim == 2:
            return special.jv(0, x)
        return np.sinc(x / np.pi)

    def tables_r(self, ir):
        """Gain and exp tables of radial node ``ir``: (n_sigma, n, n, n) complex128 (:91-105)."""
        if ir in self._cache:
            return self._cache[ir]
        out = self._tables_r(ir)
        if self._cache_ok:
            self._cache[ir] = out
        return out

    def _tables_r(self, ir):
        r = self.m.r[ir]
        wr = self.m.wr[ir]
        a = self.exp_fac[ir]
        mesh_r = self.kdotsig * r
        gain = self.pre_fac(r) * np.exp(1j * a * mesh_r) * self.sinc(a * r * self.idx_norm)
        gain *= wr
        gain *= self.m.wsigma
        exp = np.exp(-1j * math.pi * mesh_r / self.m.L)
        return gain, exp

    def sp_r(self, ir):
        return self.sinc(math.pi * self.m.r[ir] * self.idx_norm / self.m.L)  # :111-114

    def collide_cell(self, f, with_loss=False, workers=None):
        """One cell of ``collide`` (``src/collision/inelastic_collisions.py:208-227``)."""
        f = np.asarray(f, dtype=np.float64)
        d = self.dim
        f_hat = fftn(f, workers, d)
        gain_hat = np.zeros(f.shape, dtype=np.complex128)
        for ir in range(self.m.nr):
            g_r, e_r = self.tables_r(ir)
            b = fftn(ifftn(e_r * f_hat, workers, d) * f, workers, d)
            b *= g_r
            gain_hat += b.sum(axis=0)
        gain = ifftn(gain_hat, workers, d)
        loss = np.zeros(f.shape, dtype=np.complex128)
        for ir in range(self.m.nr):
            loss += ifftn(self.sp_r(ir) * f_hat, workers, d) * (self.loss_kern[ir] * f)
        if with_loss:
            return (gain / self.sphr_fac - loss).real
        return (gain / self.sphr_fac).real

    def collide(self, f, with_loss=False, workers=None):
        f = np.asarray(f, dtype=np.float64)
        d = self.dim
        lead = f.shape[:-d]
        flat = f.reshape((-1,) + f.shape[-d:])
        out = np.empty_like(flat)
        for c in range(flat.shape[0]):
            out[c] = self.collide_cell(flat[c], with_loss, workers)
        return out.reshape(lead + f.shape[-d:])

    def laplacian(self, f, workers=None):
        """Heat-bath term (``src/collision/inelastic_collisions.py:229-230``)."""
        return ifftn(self.lapl * fftn(f, workers, self.dim), workers, self.dim).real

    def __call__(self, f, heat_bath=None, with_loss=False):
        """``BaseCollision.__call__`` on the CPU (``src/collision/base.py:32-42``)."""
        out = self.collide(f, with_loss)
        if heat_bath:
            out = out + heat_bath * self.laplacian(f)
        return out


def mass_mode_correction(q, dim=3):
    """Subtract the velocity-grid mean so that sum_v Q = 0 (the k = 0 mode).

    Not in the reference: the product offers it as an opt-in FP64 fix-up after
    the parity-checked operator, and this restatement is its checker.
    """
    q = np.asarray(q, np.float64)
    return q - q.mean(axis=tuple(range(-dim, 0)), keepdims=True)
