"""The algebra behind the packed (antipodal) gain path, checked in FP64 on the CPU.

The n = 32 FP32 default gain path evaluates each antipodal direction pair
(sigma, -sigma) of the symmetric designs in one real-phase pass
(`k_gain_parity<1>`) and adds what that pass leaves out, which lives on the
Nyquist planes only, with `k_nyq_corr`.  The GPU tests check the result against
the oracle; these tests check the identities themselves with NumPy, on the
oracle's own tables (`src/collision/inelastic_collisions.py:91-105`) and the
reference's per-pair gain term (`:212-217`):

1. per antipodal pair (p, q = -sigma_p), with Herm(X)(k) = (X(k) + conj X(-k)) / 2
   (only Re IFFT3 of the gain sum is used, and Re IFFT3 X = IFFT3 Herm X),
     Herm(g_p B_p + g_q B_q) = Herm(2 s F) + C,
   B = FFT3(IFFT3(E f^) f), F = FFT3(IFFT3(f^ t) f), t = Re E+_p + Im E+_p,
   s = Re g+_p - Im g+_p, and on the Nyquist planes only
   C = (w.x - w.y) U - (w.x + w.y) conj U(-k), w = g-_p, U = FFT3(IFFT3(f^ t-) f),
   t- = Re E-_p + Im E-_p (X+ = Herm X, X- = X - X+);
2. U on the three Nyquist planes from 2D transforms only: V = IFFT3(f^ t-) is
   (-1)^a P_a(b, c) + (-1)^b P_b(a, c) + (-1)^c P_c(a, b) over n^3, and the plane
   k_a = n/2 of U is the 2D forward transform of R_a(b, c) = sum_a (-1)^a V f,
   with R_a = (P_a F_a + (-1)^b sum_a (-1)^a P_b f + (-1)^c sum_a (-1)^a P_c f) / n^3
   (likewise k_b, k_c), the reductions `k_nyq_corr` runs in shared memory.
"""
import numpy as np
import pytest

from conftest import L8_S
from oracle import fs_inelastic as fo


def _herm(x):
    """(X(k) + conj X(-k)) / 2 on the grid (indices mod n)."""
    xr = np.conj(np.roll(np.flip(x, axis=(-3, -2, -1)), 1, axis=(-3, -2, -1)))
    return 0.5 * (x + xr)


def _reflect(x):
    """X(-k) on the grid (indices mod n)."""
    return np.roll(np.flip(x, axis=(-3, -2, -1)), 1, axis=(-3, -2, -1))


def _fft3(x):
    return np.fft.fftn(x, axes=(-3, -2, -1))


def _ifft3(x):
    return np.fft.ifftn(x, axes=(-3, -2, -1))


def _nyquist_mask(n):
    h = n // 2
    m = np.zeros((n, n, n), bool)
    m[h, :, :] = m[:, h, :] = m[:, :, h] = True
    return m


def _antipodes(sigma):
    d = np.abs(sigma[:, None, :] + sigma[None, :, :]).max(-1)
    q = d.argmin(axis=1)
    assert np.all(d[np.arange(len(sigma)), q] < 1e-12), "design is not antipodally symmetric"
    return [(p, int(q[p])) for p in range(len(sigma)) if p < q[p]]


@pytest.mark.parametrize("n,nsphr,e,gamma", [(8, 6, 0.8, 1.0), (16, 32, 0.7, 0.0)])
def test_packed_pair_plus_nyquist_correction_equals_direct_pair(n, nsphr, e, gamma):
    mesh = fo.Mesh(n, L8_S, 3, nsphr)
    op = fo.FSInelasticVHS(mesh, e, e, gamma)
    rng = np.random.default_rng(20260 + n)
    f = rng.uniform(0.1, 1.0, (n, n, n))  # a full spectrum: the Nyquist planes carry weight
    fh = _fft3(f)
    nyq = _nyquist_mask(n)
    worst, corr_scale = 0.0, 0.0
    for ir in range(mesh.nr):
        gain, expt = op.tables_r(ir)
        for p, q in _antipodes(mesh.sigma):
            # the antipode's tables are the conjugates (k . sigma changes sign)
            assert np.allclose(expt[q], np.conj(expt[p]), rtol=0, atol=1e-14)
            assert np.allclose(gain[q], np.conj(gain[p]), rtol=0, atol=1e-14 * np.abs(gain[p]).max())
            direct = _herm(gain[p] * _fft3(_ifft3(expt[p] * fh) * f) + gain[q] * _fft3(_ifft3(expt[q] * fh) * f))
            ep, gp = _herm(expt[p]), _herm(gain[p])
            t = ep.real + ep.imag
            s = gp.real - gp.imag
            packed = _herm(2.0 * s * _fft3(_ifft3(fh * t) * f))
            em, gm = expt[p] - ep, gain[p] - gp
            assert np.all(em[~nyq] == 0) and np.all(gm[~nyq] == 0)  # E-, g- live on the Nyquist planes
            tm = em.real + em.imag
            u = _fft3(_ifft3(fh * tm) * f)
            corr = (gm.real - gm.imag) * u - (gm.real + gm.imag) * np.conj(_reflect(u))
            scale = np.abs(direct).max()
            worst = max(worst, np.abs(packed + corr - direct).max() / scale)
            corr_scale = max(corr_scale, np.abs(corr).max() / scale)
    assert worst < 1e-13, worst
    assert corr_scale > 1e-6  # the correction is not vacuous on this input


def test_nyquist_planes_from_2d_transforms():
    n, h = 16, 8
    mesh = fo.Mesh(n, L8_S, 2, 32)
    op = fo.FSInelasticVHS(mesh, 0.8, 0.8, 1.0)
    rng = np.random.default_rng(7)
    f = rng.uniform(0.1, 1.0, (n, n, n))
    fh = _fft3(f)
    _, expt = op.tables_r(1)
    ep = _herm(expt[5])
    em = expt[5] - ep
    y = fh * (em.real + em.imag)  # f^ t-, zero off the Nyquist planes
    # the three point sets: A = {k_a = h}, B = {k_b = h, k_a != h}, C = {k_c = h, k_a, k_b != h}
    ya = y[h, :, :]
    yb = y[:, h, :].copy()
    yb[h, :] = 0
    yc = y[:, :, h].copy()
    yc[h, :] = 0
    yc[:, h] = 0
    n2 = n * n
    pa = np.fft.ifft2(ya) * n2  # unnormalised 2D inverse transforms
    pb = np.fft.ifft2(yb) * n2
    pc = np.fft.ifft2(yc) * n2
    sg = (-1.0) ** np.arange(n)
    a_, b_, c_ = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    v = (sg[a_] * pa[b_, c_] + sg[b_] * pb[a_, c_] + sg[c_] * pc[a_, b_]) / n**3
    assert np.abs(v - _ifft3(y)).max() < 1e-14 * np.abs(v).max()
    u = _fft3(v * f)
    # plane k_a = h from R_a, the form with the own-plane term P_a F_a
    fa, fb, fc = f.sum(0), f.sum(1), f.sum(2)
    ra = (pa * fa + sg[:, None] * np.einsum("a,ac,abc->bc", sg, pb, f)
          + sg[None, :] * np.einsum("a,ab,abc->bc", sg, pc, f)) / n**3
    rb = (sg[:, None] * np.einsum("b,bc,abc->ac", sg, pa, f) + pb * fb
          + sg[None, :] * np.einsum("b,ab,abc->ac", sg, pc, f)) / n**3
    rc = (sg[:, None] * np.einsum("c,bc,abc->ab", sg, pa, f)
          + sg[None, :] * np.einsum("c,ac,abc->ab", sg, pb, f) + pc * fc) / n**3
    scale = np.abs(u).max()
    assert np.abs(np.fft.fft2(ra) - u[h, :, :]).max() < 1e-13 * scale
    assert np.abs(np.fft.fft2(rb) - u[:, h, :]).max() < 1e-13 * scale
    assert np.abs(np.fft.fft2(rc) - u[:, :, h]).max() < 1e-13 * scale


def test_nyquist_correction_as_quadratic_form():
    """3. summed over the antipodal pairs, the correction is a quadratic form in
    f^ with REAL kernels that depend on the tables only (what the default
    correction, nyq_quad.cu, evaluates):
      sum_p C_p(k) = sum_q A(k, q) f^(q) f^(k - q) - B(k, q) conj f^(q) f^(k + q),
      A(k, q) = sum_p (w.x - w.y)_p(k) t-_p(q),  B(k, q) = sum_p (w.x + w.y)_p(k) t-_p(q),
    with k, q over the Nyquist points (t-_p carries the inverse transform's 1/N)."""
    n = 8
    mesh = fo.Mesh(n, L8_S, 3, 6)
    op = fo.FSInelasticVHS(mesh, 0.8, 0.8, 1.0)
    f = np.random.default_rng(1).uniform(0.1, 1.0, (n, n, n))
    fh = _fft3(f)
    pts = np.argwhere(_nyquist_mask(n))
    idx = tuple(pts.T)
    ctot = np.zeros((n, n, n), complex)
    A = np.zeros((len(pts), len(pts)))
    B = np.zeros_like(A)
    for ir in range(mesh.nr):
        gain, expt = op.tables_r(ir)
        for p, _ in _antipodes(mesh.sigma):
            ep, gp = _herm(expt[p]), _herm(gain[p])
            em, gm = expt[p] - ep, gain[p] - gp
            tm = em.real + em.imag
            u = _fft3(_ifft3(fh * tm) * f)
            ctot += (gm.real - gm.imag) * u - (gm.real + gm.imag) * np.conj(_reflect(u))
            tq = tm[idx] / n**3
            A += np.outer((gm.real - gm.imag)[idx], tq)
            B += np.outer((gm.real + gm.imag)[idx], tq)
    km = (pts[:, None, :] - pts[None, :, :]) % n
    kp = (pts[:, None, :] + pts[None, :, :]) % n
    fq = fh[idx][None, :]
    quad = (A * fq * fh[tuple(km.transpose(2, 0, 1))] - B * np.conj(fq) * fh[tuple(kp.transpose(2, 0, 1))]).sum(1)
    ref = ctot[idx]
    assert np.abs(quad - ref).max() < 1e-13 * np.abs(ref).max()
