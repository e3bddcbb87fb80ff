"""FP64 NumPy restatement of the 1D-space transport step (oracle, test infrastructure).

Second-order wave-propagation upwind flux in x with a minmod-limited
correction and two ghost cells, as in

* ``BoltzmannSolver1D.df_advection`` (``src/boltzmann.py:177-205``),
* ``Solver._apply_bcs / _bc_lower / _bc_upper`` (``src/solver.py:59-105``),
* ``advection_1D`` (``src/riemann/advection_1D.py:4-21``),
* ``tvd.limit`` / ``tvd.minmod`` (``src/limiters/tvd.py:6-40``).

The state is ``f`` with shape ``(n_x, n, n, n)`` (3D velocity) or
``(n_x, n, n)`` (2D velocity); the advection speed is the first velocity
coordinate ``v1`` (``src/solution.py:55``), broadcast over the other velocity
axes.

The reference slices the speed array as ``s[LL-1:UL-1]`` on its *velocity*
axis (``src/boltzmann.py:200``); that slice is the whole array whenever
``n_x + 2 >= n`` and otherwise fails to broadcast.  This restatement uses the
intended whole-array ``|s|`` (identical in every case the reference runs).
"""
import numpy as np

EXTRAP = "extrap"
PERIODIC = "periodic"
NUM_GHOST = 2


def ghosted(f, bc_lower=EXTRAP, bc_upper=EXTRAP, ng=NUM_GHOST):
    """``fbc`` with ghost cells filled (``src/solver.py:59-105``, ``src/state.py:109-122``)."""
    f = np.asarray(f, np.float64)
    fbc = np.zeros((f.shape[0] + 2 * ng,) + f.shape[1:])
    fbc[ng:-ng] = f
    if bc_lower == EXTRAP:
        for i in range(ng):
            fbc[i] = fbc[ng]
    elif bc_lower == PERIODIC:
        fbc[:ng] = fbc[-2 * ng : -ng]
    else:
        raise NotImplementedError(f"Boundary condition {bc_lower} not implemented")
    if bc_upper == EXTRAP:
        for i in range(ng):
            fbc[-i - 1] = fbc[-ng - 1]
    elif bc_upper == PERIODIC:
        fbc[-ng:] = fbc[ng : 2 * ng]
    else:
        raise NotImplementedError(f"Boundary condition {bc_upper} not implemented")
    return fbc


def minmod(r, cfl):
    """``tvd.minmod`` (``src/limiters/tvd.py:30-40``): max(0, min(1, r))."""
    a = np.ones((2,) + r.shape)
    b = np.zeros((2,) + r.shape)
    a[1, :] = r
    b[1, :] = np.minimum(a[0], a[1])
    return np.maximum(b[0], b[1])


def limit(wave, s, dtdx, limiter=minmod):
    """``tvd.limit`` (``src/limiters/tvd.py:6-27``), masked division kept."""
    wave = wave.copy()
    wave_norm2 = wave**2
    wave_zero_mask = np.array((wave == 0), dtype=float)
    wave_nonzero_mask = 1.0 - wave_zero_mask
    dotls = wave[1:] * wave[:-1]
    spos = np.array(s > 0.0, dtype=float)
    r = np.ma.array(spos * dotls[:-1] + (1 - spos) * dotls[1:])
    r /= np.ma.array(wave_norm2[1:-1])
    r.fill_value = 0
    r = r.filled()
    cfl = np.abs(s * dtdx)
    wlimitr = limiter(r, cfl)
    wave[1:-1] = wave[1:-1] * wave_zero_mask[1:-1] + wlimitr * wave[1:-1] * wave_nonzero_mask[1:-1]
    return wave


def df_advection(f, v1, dt, dx, bc_lower=EXTRAP, bc_upper=EXTRAP, order=2):
    """Transport increment for one step of size ``dt`` (``src/boltzmann.py:177-205``).

    ``v1`` is the 1D array of first-axis velocity centres (length n).
    """
    f = np.asarray(f, np.float64)
    n = f.shape[1]
    vv = np.asarray(v1, np.float64).reshape((n,) + (1,) * (f.ndim - 2))
    s = np.broadcast_to(vv, (n,) + f.shape[2:]).copy()
    fb = ghosted(f, bc_lower, bc_upper)
    dtdx = dt / dx
    df = np.zeros(fb.shape)
    wave = fb[1:] - fb[:-1]  # advection_1D.py:16
    apdf = np.maximum(s, 0.0) * wave
    amdf = np.minimum(s, 0.0) * wave
    nx = f.shape[0]
    LL = NUM_GHOST - 1
    UL = nx + NUM_GHOST + 1
    df[LL:UL] = -dtdx * (amdf[LL:UL] + apdf[LL - 1 : UL - 1])  # :194
    if order == 2:
        F = np.zeros(fb.shape)
        wave = limit(wave, s, dtdx)
        sabs = np.abs(s)
        om = 1.0 - sabs * dtdx
        F[LL:UL] = 0.5 * sabs * om * wave[LL - 1 : UL - 1]  # :202
        df[LL : UL - 1] -= dtdx * (F[LL + 1 : UL] - F[LL : UL - 1])  # :203
    return df[NUM_GHOST:-NUM_GHOST]
