"""FP64 restatement of the explicit / projective / telescopic steps (oracle).

Test infrastructure, not product code.  ``df`` is any callable
``df(f, dt) -> increment``; the step functions update ``f`` in place exactly
as ``BoltzmannSolver`` does (``src/boltzmann.py:82-84,120-158``):

* Euler:  ``f += df(dt)``
* PFE:    ``M = dt/dt0 - K0``; K0 x { d = df(dt0); f += d }; ``f += M d``
* TPI2/3: the same nesting over 2 / 3 levels with
  ``M_l = dt_{l+1}/dt_l - K_l`` and ``d_{l+1} = M_l d_l``.
"""
import numpy as np


def boltzmann_df(f, dt, collision, kn, advection=None):
    """``BoltzmannSolver.df`` (``src/boltzmann.py:160-164``)."""
    d = advection(f, dt) if advection is not None else np.zeros_like(f)
    if collision is not None:
        d = d + dt * collision(f) / kn
    return d


def euler_step(f, dt, df):
    f += df(f, dt)  # :82-84


def proj_euler_step(f, dt, df, inner_steps, inner_dt):
    M = dt / inner_dt[0] - inner_steps[0]  # :120-128
    for _ in range(inner_steps[0]):
        d = df(f, inner_dt[0])
        f += d
    f += M * d


def tel_proj_step2(f, dt, df, inner_steps, inner_dt):
    M1 = dt / inner_dt[1] - inner_steps[1]  # :130-140
    for _ in range(inner_steps[1]):
        M0 = inner_dt[1] / inner_dt[0] - inner_steps[0]
        for _ in range(inner_steps[0]):
            d0 = df(f, inner_dt[0])
            f += d0
        d1 = M0 * d0
        f += d1
    f += M1 * d1


def tel_proj_step3(f, dt, df, inner_steps, inner_dt):
    M2 = dt / inner_dt[2] - inner_steps[2]  # :142-158
    for _ in range(inner_steps[2]):
        M1 = inner_dt[2] / inner_dt[1] - inner_steps[1]
        for _ in range(inner_steps[1]):
            M0 = inner_dt[1] / inner_dt[0] - inner_steps[0]
            for _ in range(inner_steps[0]):
                d0 = df(f, inner_dt[0])
                f += d0
            d1 = M0 * d0
            f += d1
        d2 = M1 * d1
        f += d2
    f += M2 * d2


def convex_splitting_step(f, dt, collision, kn, penalty, advection=None):
    """CONSP (src/boltzmann.py:86-94): collision update, then transport of the updated f."""
    f += dt / (kn + penalty * dt) * collision(f)
    if advection is not None:
        f += advection(f, dt)


def convex_splitting_maxwellian_step(f, dt, collision, kn, penalty, e, tau, v, delta, advection=None):
    """CONSP_M (src/boltzmann.py:96-118) in 3D velocity.

    The reference writes it for 2D velocity only; this restatement uses the 3D
    Maxwellian with bulk velocity (u1, 0, 0) and the 3D temperature, the same
    cooling law T_new = (T - 8 tau/(1-e^2)) exp(-(1-e^2) rho dt / (4 kn)) + 8 tau/(1-e^2).
    """
    mo = moments(f, v, delta)
    rho, u1, T = mo["rho"], mo["u"][..., 0], mo["T"]
    T_new = (T - 8 * tau / (1 - e**2)) * np.exp(-(1 - e**2) / kn / 4 * rho * dt) + 8 * tau / (1 - e**2)
    V = np.meshgrid(v, v, v, indexing="ij")

    def maxw(T_):
        sh = (slice(None),) + (None,) * 3 if np.ndim(rho) else ()
        r, uu, tt = (np.asarray(x)[sh] for x in (rho, u1, T_))
        return r / (2 * np.pi * tt) ** 1.5 * np.exp(-((V[0] - uu) ** 2 + V[1] ** 2 + V[2] ** 2) / (2 * tt))

    dm = maxw(T_new) - maxw(T)
    f += dt / (kn + penalty * dt) * collision(f) + penalty * dt / (kn + penalty * dt) * dm
    if advection is not None:
        f += advection(f, dt)


def maxwellian_2d(vx, vy, rho, u, T):
    """``maxwellian`` of the reference solver (``src/boltzmann.py:9-13``): 2D
    velocity, bulk velocity (u, 0); rho, u, T per cell."""
    rho = np.asarray(rho)[:, None, None]
    u = np.asarray(u)[:, None, None]
    T = np.asarray(T)[:, None, None]
    return rho / (2 * np.pi * T) * np.exp(-((vx - u) ** 2 + vy**2) / (2 * T))


def convex_splitting_maxwellian_step_2d(f, dt, collision, kn, penalty, e, tau, v, delta, advection=None):
    """CONSP_M exactly as the reference writes it for 2D velocity
    (``src/boltzmann.py:96-118``), with the 2D moments of ``State``
    (``src/state.py:31-52,91-92``)."""
    mo = moments(f, v, delta, dim=2)
    rho, u, T = mo["rho"], mo["u"][..., 0], mo["T"]
    vx, vy = np.meshgrid(v, v, indexing="ij")
    T_new = (T - 8 * tau / (1 - e**2)) * np.exp(-(1 - e**2) / kn / 4 * rho * dt) + 8 * tau / (1 - e**2)
    dm = maxwellian_2d(vx, vy, rho, u, T_new) - maxwellian_2d(vx, vy, rho, u, T)
    f += dt / (kn + penalty * dt) * collision(f) + penalty * dt / (kn + penalty * dt) * dm
    if advection is not None:
        f += advection(f, dt)


def fast_sweep_step(f, v1, dx, kn, collision, delta, dim):
    """One ``BoltzmannFastSweep.step`` (``src/iter_solver.py:38-62``): the
    collision term and the density of the current state, then a Gauss-Seidel
    upwind sweep in x for v1 > 0 (left to right) and v1 < 0 (right to left) over
    the interior cells; returns max |f_new - f_old|.  The reference writes it
    for 2D velocity; with ``dim = 3`` the same sweep runs over the other two
    velocity axes."""
    f_old = f.copy()
    nx = f.shape[0]
    v = np.asarray(v1, np.float64)
    vdx = v / dx
    nu = 1 / np.sqrt(np.pi / 2) / kn
    rho = moments(f, v, delta, dim=dim)["rho"]
    rho = rho.reshape((nx,) + (1,) * dim)
    gain = collision(f)
    pos, neg = v > 0, v < 0
    ext = (slice(None),) + (None,) * (dim - 1)
    for i in range(1, nx - 1):
        f[i, pos] = (nu * gain[i, pos] + vdx[pos][ext] * f[i - 1, pos]) / (nu * rho[i] + vdx[pos][ext])
    for j in range(1, nx - 1):
        f[-j - 1, neg] = (nu * gain[-j - 1, neg] - vdx[neg][ext] * f[-j, neg]) / (nu * rho[-j - 1] - vdx[neg][ext])
    return np.max(np.abs(f - f_old))


STEPS = {
    "Euler": lambda f, dt, df, K, h: euler_step(f, dt, df),
    "PFE": proj_euler_step,
    "TPI2": tel_proj_step2,
    "TPI3": tel_proj_step3,
}


def evolve(f, t0, tend, dt, df, integrator="Euler", inner_steps=(3, 3, 3), inner_dt=None):
    """``Solver.evolve_to_time`` with fixed ``dt`` (``src/solver.py:107-143``)."""
    max_steps = int((tend - t0 + 1e-10) / dt)
    if abs(max_steps * dt - (tend - t0)) > 1e-5 * (tend - t0):
        raise Exception("dt does not divide (tend-tstart) and dt is fixed!")
    step = STEPS[integrator]
    for _ in range(max_steps):
        step(f, dt, df, inner_steps, inner_dt)
    return f


def moments(f, v, delta, dim=3):
    """FP64 density, bulk velocity, energy density and temperature per cell.

    ``dim = 2`` is the reference's ``State.rho/u/T`` (``src/state.py:31-52,91-92``):
    sums over the two velocity axes times delta^2, ``T = E / rho - |u|^2 / 2``.
    ``dim = 3`` is the 3D-velocity form: ``rho = sum f dv``,
    ``u = sum f v dv / rho``, ``E = 1/2 sum f |v|^2 dv`` and
    ``T = (2/3) (E / rho - |u|^2 / 2)``.
    """
    f = np.asarray(f, np.float64)
    V = np.meshgrid(*([v] * dim), indexing="ij")
    ax = tuple(range(-dim, 0))
    dv = delta**dim
    rho = f.sum(axis=ax) * dv
    mom = np.stack([(f * V[d]).sum(axis=ax) * dv for d in range(dim)], axis=-1)
    E = 0.5 * (f * sum(V[d] ** 2 for d in range(dim))).sum(axis=ax) * dv
    u = mom / rho[..., None]
    T = (2.0 / dim) * (E / rho - 0.5 * (u**2).sum(-1))
    return {"rho": rho, "u": u, "E": E, "T": T}
