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


def moments(f, v, delta):
    """FP64 density, bulk velocity (3), energy density and temperature per cell.

    The reference's ``State.rho/u/T`` reduce over two velocity axes only
    (``src/state.py:31-52,91-92``); this is the 3D-velocity form:
    ``rho = sum f dv``, ``u = sum f v dv / rho``, ``E = 1/2 sum f |v|^2 dv`` and
    ``T = (2/3) (E / rho - |u|^2 / 2)``.
    """
    f = np.asarray(f, np.float64)
    V = np.meshgrid(v, v, v, indexing="ij")
    dv = delta**3
    rho = f.sum(axis=(-3, -2, -1)) * dv
    mom = np.stack([(f * V[d]).sum(axis=(-3, -2, -1)) * dv for d in range(3)], axis=-1)
    E = 0.5 * (f * (V[0] ** 2 + V[1] ** 2 + V[2] ** 2)).sum(axis=(-3, -2, -1)) * dv
    u = mom / rho[..., None]
    T = (2.0 / 3.0) * (E / rho - 0.5 * (u**2).sum(-1))
    return {"rho": rho, "u": u, "E": E, "T": T}
