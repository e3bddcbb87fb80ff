"""Time integrators with the reference's solver interface, stepping on the GPU.

* ``BC``, ``Solver``, ``BoltzmannSolver``, ``BoltzmannSolver1D`` keep the
  attributes and methods of src/solver.py:1-146 and src/boltzmann.py:16-205
  (``kn``, ``dt``, ``time_integrator`` in {"Euler", "PFE", "TPI2", "TPI3",
  "CONSP", "CONSP_M"}, ``inner_steps``, ``inner_dt``, ``bc_lower`` /
  ``bc_upper`` / ``all_bcs``, ``step`` and the per-integrator ``euler_step``,
  ``proj_euler_step``, ``tel_proj_step2``, ``tel_proj_step3``,
  ``convex_splitting_step``, ``convex_splitting_maxwellian_step``, ``df``,
  ``df_advection``, ``evolve_to_time``), and ``maxwellian`` of
  src/boltzmann.py:9-13.
* ``State`` / ``Solution`` hold f as a torch CUDA FP64 tensor of shape
  (n_x, n, n, n) or (n_x, n, n) (3D or 2D velocity; no n_x for a
  space-homogeneous problem), with FP64 moments ``rho``, ``u``, ``T``, the
  reference's helpers and ``state.grid`` (``Grid``: per-axis cells, centres,
  nodes, ``c_centers``) (src/state.py, src/solution.py, src/geometry.py).
* ``IterativeBoltzmannSolver`` keeps ``solve`` / ``step``
  (src/iter_solver.py:9-35); ``BoltzmannFastSweep`` is its Gauss-Seidel
  upwind sweep (src/iter_solver.py:38-62) on the GPU.

With the GB300 ``FSInelasticVHSCollision`` as the collision operator, a whole
macro-step (all inner steps, transport, FP64 extrapolations) runs as one
``pii_step`` call, captured into a CUDA graph on first use.  Any other
collision callable is stepped by the same nesting in Python, with the
transport and FP64 updates still on the GPU.
"""
import logging
import math

import numpy as np
import torch

from . import _lib
from .collision import FSInelasticVHSCollision

_INTEGRATORS = {"Euler": _lib.INT_EULER, "PFE": _lib.INT_PFE, "TPI2": _lib.INT_TPI2, "TPI3": _lib.INT_TPI3}
_LEVELS = {"Euler": 0, "PFE": 1, "TPI2": 2, "TPI3": 3}
_METHODS = {"Euler": "euler_step", "PFE": "proj_euler_step", "TPI2": "tel_proj_step2", "TPI3": "tel_proj_step3",
            "CONSP": "convex_splitting_step", "CONSP_M": "convex_splitting_maxwellian_step"}


def maxwellian(vx, vy, rho, u, T):
    """The reference solver's ``maxwellian`` (src/boltzmann.py:9-13): the 2D
    Maxwellian with bulk velocity (u, 0) for per-cell rho, u, T on the velocity
    coordinates vx, vy (e.g. ``state.c_centers[1:]``); NumPy, or torch tensors."""
    rho = rho[:, None, None]
    u = u[:, None, None]
    T = T[:, None, None]
    exp = torch.exp if isinstance(vx, torch.Tensor) else np.exp
    return rho / (2 * math.pi * T) * exp(-((vx - u) ** 2 + vy**2) / (2 * T))


class BC:
    extrap = _lib.BC_EXTRAP
    periodic = _lib.BC_PERIODIC


class Grid:
    """The state's grid (src/geometry.py:45-172, one ``Dimension`` per axis, x
    axes first, then velocity): per-axis ``num_cells``, ``lower``, ``upper``,
    ``delta``, ``centers``, ``nodes`` (lists over the axes), ``num_dim``,
    ``num_dim_x``, and ``c_centers`` / ``c_nodes``, the per-axis coordinates
    broadcast over the whole grid (host NumPy, built on first use as the
    reference does)."""

    def __init__(self, num_cells, lower, upper, num_dim_x):
        self.num_cells = [int(n) for n in num_cells]
        self.lower = [float(x) for x in lower]
        self.upper = [float(x) for x in upper]
        self.num_dim_x = int(num_dim_x)
        # Dimension.delta / centers / nodes (src/geometry.py:176-194)
        self.delta = [(u - lo) / float(n) for lo, u, n in zip(self.lower, self.upper, self.num_cells)]
        self._c_centers = None
        self._c_nodes = None

    @property
    def num_dim(self):
        return len(self.num_cells)

    @property
    def centers(self):
        return [np.array([lo + (i + 0.5) * d for i in range(n)])
                for lo, d, n in zip(self.lower, self.delta, self.num_cells)]

    @property
    def nodes(self):
        return [np.array([lo + i * d for i in range(n + 1)]) for lo, d, n in zip(self.lower, self.delta, self.num_cells)]

    @property
    def c_centers(self):
        if self._c_centers is None:
            self._c_centers = list(np.meshgrid(*self.centers, indexing="ij"))
        return self._c_centers

    @property
    def c_nodes(self):
        if self._c_nodes is None:
            self._c_nodes = list(np.meshgrid(*self.nodes, indexing="ij"))
        return self._c_nodes


class State:
    """Phase-space state: f on the GPU, FP64 (src/state.py:6-122).  Grid
    attributes (``num_cells``, ``lower``, ``upper``, ``delta``, ``centers``,
    ``nodes``, ``c_centers``, ``c_nodes``, ``num_dim``, ``num_dim_x``) are read
    from ``state.grid`` as in the reference (src/state.py:10-29)."""

    _GRID_KEYS = ("num_dim", "num_dim_x", "c_centers", "c_nodes", "num_cells", "lower", "upper", "delta", "centers",
                  "nodes")

    def __init__(self, num_cells, lower, upper, num_dim_x, device=0):
        self.grid = Grid(num_cells, lower, upper, num_dim_x)
        self.device = int(device)
        self.t = 0.0
        self.problem_data = {}
        self.f = self.new_array().zero_()

    def __getattr__(self, key):
        grid = self.__dict__.get("grid")
        if grid is not None and key in State._GRID_KEYS:
            return getattr(grid, key)
        raise AttributeError(f"'State' object has no attribute '{key}'")

    def new_array(self):
        """An uninitialised f of the grid's shape (src/state.py:66-69): FP64 on the state's GPU."""
        return torch.empty(self.grid.num_cells, dtype=torch.float64, device=f"cuda:{self.device}")

    def get_f_global(self):
        """A copy of f (src/state.py:88-89)."""
        return self.f.clone()

    def sum_f(self, f):
        """Velocity integral per cell (src/state.py:91-92, written there for 2D
        velocity): the sum over the dim_v velocity axes times the cell volume.
        Torch in -> torch out, NumPy in -> NumPy out."""
        d = self.dim_v
        axes = tuple(range(-d, 0))
        vol = 1.0
        for dv in self.grid.delta[-d:]:
            vol *= dv
        if isinstance(f, torch.Tensor):
            return f.sum(dim=axes) * vol
        return np.sum(f, axis=axes) * vol

    def set_f_from_fbc(self, num_ghost, fbc):
        """f = the interior of the ghosted array fbc (src/state.py:94-107)."""
        if self.grid.num_dim_x == 1:
            self.f = fbc[num_ghost:-num_ghost]
        elif self.grid.num_dim_x == 2:
            self.f = fbc[num_ghost:-num_ghost, num_ghost:-num_ghost]
        else:
            raise Exception("Assumption (1 <= num_dim_x <= 2) violated.")

    def get_fbc_from_f(self, num_ghost, fbc):
        """Copy f into the interior of fbc (src/state.py:109-120)."""
        if self.grid.num_dim_x == 1:
            fbc[num_ghost:-num_ghost] = self.f
        elif self.grid.num_dim_x == 2:
            fbc[num_ghost:-num_ghost, num_ghost:-num_ghost] = self.f
        else:
            raise Exception("Assumption (1 <= num_dim <= 2) violated.")

    def __copy__(self):
        new = State.__new__(State)
        new.__dict__.update(self.__dict__)
        return new

    def __deepcopy__(self, memo):
        """A new state with copies of the grid, t, problem_data and f (src/state.py:74-86)."""
        import copy

        new = State.__new__(State)
        new.grid = copy.deepcopy(self.grid, memo)
        new.device = self.device
        new.t = self.t
        new.problem_data = copy.deepcopy(self.problem_data, memo)
        new.f = self.f.clone()
        return new

    @property
    def dim_v(self):
        return self.grid.num_dim - self.grid.num_dim_x

    @property
    def v(self):
        """Velocity centres (same on every velocity axis)."""
        return self.grid.centers[self.grid.num_dim_x]

    @property
    def v1(self):
        return self.v

    @property
    def dv(self):
        return self.grid.delta[self.grid.num_dim_x]

    def moments(self):
        """FP64 (rho, u[dim], T) per cell from ``pii_moments``: State.rho / u / T
        (src/state.py:31-52; T = E / rho - |u|^2 / 2 in 2D, (2/3)(E / rho -
        |u|^2 / 2) in 3D)."""
        f = self.f
        d = self.dim_v
        n = f.shape[-1]
        cells = f.numel() // (n**d)
        out = torch.empty((cells, 5), dtype=torch.float64, device=f.device)
        plan = _moment_plan(n, f.device.index or 0, d, cells)
        v = np.ascontiguousarray(self.v, np.float64)
        st = plan._lib.pii_moments(plan.handle, f.contiguous().data_ptr(), out.data_ptr(), cells, _lib.dptr(v),
                                   float(self.dv), torch.cuda.current_stream().cuda_stream)
        _lib.check(st, "pii_moments")
        return _split_moments(out.cpu().numpy(), d, f.shape[:-d])

    @property
    def rho(self):
        return self.moments()[0]

    @property
    def u(self):
        return self.moments()[1]

    @property
    def T(self):
        return self.moments()[2]


def _split_moments(m, d, shape):
    """(rho, u, T) from the per-cell sums [rho, m1, m2, m3, E] of pii_moments."""
    rho = m[:, 0]
    u = m[:, 1 : 1 + d] / rho[:, None]
    T = (2.0 / d) * (m[:, 4] / rho - 0.5 * (u**2).sum(-1))
    return rho.reshape(shape), u.reshape(tuple(shape) + (d,)), T.reshape(shape)


_MPLANS = {}


def _moment_plan(n, device, dim=3, cells=1):
    """A minimal plan used only for its moment / velocity / transport buffers."""
    key = (n, device, dim)
    if key in _MPLANS and _MPLANS[key].batch_max < cells:
        _MPLANS.pop(key).close()
    if key not in _MPLANS:
        from .collision import Plan

        class _Mesh:
            nv = n
            ndim = dim
            L = 1.0
            R = 1.0

            @staticmethod
            def rquad():
                return np.array([0.5]), np.array([1.0])

            @staticmethod
            def circ_or_sphr_quad():
                return (np.array([[0.0, 0.0, 1.0]]), 4 * math.pi) if dim == 3 else (np.array([[1.0, 0.0]]),
                                                                                     2 * math.pi)

        _MPLANS[key] = Plan(_Mesh, 1.0, 1.0, 0.0, _lib.PREC_FP64, max(1, int(cells)), device)
    return _MPLANS[key]


class Solution:
    """``Solution(config)`` (src/solution.py:47-57): config has dim_x, dim_v,
    xmin, xmax, l, nx, nv (attribute or key access).  dim_x = 0 gives a
    space-homogeneous state f of shape (nv, nv, nv)."""

    def __init__(self, config, device=0):
        get = (lambda k: config[k]) if isinstance(config, dict) else (lambda k: getattr(config, k))
        dim_x, dim_v = int(get("dim_x")), int(get("dim_v"))
        if dim_v not in (2, 3):
            raise ValueError("Dimension must be 2 or 3.")
        lower, upper, nn = [], [], []
        if dim_x:
            lower += [float(get("xmin"))] * dim_x
            upper += [float(get("xmax"))] * dim_x
            nn += [int(get("nx"))] * dim_x
        lower += [-float(get("l"))] * dim_v
        upper += [float(get("l"))] * dim_v
        nn += [int(get("nv"))] * dim_v
        self.state = State(nn, lower, upper, dim_x, device)
        self.state.problem_data = {"v1": self.state.v}

    @property
    def t(self):
        return self.state.t

    @t.setter
    def t(self, value):
        self.state.t = value

    @property
    def f(self):
        return self.state.f

    @property
    def grid(self):
        return self.state.grid

    def set_all_states(self, attr, value, overwrite=True):
        """src/solution.py:36-38."""
        if getattr(self.state, attr) is None or overwrite:
            setattr(self.state, attr, value)

    def __getattr__(self, key):
        if key in ("rho", "u", "T", "num_dim", "num_dim_x", "c_nodes", "c_centers", "num_cells", "lower", "upper",
                   "delta", "centers", "nodes", "v", "dim_v", "problem_data"):
            state = self.__dict__.get("state")
            if state is not None:
                return getattr(state, key)
        raise AttributeError(f"'Solution' object has no attribute '{key}'")


class Solver:
    """``Solver`` (src/solver.py:13-146)."""

    num_dim_x = 1

    @property
    def all_bcs(self):
        return self.bc_lower, self.bc_upper

    @all_bcs.setter
    def all_bcs(self, all_bcs):
        for i in range(self.num_dim_x):
            self.bc_lower[i] = all_bcs
            self.bc_upper[i] = all_bcs

    def __init__(self, riemann_solver=None, collision_operator=None):
        self.dt_initial = 0.01
        self.dt_max = 1e99
        self.max_steps = 10000
        self.dt_variable = False
        self.rp = riemann_solver
        self.collision = collision_operator
        self.before_step = None
        self.dt = self.dt_initial
        self.bc_lower = [None] * max(self.num_dim_x, 1)
        self.bc_upper = [None] * max(self.num_dim_x, 1)
        self._is_set_up = False

    def setup(self, solution):
        self._is_set_up = True

    def evolve_to_time(self, solution, tend=None):
        """src/solver.py:107-143."""
        if not self._is_set_up:
            self.setup(solution)
        take_one_step = tend is None
        tstart = solution.t
        if not self.dt_variable:
            if take_one_step:
                self.max_steps = 1
            else:
                self.max_steps = int((tend - tstart + 1e-10) / self.dt)
                if abs(self.max_steps * self.dt - (tend - tstart)) > 1e-5 * (tend - tstart):
                    raise Exception("dt does not divide (tend-tstart) and dt is fixed!")
        for n in range(self.max_steps):
            if self.before_step is not None:
                self.before_step(self, solution.state)
            self.step(solution, take_one_step, tstart, tend)
            solution.t = tstart + (n + 1) * self.dt

    def step(self, solution, take_one_step, tstart, tend):
        raise NotImplementedError("No stepping routine has been defined!")


class BoltzmannSolver(Solver):
    """``BoltzmannSolver`` (src/boltzmann.py:16-167) on the GPU.

    Extra attributes: ``with_loss`` (None: use the operator's own default,
    i.e. gain only as the reference solver does), ``mass_fix`` (FP64 k = 0
    correction of Q) and ``use_graph`` (capture each macro-step as a CUDA graph).
    """

    num_dim_x = 0

    def __init__(self, kn=1.0, riemann_solver=None, collision_operator=None):
        self.kn = kn
        self.tau = None
        self.e = None
        self.num_ghost = 2
        self.order = 2
        self.limiters = "minmod"
        self.time_integrator = "Euler"
        self.penalty = None
        self.num_levels = 3
        self.inner_steps = [3, 3, 3]
        self.inner_dt = [kn, 5 * kn, 10 * kn]
        self.with_loss = None
        self.mass_fix = None
        self.use_graph = True
        self.check_every = 0
        self.mass_drift_tol = None
        self._mass0 = None
        self._stream = None
        super().__init__(riemann_solver, collision_operator)

    # -- helpers -----------------------------------------------------------
    def _transport_args(self, state):
        """(nx, dx, v1, bc_lo, bc_hi); dx = 0 disables transport."""
        f = state.f
        n = f.shape[-1]
        cells = f.numel() // n**state.dim_v
        return cells, 0.0, np.ascontiguousarray(state.v, np.float64), _lib.BC_EXTRAP, _lib.BC_EXTRAP


    def _wl(self):
        if self.with_loss is not None:
            return bool(self.with_loss)
        return bool(getattr(self.collision, "default_with_loss", False))

    def _mf(self):
        if self.mass_fix is not None:
            return bool(self.mass_fix)
        return bool(getattr(self.collision, "mass_fix", False))

    def _get_stream(self, device):
        if self._stream is None:
            self._stream = torch.cuda.Stream(device=device)
        return self._stream

    # -- stepping ----------------------------------------------------------
    def step(self, solution, take_one_step, tstart, tend):
        """``BoltzmannSolver.step`` (src/boltzmann.py:46-80)."""
        ti = self.time_integrator
        state = solution.state
        if ti == "CONSP":
            if not self.penalty:
                raise ValueError("The penalty parameter is not given. Please specify it!")
        elif ti == "CONSP_M":
            if not (self.penalty and self.e and (self.tau is not None)):
                raise ValueError("The penalty parameter, e or tau are not given. Please specify it!")
        elif ti not in _INTEGRATORS:
            raise NotImplementedError("This time integrator is not implemented.")
        getattr(self, _METHODS[ti])(solution, take_one_step, tstart, tend)
        self._steps_done = getattr(self, "_steps_done", 0) + 1
        if self.check_every and self._steps_done % self.check_every == 0:
            self.check_state(state)

    # the reference's per-integrator steps (src/boltzmann.py:82-158), each one
    # macro-step of self.dt whatever self.time_integrator names
    def euler_step(self, solution, take_one_step, tstart, tend):
        """f += df(dt) (src/boltzmann.py:82-84)."""
        self._integrate(solution.state, "Euler")

    def convex_splitting_step(self, solution, take_one_step, tstart, tend):
        """f += dt / (kn + P dt) Q(f), then f += transport(f, dt) (src/boltzmann.py:86-94)."""
        self._integrate(solution.state, "CONSP")

    def convex_splitting_maxwellian_step(self, solution, take_one_step, tstart, tend):
        """CONSP plus the penalised Maxwellian relaxation term (src/boltzmann.py:96-118)."""
        self._integrate(solution.state, "CONSP_M")

    def proj_euler_step(self, solution, take_one_step, tstart, tend):
        """K inner Euler steps of inner_dt[0], then f += (dt / inner_dt[0] - K) df (src/boltzmann.py:120-128)."""
        self._integrate(solution.state, "PFE")

    def tel_proj_step2(self, solution, take_one_step, tstart, tend):
        """Two-level telescopic projective step (src/boltzmann.py:130-140)."""
        self._integrate(solution.state, "TPI2")

    def tel_proj_step3(self, solution, take_one_step, tstart, tend):
        """Three-level telescopic projective step (src/boltzmann.py:142-158)."""
        self._integrate(solution.state, "TPI3")

    def _integrate(self, state, ti):
        if isinstance(self.collision, FSInelasticVHSCollision):
            if ti in ("CONSP", "CONSP_M"):
                self._fused_splitting(state, ti)
            else:
                self._fused_step(state, ti)
        else:
            if ti == "CONSP_M":
                raise NotImplementedError("CONSP_M needs the GB300 collision operator")
            self._generic_step(state, ti)

    def check_state(self, state):
        """FP64 guard: raise FloatingPointError if f holds NaN / Inf, and
        RuntimeError if the total mass drifted by more than ``mass_drift_tol``
        (relative) since the first check.  Returns (rho, u, T) per cell."""
        f = state.f
        n = f.shape[-1]
        d = state.dim_v
        cells = f.numel() // n**d
        out = torch.empty((cells, 5), dtype=torch.float64, device=f.device)
        plan = _moment_plan(n, f.device.index or 0, d, cells)
        v = np.ascontiguousarray(state.v, np.float64)
        st = plan._lib.pii_state_check(plan.handle, f.contiguous().data_ptr(), out.data_ptr(), cells, _lib.dptr(v),
                                       float(state.dv), torch.cuda.current_stream(f.device).cuda_stream)
        _lib.check(st, "pii_state_check")
        m = out.cpu().numpy()
        mass = float(m[:, 0].sum())
        if self._mass0 is None:
            self._mass0 = mass
        elif self.mass_drift_tol is not None and abs(mass - self._mass0) > self.mass_drift_tol * abs(self._mass0):
            raise RuntimeError(f"total mass drifted from {self._mass0:.12g} to {mass:.12g}")
        return _split_moments(m, d, (cells,))

    def _fused_splitting(self, state, ti):
        f = state.f
        if not (f.is_cuda and f.dtype == torch.float64 and f.is_contiguous()):
            raise ValueError("state.f must be a contiguous CUDA float64 tensor")
        nx, dx, v1, lo, hi = self._transport_args(state)
        plan = self.collision._ensure_plan(nx)
        cur = torch.cuda.current_stream(f.device)
        s = self._get_stream(f.device) if self.use_graph else cur
        if s is not cur:
            s.wait_stream(cur)
        code = _lib.INT_CONSP if ti == "CONSP" else _lib.INT_CONSP_M
        st = plan._lib.pii_step_splitting(plan.handle, code, f.data_ptr(), nx, float(self.dt), float(dx), _lib.dptr(v1),
                                          int(lo), int(hi), float(self.kn), float(self.penalty or 0.0),
                                          float(self.e or 0.0), float(self.tau or 0.0), int(self._wl()),
                                          int(self._mf()), int(bool(self.use_graph)), s.cuda_stream)
        _lib.check(st, "pii_step_splitting")
        if s is not cur:
            cur.wait_stream(s)

    def _fused_step(self, state, ti):
        f = state.f
        if not (f.is_cuda and f.dtype == torch.float64 and f.is_contiguous()):
            raise ValueError("state.f must be a contiguous CUDA float64 tensor")
        nx, dx, v1, lo, hi = self._transport_args(state)
        plan = self.collision._ensure_plan(nx)
        lev = _LEVELS[ti]
        K = np.ascontiguousarray(list(self.inner_steps[:lev]) + [0] * (3 - lev), np.int32)
        h = np.ascontiguousarray(list(self.inner_dt[:lev]) + [0.0] * (3 - lev), np.float64)
        cur = torch.cuda.current_stream(f.device)
        s = self._get_stream(f.device) if self.use_graph else cur
        if s is not cur:
            s.wait_stream(cur)
        st = plan._lib.pii_step(plan.handle, _INTEGRATORS[ti], f.data_ptr(), nx, float(self.dt), _lib.iptr(K),
                                _lib.dptr(h), max(lev, 1), float(dx), _lib.dptr(v1), int(lo), int(hi),
                                float(self.kn), int(self._wl()), int(self._mf()), int(bool(self.use_graph)),
                                s.cuda_stream)
        _lib.check(st, "pii_step")
        if s is not cur:
            cur.wait_stream(s)

    def _generic_step(self, state, ti):
        """Same nesting as src/boltzmann.py:82-158 for an arbitrary collision callable."""
        f = state.f
        dt, K, h = self.dt, self.inner_steps, self.inner_dt
        if ti == "CONSP":
            if self.collision is not None:
                f += dt / (self.kn + self.penalty * dt) * self._q(state)
            f += self.df_advection(state, dt)
        elif ti == "Euler":
            f += self.df(state, dt)
        elif ti == "PFE":
            M = dt / h[0] - K[0]
            for _ in range(K[0]):
                d = self.df(state, h[0])
                f += d
            f += M * d
        elif ti == "TPI2":
            M1 = dt / h[1] - K[1]
            for _ in range(K[1]):
                M0 = h[1] / h[0] - K[0]
                for _ in range(K[0]):
                    d0 = self.df(state, h[0])
                    f += d0
                d1 = M0 * d0
                f += d1
            f += M1 * d1
        else:
            M2 = dt / h[2] - K[2]
            for _ in range(K[2]):
                M1 = h[2] / h[1] - K[1]
                for _ in range(K[1]):
                    M0 = h[1] / h[0] - K[0]
                    for _ in range(K[0]):
                        d0 = self.df(state, h[0])
                        f += d0
                    d1 = M0 * d0
                    f += d1
                d2 = M1 * d1
                f += d2
            f += M2 * d2

    def _q(self, state):
        q = self.collision(state.f)
        if not isinstance(q, torch.Tensor):
            q = torch.as_tensor(q, device=state.f.device)
        return q

    def df(self, state, dt):
        """``BoltzmannSolver.df`` (src/boltzmann.py:160-164)."""
        deltaf = self.df_advection(state, dt)
        if self.collision is not None:
            deltaf += dt * self._q(state) / self.kn
        return deltaf

    def df_advection(self, state, dt):
        return torch.zeros_like(state.f)


class BoltzmannSolver0D(BoltzmannSolver):
    """Space-homogeneous solver: df = dt Q / kn (no transport)."""

    num_dim_x = 0


class BoltzmannSolver1D(BoltzmannSolver):
    """``BoltzmannSolver1D`` (src/boltzmann.py:170-205): transport in x with the
    second-order upwind + minmod TVD flux, two ghost cells."""

    num_dim_x = 1

    def __init__(self, kn=1, riemann_solver=None, collision_operator=None):
        super().__init__(kn, riemann_solver, collision_operator)

    def setup(self, solution):
        """Checks the boundary conditions as the reference's ghost fill does
        (src/solver.py:67-105: lower side first)."""
        for b, side in ((self.bc_lower[0], "Lower"), (self.bc_upper[0], "Upper")):
            if b is None:
                raise Exception(f"{side} boundary condition not specified.")
            if b not in (BC.extrap, BC.periodic):
                raise NotImplementedError("Boundary condition %s not implemented" % b)
        super().setup(solution)

    def _transport_args(self, state):
        f = state.f
        nx = f.shape[0]
        return (nx, float(state.delta[0]), np.ascontiguousarray(state.v, np.float64), int(self.bc_lower[0]),
                int(self.bc_upper[0]))

    def df_advection(self, state, dt):
        if not self._is_set_up:
            self.setup(None)
        f = state.f.contiguous()
        nx, dx, v1, lo, hi = self._transport_args(state)
        out = torch.empty_like(f)
        plan = _moment_plan(f.shape[-1], f.device.index or 0, state.dim_v, nx)
        st = plan._lib.pii_transport_df(plan.handle, f.data_ptr(), out.data_ptr(), nx, float(dt), dx, _lib.dptr(v1),
                                        lo, hi, torch.cuda.current_stream().cuda_stream)
        _lib.check(st, "pii_transport_df")
        return out


class IterativeBoltzmannSolver:
    """``IterativeBoltzmannSolver`` (src/iter_solver.py:9-35): ``solve`` loops
    ``step(state)`` until the returned error is below ``tol``."""

    def __init__(self, log_path=None, collision=None, kn=0.1, tol=1e-6):
        if log_path:
            logger = logging.getLogger()
            logger.setLevel(logging.INFO)
            if not logger.handlers:
                fh = logging.FileHandler(log_path)
                fh.setFormatter(logging.Formatter("%(asctime)s:%(levelname)s: %(message)s"))
                logger.addHandler(fh)
                sh = logging.StreamHandler()
                sh.setFormatter(logging.Formatter("%(message)s"))
                logger.addHandler(sh)
        self.collision = collision
        self.kn = kn
        self.tol = tol

    def solve(self, solution, n_iter=0, disp=False):
        err = 1
        num_steps = 1
        while err > self.tol:
            if n_iter and num_steps >= n_iter:
                return err, num_steps
            err = self.step(solution.state)
            num_steps += 1
            if disp and (num_steps % 1 == 0):
                logging.info("Current error: {}; Number of iterations: {}".format(err, num_steps))
        return err, num_steps

    def step(self, solution):
        raise NotImplementedError("No stepping routine has been defined!")


class BoltzmannFastSweep(IterativeBoltzmannSolver):
    """``BoltzmannFastSweep`` (src/iter_solver.py:38-62): one ``step(state)`` =
    the collision term and densities of the current state, then a Gauss-Seidel
    upwind sweep in x (v1 > 0 left to right, v1 < 0 right to left, interior
    cells) in FP64 on the GPU (``pii_fast_sweep``); returns max |f_new - f_old|.
    The reference writes it for 2D velocity; 3D states sweep the same way over
    (v2, v3)."""

    def step(self, state):
        f = state.f
        if not (f.is_cuda and f.dtype == torch.float64 and f.is_contiguous()):
            raise ValueError("state.f must be a contiguous CUDA float64 tensor")
        q = self.collision(f)
        if not isinstance(q, torch.Tensor):
            q = torch.as_tensor(q, device=f.device)
        q = q.to(torch.float64).contiguous()
        nx = f.shape[0]
        plan = _moment_plan(f.shape[-1], f.device.index or 0, state.dim_v, nx)
        v1 = np.ascontiguousarray(state.v, np.float64)
        err = _lib.ctypes.c_double()
        st = plan._lib.pii_fast_sweep(plan.handle, f.data_ptr(), q.data_ptr(), nx, float(state.delta[0]),
                                      float(self.kn), _lib.dptr(v1), _lib.ctypes.byref(err),
                                      torch.cuda.current_stream(f.device).cuda_stream)
        _lib.check(st, "pii_fast_sweep")
        return err.value
