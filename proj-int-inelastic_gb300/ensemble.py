"""Ensembles of independent space-homogeneous problems stepped as one graph.

Each instance has its own velocity grid (n may differ), restitution law and
state f of shape (n, n, n).  Instances that share everything but the
restitution law (n, L, the quadrature, gamma and the precision) form one size
class: their states are stacked into one (cells, n, n, n) array and one
operator plan evaluates Q(f,f) for all of them in one batched launch sequence,
with per-cell gain tables for the per-instance (e, e0)
(``pii_plan_set_restitution``).  The macro-steps of every class (Euler or
projective forward Euler, src/boltzmann.py:82-84,120-128, with df = dt Q(f) /
kn) are captured into one CUDA graph on the first call of
:meth:`Ensemble.step` and replayed as a single launch afterwards.

This generalises the reference's per-problem driver loop to a batch; the
reference has no ensemble driver of its own.
"""
import numpy as np
import torch

from . import _lib
from .collision import FSInelasticVHSCollision, SpectralMesh

_INT = {"Euler": _lib.INT_EULER, "PFE": _lib.INT_PFE}


def _class_key(config):
    """Everything that fixes a plan except the restitution law."""
    vm, sd, cm = config["velocity-mesh"], config["spherical-design-rule"], config["collision-model"]
    return (int(vm["nv"]), float(vm["s"]), int(vm.get("nr", int(vm["nv"]) // 2)), int(sd["nsphr"]),
            float(cm.get("gamma", 0.0)))


def _restitution(config):
    cm = config["collision-model"]
    return float(cm.get("e", 1.0)), float(cm.get("e0", 1.0))


class Ensemble:
    def __init__(self, configs, f0s, dt, kn=1.0, integrator="PFE", inner_steps=(2,), inner_dt=None,
                 precision="mixed", with_loss=True, mass_fix=False, device=0):
        if len(configs) != len(f0s):
            raise ValueError("one initial state per configuration")
        if integrator not in _INT:
            raise NotImplementedError("This time integrator is not implemented.")
        self.device = int(device)
        self.dt, self.kn = float(dt), float(kn)
        self.integrator = integrator
        self.K = np.ascontiguousarray(list(inner_steps) + [0, 0], np.int32)[:3]
        self.h = np.ascontiguousarray(list(inner_dt or [dt]) + [0.0, 0.0], np.float64)[:3]
        self.with_loss, self.mass_fix = bool(with_loss), bool(mass_fix)
        count = len(configs)
        self.meshes, self.ops, self.f = [None] * count, [None] * count, [None] * count
        members = {}
        for i, cfg in enumerate(configs):
            members.setdefault(_class_key(cfg), []).append(i)
        # one size class = one plan, one stacked state, per-cell restitution tables
        self._classes = []
        for idx in members.values():
            cfg0 = configs[idx[0]]
            sm = SpectralMesh(cfg0)
            op = FSInelasticVHSCollision(cfg0, sm, precision=precision, with_loss=with_loss, mass_fix=mass_fix,
                                         batch_max=len(idx), device=device)
            es, e0s = zip(*(_restitution(configs[i]) for i in idx))
            op.plan.set_restitution(es, e0s)
            states = []
            for i in idx:
                f = np.asarray(f0s[i], np.float64)
                if f.shape != (sm.nv,) * 3:
                    raise ValueError(f"initial state of shape {f.shape} for a {sm.nv}^3 grid")
                states.append(f)
            F = torch.as_tensor(np.stack(states), device=f"cuda:{self.device}").contiguous()
            for j, i in enumerate(idx):
                self.meshes[i], self.ops[i], self.f[i] = sm, op, F[j]
            self._classes.append((op, F, idx))
        self._graph = None
        self._stream = torch.cuda.Stream(device=self.device)
        # one stream per size class: the classes are independent, so their
        # kernels run side by side (parallel branches of the captured graph),
        # the smaller classes on the SMs the largest one leaves free
        self._side = [torch.cuda.Stream(device=self.device) for _ in self._classes]

    @property
    def plan_count(self):
        """Operator plans the ensemble holds (one per size class)."""
        return len(self._classes)

    def autotune(self):
        """Kernel choices of every class's plan, timed for its batch (``pii_plan_autotune``)."""
        out = [op.plan.autotune(len(idx)) for op, F, idx in self._classes]
        self._graph = None  # a replay would run the old choices
        return out

    def _launch_all(self):
        v1 = np.zeros(1)
        main = torch.cuda.current_stream(self.device)
        for (op, F, idx), side in zip(self._classes, self._side):
            side.wait_stream(main)
            plan = op.plan
            st = plan._lib.pii_step(plan.handle, _INT[self.integrator], F.data_ptr(), len(idx), self.dt,
                                    _lib.iptr(self.K), _lib.dptr(self.h), 1, 0.0, _lib.dptr(v1), _lib.BC_EXTRAP,
                                    _lib.BC_EXTRAP, self.kn, int(self.with_loss), int(self.mass_fix), 0,
                                    side.cuda_stream)
            _lib.check(st, "pii_step")
        for side in self._side:
            main.wait_stream(side)

    def step(self, use_graph=True):
        """One macro-step of every instance (one CUDA-graph launch after the first call)."""
        cur = torch.cuda.current_stream(self.device)
        self._stream.wait_stream(cur)
        with torch.cuda.stream(self._stream):
            if not use_graph:
                self._launch_all()
            else:
                if self._graph is None:
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g, stream=self._stream):
                        self._launch_all()
                    self._graph = g
                self._graph.replay()
        cur.wait_stream(self._stream)

    def collide(self):
        """Q(f,f) (gain - loss when the ensemble was built with_loss) of every
        instance's current state, one array per instance (one batched
        evaluation per size class)."""
        out = [None] * len(self.f)
        for op, F, idx in self._classes:
            Q = op.collide(F, with_loss=self.with_loss)
            for j, i in enumerate(idx):
                out[i] = Q[j]
        return out

    def moments(self):
        """FP64 (rho, u[3], T) of every instance."""
        out = []
        for sm, f in zip(self.meshes, self.f):
            v = sm.v_center
            V = np.meshgrid(v, v, v, indexing="ij")
            Vt = [torch.as_tensor(x, device=f.device) for x in V]
            dv = sm.delta**3
            rho = float(f.sum()) * dv
            u = np.array([float((f * Vt[d]).sum()) * dv / rho for d in range(3)])
            E = 0.5 * float((f * (Vt[0] ** 2 + Vt[1] ** 2 + Vt[2] ** 2)).sum()) * dv
            out.append((rho, u, (2.0 / 3.0) * (E / rho - 0.5 * float((u**2).sum()))))
        return out
