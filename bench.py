#!/usr/bin/env python
"""Benchmark: Q(f,f) cell-evaluations per second on the 1D Riemann workload.

Workload (one step = one projective forward-Euler macro-step): n_x = 128
cells on [0, 1] with outflow (extrapolation) ghost cells, Sod data
(rho = 1, T = 1 | rho = 0.125, T = 0.8, zero velocity, local Maxwellians),
velocity grid 32^3 on [-8, 8]^3, 32 Gauss-Legendre radial nodes x the
32-point symmetric spherical design, hard spheres, e = e0 = 0.8,
kn = 1e-2, K = 2 inner steps of dt0 = 4e-4 (CFL 0.40) and macro-step 2e-3.
Each step evaluates Q(f,f) (gain - loss) twice on every cell: 256
cell-evaluations per step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Under torchrun (N > 1) every rank runs an
independent replica (the operator has no data-path collective; cells shard
with a 2-cell halo, which one GPU cannot exercise).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Q(f,f) cell-evals/s at N_v=32³/64³, mixed vs FP64 GPU at ≤1e-5 rel L∞ err"
UNIT = "cell-evals/s"
NX, NV, NR, NS = 128, 32, 32, 32
S_L8 = 16.0 / (3.0 + math.sqrt(2.0))
E = 0.8
KN = 1e-2
K_INNER, DT0, DT = 2, 4e-4, 2e-3
CELL_EVALS_PER_STEP = K_INNER * NX
WORKLOAD = (f"1D Riemann (Sod) PFE macro-step: n_x={NX} cells, N_v={NV}^3 on [-8,8]^3, {NR} GL radial x {NS} "
            f"symmetric spherical design, hard spheres, e=e0={E}, kn={KN}, K={K_INNER} inner steps dt0={DT0}, "
            f"macro dt={DT}, Q = gain - loss")


def op_config():
    return {
        "velocity-mesh": {"nv": NV, "s": S_L8, "nr": NR},
        "spherical-design-rule": {"ssrule": "womersley", "nsphr": NS},
        "collision-model": {"dim": 3, "type": "vhs", "e": E, "e0": E, "gamma": 1.0},
    }


def maxwellian(v, rho, u, T):
    import numpy as np

    V = np.meshgrid(v, v, v, indexing="ij")
    d2 = (V[0] - u[0]) ** 2 + (V[1] - u[1]) ** 2 + (V[2] - u[2]) ** 2
    return rho / (2 * math.pi * T) ** 1.5 * np.exp(-d2 / (2 * T))


def sod_state(v):
    import numpy as np

    x = (np.arange(NX) + 0.5) / NX
    left = maxwellian(v, 1.0, (0, 0, 0), 1.0)
    right = maxwellian(v, 0.125, (0, 0, 0), 0.8)
    return np.stack([left if xi < 0.5 else right for xi in x])


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
            return
        # nvidia-smi takes a few hundred ms to start: wait (at most 5 s) for its
        # first sample so that the record covers the whole timed region
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        os.unlink(self.path)
        if not rows:
            return out
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(nm)
        out.update(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=max(mx) if mx else None,
                   reasons=sorted(reasons), samples=len(rows),
                   power_w_max=max((float(r[3]) for r in rows if r[3].replace(".", "").isdigit()), default=None))
        return out


# ---------------------------------------------------------------------------
# the plain FP64 GPU implementation of the same method (torch.fft complex128),
# the reference's broadcast evaluation (src/collision/inelastic_collisions.py:208-227)
# ---------------------------------------------------------------------------
class TorchFP64Operator:
    def __init__(self, mesh, device, e=E, gamma=1.0):
        import numpy as np
        import torch

        n = mesh.nv
        r, wr = mesh.rquad()
        sigma, wsig = mesh.circ_or_sphr_quad()
        idx = np.fft.fftshift(np.arange(-n // 2, n // 2)).astype(np.float64)
        t = lambda a: torch.as_tensor(a, device=device)
        kx, ky, kz = torch.meshgrid(t(idx), t(idx), t(idx), indexing="ij")
        knorm = torch.sqrt(kx**2 + ky**2 + kz**2)
        sig = t(sigma)
        kdots = sig[:, 0, None, None, None] * kx + sig[:, 1, None, None, None] * ky + sig[:, 2, None, None, None] * kz
        rr = t(r)[:, None, None, None, None]
        er = 0.5 * (e - e) * np.tanh(r - 0.5 * mesh.R) + 0.5 * (e + e)
        a = t(0.25 * math.pi * (1 + er) / mesh.L)[:, None, None, None, None]
        pre = 4 * math.pi * rr ** (gamma + 2.0)
        sinc = lambda x: torch.where(x == 0, torch.ones_like(x), torch.sin(x) / torch.where(x == 0, torch.ones_like(x), x))
        self.gain = pre * torch.exp(1j * a * rr * kdots) * sinc(a * rr * knorm) * t(wr)[:, None, None, None, None] * wsig
        self.exp = torch.exp(-1j * math.pi * rr * kdots / mesh.L)
        loss = 4 * math.pi * t(r) ** (gamma + 2.0) * t(wr)
        self.loss = loss[:, None, None, None]
        self.sp = sinc(math.pi * t(r)[:, None, None, None] * knorm / mesh.L)

    def collide(self, f):
        import torch

        fft = lambda x: torch.fft.fftn(x, dim=(-3, -2, -1))
        ifft = lambda x: torch.fft.ifftn(x, dim=(-3, -2, -1))
        fh = fft(f)
        gain_hat = fft(ifft(self.exp * fh) * f)
        gain_hat *= self.gain
        gain = ifft(gain_hat.sum(dim=(0, 1)))
        loss = (ifft(self.sp * fh) * (self.loss * f)).sum(dim=0)
        return (gain / (4 * math.pi) - loss).real


def time_torch_fp64(mesh, f_dev, cells, device):
    import torch

    op = TorchFP64Operator(mesh, device)
    fc = f_dev[:cells].to(torch.complex128)
    op.collide(fc[0])
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for c in range(cells):
        op.collide(fc[c])
    e1.record()
    torch.cuda.synchronize()
    return cells / (e0.elapsed_time(e1) / 1e3)


# ---------------------------------------------------------------------------
# the 64^3 configuration: n = 64 on [-10, 10]^3, 48 GL radial nodes x the
# 70-point symmetric design (no 64-point design exists), e = e0 = 0.7, hard
# spheres, 3-Maxwellian mixtures (means in [-3, 3]^3, T in [0.5, 3])
# ---------------------------------------------------------------------------
N64, NR64, NS64, E64 = 64, 48, 70, 0.7
S_L10 = 20.0 / (3.0 + math.sqrt(2.0))


def mixture_states(v, cells, seed):
    import numpy as np

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(cells):
        f = sum(maxwellian(v, rng.uniform(0.5, 1.5), rng.uniform(-3, 3, 3), rng.uniform(0.5, 3.0)) for _ in range(3))
        out.append(f / (f.sum() * (v[1] - v[0]) ** 3))
    return np.stack(out)


def measure_n64(pkg, device, cells=256, cells_fp64=2):
    """Q(f,f) (gain - loss) at 64^3 on the configuration's 256 cells:
    mixed-precision throughput, the plain FP64 GPU method (torch.fft
    complex128) on `cells_fp64` cells, and the relative L-inf error of the mixed
    path against it."""
    import torch

    cfg = {"velocity-mesh": {"nv": N64, "s": S_L10, "nr": NR64},
           "spherical-design-rule": {"ssrule": "womersley", "nsphr": NS64},
           "collision-model": {"dim": 3, "type": "vhs", "e": E64, "e0": E64, "gamma": 1.0}}
    sm = pkg.SpectralMesh(cfg)
    f = torch.as_tensor(mixture_states(sm.v_center, cells, 64), device=device).contiguous()
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", with_loss=True, batch_max=cells, device=device.index)
    col.plan.autotune(min(cells, 16))
    q = col.collide(f[:16], with_loss=True)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    q = col.collide(f, with_loss=True)
    b.record()
    torch.cuda.synchronize()
    mixed = cells / (a.elapsed_time(b) / 1e3)
    out = {"config": f"n_v={N64}^3 on [-10,10]^3, {NR64} GL radial x {NS64}-point symmetric design, "
                     f"hard spheres, e=e0={E64}, 3-Maxwellian mixtures", "cells": cells,
           "mixed": mixed, "unit": UNIT, "tuning": col.plan.tuning}
    # the gain paths side by side (32 cells each): the fused cluster kernel, and
    # the packed pipeline with both first-axis column paths (in-register
    # CUDA-core FFT, tensor-core split-FP16 DFT)
    tuned = col.plan.tuning
    paths, q_path = {}, {}
    nc = min(cells, 32)
    for path in ("fused", "fft", "tensor"):
        if path == "fused":
            col.plan.set_tuning("fused", tuned["items_per_cluster"], tuned["chunk_points"])
        else:
            col.plan.set_tuning("packed", tuned["items_per_cluster"], tuned["chunk_points"], dft_path=path)
        col.collide(f[:nc], with_loss=True)
        torch.cuda.synchronize()
        a.record()
        col.collide(f[:nc], with_loss=True)
        b.record()
        torch.cuda.synchronize()
        paths[path] = nc / (a.elapsed_time(b) / 1e3)
        q_path[path] = col.collide(f[:cells_fp64], with_loss=True).clone()
    out["dft_paths"] = {"cells": nc, "unit": UNIT, **paths, "tensor_core_stalled": col.plan.dft_stalled}
    col.plan.set_tuning(**tuned)
    try:
        op = TorchFP64Operator(sm, device, e=E64, gamma=1.0)
        fc = f[:cells_fp64].to(torch.complex128)
        q64 = [op.collide(fc[0])]
        torch.cuda.synchronize()
        a.record()
        q64 = [op.collide(fc[c]) for c in range(cells_fp64)]
        b.record()
        torch.cuda.synchronize()
        out["fp64_torch"] = cells_fp64 / (a.elapsed_time(b) / 1e3)
        out["speedup_vs_fp64_gpu"] = mixed / out["fp64_torch"]
        errs = [float((q[c] - q64[c]).abs().max() / q64[c].abs().max()) for c in range(cells_fp64)]
        out["rel_linf_err_vs_fp64"] = max(errs)
        for path, qp in q_path.items():
            out["dft_paths"][f"rel_linf_err_{path}"] = max(
                float((qp[c] - q64[c]).abs().max() / q64[c].abs().max()) for c in range(cells_fp64))
        del op
    except Exception as ex:  # noqa: BLE001
        out["fp64_torch_error"] = str(ex)[:200]
    col.close()
    torch.cuda.empty_cache()
    return out


# ---------------------------------------------------------------------------
# ensemble configuration: 64 independent homogeneous problems, n drawn from
# {16, 24, 32, 48} (16 each), e = e0 ~ U[0.2, 1], n_r = n / 2 radial nodes x the
# 32-point design, L = 8, hard spheres; each f a sum of 2-4 Maxwellians (means
# in [-2, 2]^3, T in [0.5, 2]) of unit mass; PFE macro-steps (K = 2 inner
# Euler steps of 0.005, macro-step 0.02, kn = 1), Q = gain - loss
# ---------------------------------------------------------------------------
C3_KW = dict(dt=0.02, kn=1.0, integrator="PFE", inner_steps=[2], inner_dt=[0.005], with_loss=True)


def ensemble_problem(pkg, count=64, seed=2026):
    import numpy as np

    rng = np.random.default_rng(seed)
    sizes = [16, 24, 32, 48]
    configs, f0s = [], []
    for i in range(count):
        n = sizes[i % 4]
        e = float(rng.uniform(0.2, 1.0))
        cfg = {"velocity-mesh": {"nv": n, "s": S_L8, "nr": n // 2},
               "spherical-design-rule": {"ssrule": "womersley", "nsphr": 32},
               "collision-model": {"dim": 3, "type": "vhs", "e": e, "e0": e, "gamma": 1.0}}
        v = pkg.SpectralMesh(cfg).v_center
        k = int(rng.integers(2, 5))
        f = sum(maxwellian(v, rng.uniform(0.5, 1.5), rng.uniform(-2.0, 2.0, 3), rng.uniform(0.5, 2.0))
                for _ in range(k))
        configs.append(cfg)
        f0s.append(f / (f.sum() * (v[1] - v[0]) ** 3))
    return configs, f0s


def measure_c3(pkg, device, steps=5):
    """Aggregate instance-evaluations per second of the 64-problem ensemble
    (one captured graph per macro-step), and the per-instance relative L-inf
    error of the mixed path against the FP64 path: of Q on the initial states,
    and of f after the timed macro-steps."""
    import torch

    configs, f0s = ensemble_problem(pkg)
    ens = pkg.Ensemble(configs, f0s, precision="mixed", device=device.index, **C3_KW)
    tuning = [t for _, t in ens.autotune()]  # kernel choices per size class, timed on the device
    dbl = pkg.Ensemble(configs, f0s, precision="double", device=device.index, **C3_KW)
    qm, qd = ens.collide(), dbl.collide()
    q_err = [float((a - b).abs().max() / b.abs().max()) for a, b in zip(qm, qd)]
    warm = 2
    for _ in range(warm):
        ens.step()  # the first call captures the graph
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        ens.step()
    b.record()
    torch.cuda.synchronize()
    sec = a.elapsed_time(b) / 1e3
    evals = len(configs) * C3_KW["inner_steps"][0] * steps
    for _ in range(warm + steps):
        dbl.step(use_graph=False)
    torch.cuda.synchronize()
    f_err = [float((x - y).abs().max() / y.abs().max()) for x, y in zip(ens.f, dbl.f)]
    sizes = sorted({c["velocity-mesh"]["nv"] for c in configs})
    out = {"config": "64 homogeneous problems, n_v in {16,24,32,48}^3 (16 each) on [-8,8]^3, e=e0~U[0.2,1], "
                     "n_r=n/2 GL radial x 32-point design, 2-4 Maxwellian mixtures; PFE K=2 dt0=0.005 dt=0.02 kn=1",
           "instances": len(configs), "macro_steps": steps, "instance_evals_per_s": evals / sec,
           "ms_per_macro_step": sec / steps * 1e3, "plans": ens.plan_count, "tuning": tuning,
           "q_rel_linf_err_vs_fp64_max": max(q_err), "f_rel_linf_err_vs_fp64_max": max(f_err),
           "f_err_after_macro_steps": warm + steps,
           "q_rel_linf_err_by_n": {str(n): max(e for e, c in zip(q_err, configs) if c["velocity-mesh"]["nv"] == n)
                                   for n in sizes}}
    del ens, dbl
    torch.cuda.empty_cache()
    return out


# ---------------------------------------------------------------------------
# stiff telescopic configuration: TPI3 at kn = 1e-4 on n_x = 512 periodic
# cells, rho = 1 + 0.2 sin(2 pi x), T = 1 + 0.1 cos(2 pi x), zero velocity,
# local Maxwellians; 32^3 on [-8, 8]^3, 32 x 32 quadrature, e = e0 = 0.9,
# hard spheres, mass-mode fix on.  Levels dt = (1e-5, 2.5e-5, 6.25e-5), K = 2
# each, macro-step 2e-4 (M = 0.5, 0.5, 1.2; advection CFL 0.79; the inner
# step keeps the collision term's explicit bound, nu dt0 / kn <= 0.62).
# ---------------------------------------------------------------------------
C4_NX, C4_KN, C4_E = 512, 1e-4, 0.9
C4_K, C4_H, C4_DT, C4_TEND = [2, 2, 2], [1e-5, 2.5e-5, 6.25e-5], 2e-4, 0.05


def c4_state(v, nx=C4_NX):
    import numpy as np

    x = (np.arange(nx) + 0.5) / nx
    return np.stack([maxwellian(v, 1 + 0.2 * math.sin(2 * math.pi * xi), (0, 0, 0),
                                1 + 0.1 * math.cos(2 * math.pi * xi)) for xi in x])


def c4_solver(pkg, precision, device, f0):
    import torch

    cfg = {"velocity-mesh": {"nv": 32, "s": S_L8, "nr": 32},
           "spherical-design-rule": {"ssrule": "womersley", "nsphr": 32},
           "collision-model": {"dim": 3, "type": "vhs", "e": C4_E, "e0": C4_E, "gamma": 1.0}}
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision=precision, with_loss=True, mass_fix=True,
                                      batch_max=C4_NX, device=device.index)
    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": C4_NX, "nv": 32},
                       device=device.index)
    sol.state.f.copy_(torch.as_tensor(f0))
    solver = pkg.BoltzmannSolver1D(C4_KN, collision_operator=col)
    solver.all_bcs = pkg.BC.periodic
    solver.time_integrator = "TPI3"
    solver.inner_steps = list(C4_K)
    solver.inner_dt = list(C4_H)
    solver.dt = C4_DT
    solver.setup(sol)
    return col, sol, solver


def measure_c4(pkg, device, macro_steps=10, fp64_steps=1):
    """TPI3 macro-steps of the stiff periodic workload in mixed precision:
    cell-evaluations per second (device time, graph replays), total mass and
    energy after every macro-step relative to the start (FP64 moments), and
    the relative L-inf state error against the FP64 path after each of the
    first `fp64_steps` macro-steps."""
    import numpy as np
    import torch

    v = (np.arange(32) + 0.5) * (16.0 / 32) - 8.0  # the 32^3 grid on [-8, 8]^3 (cell centres)
    col, sol, solver = c4_solver(pkg, "mixed", device, c4_state(v))
    f0 = sol.f.clone()
    st = sol.state

    def mass_energy():
        rho, u, T = (np.asarray(x) for x in st.moments())
        m = float(np.sum(rho))
        e = float(np.sum(rho * (1.5 * T + 0.5 * np.sum(np.asarray(u) ** 2, axis=-1))))
        return m, e, float(np.mean(T))

    m0, e0, T0 = mass_energy()
    # time one macro-step advances under the reference's telescopic recurrence
    # (src/boltzmann.py:142-158: level l adds M_l ... M_0 inner increments of dt0)
    (K0, K1, K2), (h0, h1, h2) = C4_K, C4_H
    M0, M1, M2 = h1 / h0 - K0, h2 / h1 - K1, C4_DT / h2 - K2
    tau = K2 * (K1 * h1 + M1 * M0 * h0) + M2 * M1 * M0 * h0
    stream = solver._get_stream(device)
    solver.step(sol, False, 0.0, C4_DT)  # capture the macro-step graph (excluded from the record below)
    sol.state.f.copy_(f0)
    torch.cuda.synchronize()
    keep = []
    rec, ms = [], 0.0
    for k in range(macro_steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
            solver.step(sol, False, k * C4_DT, (k + 1) * C4_DT)
            b.record(stream)
        torch.cuda.synchronize()
        ms += a.elapsed_time(b)
        m, e, T = mass_energy()
        rec.append({"t": (k + 1) * C4_DT, "t_advanced": (k + 1) * tau, "mass_rel": m / m0 - 1.0,
                    "energy_rel": e / e0 - 1.0, "T_mean": T, "f_min": float(sol.f.min()),
                    "finite": bool(torch.isfinite(sol.f).all())})
        if k < fp64_steps:
            keep.append(sol.f.clone())
    evals = 8 * C4_NX * macro_steps
    out = {"config": f"TPI3 kn={C4_KN}, n_x={C4_NX} periodic, rho=1+0.2sin(2pi x), T=1+0.1cos(2pi x), 32^3 on "
                     f"[-8,8]^3, 32x32, e=e0={C4_E}, hard spheres, mass fix; levels dt={C4_H}, K={C4_K}, "
                     f"macro dt={C4_DT}", "cells": C4_NX, "macro_steps": macro_steps,
           "cell_evals_per_s": evals / (ms / 1e3), "ms_per_macro_step": ms / macro_steps,
           "time_advanced_per_macro_step": tau,
           "mass_drift_max": max(abs(r["mass_rel"]) for r in rec), "energy_rel_end": rec[-1]["energy_rel"],
           "T_mean_end": rec[-1]["T_mean"], "t_end": rec[-1]["t"], "all_finite": all(r["finite"] for r in rec),
           "per_macro_step": rec if macro_steps <= 20 else rec[:: max(1, macro_steps // 20)] + [rec[-1]]}
    del col, sol, solver
    if fp64_steps:
        colD, solD, solverD = c4_solver(pkg, "double", device, f0.cpu().numpy())
        errs = []
        for k in range(fp64_steps):
            solverD.step(solD, False, k * C4_DT, (k + 1) * C4_DT)
            torch.cuda.synchronize()
            errs.append(float((keep[k] - solD.f).abs().max() / solD.f.abs().max()))
        out["f_rel_linf_err_vs_fp64"] = errs
        del colD, solD, solverD
    torch.cuda.empty_cache()
    return out


# ---------------------------------------------------------------------------
# CPU baseline (the oracle restatement of the reference operator, host cores)
# ---------------------------------------------------------------------------
def cpu_baseline(budget_s=15.0, max_cells=64):
    import numpy as np

    from oracle import fs_inelastic as fo

    workers = os.cpu_count() or 1
    m = fo.Mesh(NV, S_L8, NR, NS)
    op = fo.FSInelasticVHS(m, E, E, 1.0)
    f = sod_state(m.v)
    picks = [0, NX - 1]
    op.collide_cell(f[0], True, workers)  # warm-up (tables, FFT plans)
    t0 = time.perf_counter()
    done = 0
    while done < max_cells and (time.perf_counter() - t0) < budget_s:
        op.collide_cell(f[picks[done % 2]], True, workers)
        done += 1
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": UNIT, "cores": workers, "kind": "port",
            "sample": f"{done} single-cell Q(f,f) (gain - loss) evaluations of the Sod state (left/right cells), "
                      f"FP64 NumPy/SciPy restatement of the reference operator, scipy.fft workers={workers}, "
                      f"{dt:.1f} s"}


# ---------------------------------------------------------------------------
def dist_setup(n_gpus):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
        return world, rank, local, dist
    return 1, 0, 0, None


def replica_aggregate(total_s, cell_evals, dist=None, device=None):
    """Whole-job throughput of N independent replicas (no data-path collective):
    every rank's cell-evaluations over the slowest rank's time."""
    import torch

    world = dist.get_world_size() if dist else 1
    if dist:
        t = torch.tensor([total_s], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t)
    return world * cell_evals / total_s, total_s


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import numpy as np

    from oracle import fs_inelastic as fo

    workers = os.cpu_count() or 1
    m = fo.Mesh(NV, S_L8, NR, NS)
    op = fo.FSInelasticVHS(m, E, E, 1.0)
    f = sod_state(m.v)
    cells = [0, NX - 1]
    for w in range(args.warmup):
        op.collide_cell(f[cells[w % 2]], True, workers)
    t0 = time.perf_counter()
    for k in range(args.steps):
        op.collide_cell(f[cells[k % 2]], True, workers)
    dt = time.perf_counter() - t0
    value = args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "reference_step": "one Q(f,f) cell-evaluation of the workload "
                   "(bounded sample: alternating left/right Sod cells)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": workers, "kind": "port",
                         "sample": f"{args.steps} single-cell Q(f,f) evaluations, FP64 NumPy/SciPy restatement of "
                                   f"the reference operator (the reference itself needs pyfftw/cupy, absent on the "
                                   f"benchmark host), scipy.fft workers={workers}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def ncu_case(cells, precision="mixed"):
    """Small profiling case: 3 Q(f,f) evaluations on `cells` cells of the
    workload, in mixed precision or (precision "double") in FP64."""
    import torch

    import proj_int_inelastic_gb300 as pkg

    cfg = op_config()
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision=precision, with_loss=True, batch_max=cells)
    f = torch.as_tensor(sod_state(sm.v_center)[:cells], device="cuda:0").contiguous()
    for _ in range(3):
        q = col.collide(f, with_loss=True)
    torch.cuda.synchronize()
    print(json.dumps({"ncu_case_cells": cells, "precision": precision, "tuning": col.plan.tuning,
                      "q_abs_max": float(q.abs().max())}))
    return 0


def ncu_case64(cells, dft_path, gain_path="packed"):
    """Small profiling case at 64^3 (the 48 x 70 quadrature, 3-Maxwellian cells): one
    mixed-precision Q(f,f) evaluation with the given first-axis column path
    (packed pipeline) or the fused gain kernel (gain_path "fused")."""
    import torch

    import proj_int_inelastic_gb300 as pkg

    cfg = {"velocity-mesh": {"nv": N64, "s": S_L10, "nr": NR64},
           "spherical-design-rule": {"ssrule": "womersley", "nsphr": NS64},
           "collision-model": {"dim": 3, "type": "vhs", "e": E64, "e0": E64, "gamma": 1.0}}
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", with_loss=True, batch_max=cells)
    if gain_path == "fused":
        col.plan.set_tuning("fused", 6, 131072)
    else:
        col.plan.set_dft_path(dft_path)
    f = torch.as_tensor(mixture_states(sm.v_center, cells, 64), device="cuda:0").contiguous()
    q = col.collide(f, with_loss=True)
    torch.cuda.synchronize()
    print(json.dumps({"ncu_case64_cells": cells, "dft_path": dft_path, "gain_path": col.plan.tuning["gain_path"],
                      "q_abs_max": float(q.abs().max()),
                      "stalled": col.plan.dft_stalled}))
    return 0


def ncu_case_class(n, cells):
    """Small profiling case of one ensemble size class (n^3 on [-8, 8]^3,
    n / 2 GL radial x 32-point design, e = e0 = 0.7, mixture states): two
    mixed-precision Q(f,f) evaluations with the plan's default kernels."""
    import torch

    import proj_int_inelastic_gb300 as pkg

    cfg = {"velocity-mesh": {"nv": n, "s": S_L8, "nr": n // 2},
           "spherical-design-rule": {"ssrule": "womersley", "nsphr": 32},
           "collision-model": {"dim": 3, "type": "vhs", "e": 0.7, "e0": 0.7, "gamma": 1.0}}
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", with_loss=True, batch_max=cells)
    f = torch.as_tensor(mixture_states(sm.v_center, cells, 64), device="cuda:0").contiguous()
    for _ in range(2):
        q = col.collide(f, with_loss=True)
    torch.cuda.synchronize()
    print(json.dumps({"ncu_case_class": n, "cells": cells, "q_abs_max": float(q.abs().max()),
                      "tuning": col.plan.tuning}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the plan's default kernel choices")
    ap.add_argument("--no-n64", action="store_true", help="skip the 64^3 configuration measurement")
    ap.add_argument("--no-c3", action="store_true", help="skip the ensemble configuration measurement")
    ap.add_argument("--no-c4", action="store_true", help="skip the stiff telescopic configuration measurement")
    ap.add_argument("--c4-steps", type=int, default=10,
                    help="TPI3 macro-steps of the stiff configuration (250 reach its end time t = 0.05)")
    ap.add_argument("--c4-fp64-steps", type=int, default=1,
                    help="macro-steps of the stiff configuration compared against the FP64 path")
    ap.add_argument("--c4-only", action="store_true", help="measure only the stiff configuration and exit")
    ap.add_argument("--c3-only", action="store_true", help="measure only the ensemble configuration and exit")
    ap.add_argument("--ncu-case", type=int, default=0,
                    help="profiling case: run 3 Q(f,f) evaluations on this many cells of the workload and exit")
    ap.add_argument("--ncu-precision", default="mixed", choices=["mixed", "double"],
                    help="precision of the --ncu-case evaluations")
    ap.add_argument("--ncu-class", type=int, default=0,
                    help="profiling case: one ensemble size class n^3 (with --ncu-cells cells) and exit")
    ap.add_argument("--ncu-cells", type=int, default=4)
    ap.add_argument("--ncu-case64", type=int, default=0,
                    help="profiling case: one 64^3 Q(f,f) evaluation on this many cells and exit")
    ap.add_argument("--dft-path", default="tensor", choices=["tensor", "fft"],
                    help="first-axis column path of the 64^3 profiling case")
    ap.add_argument("--gain-path", default="packed", choices=["packed", "fused"],
                    help="gain kernel of the 64^3 profiling case")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.ncu_case:
        return ncu_case(args.ncu_case, args.ncu_precision)
    if args.ncu_class:
        return ncu_case_class(args.ncu_class, args.ncu_cells)
    if args.ncu_case64:
        return ncu_case64(args.ncu_case64, args.dft_path, args.gain_path)
    if args.c4_only or args.c3_only:
        import torch

        import proj_int_inelastic_gb300 as pkg

        dev = torch.device("cuda:0")
        out = {"c4": measure_c4(pkg, dev, args.c4_steps, args.c4_fp64_steps)} if args.c4_only else {
            "c3": measure_c3(pkg, dev)}
        print(json.dumps(out), flush=True)
        return 0
    args.warmup = max(3, args.warmup)

    import numpy as np
    import torch

    world, rank, local, dist = dist_setup(args.gpus)
    device = torch.device(f"cuda:{local}")
    torch.cuda.set_device(device)
    import proj_int_inelastic_gb300 as pkg

    lib = pkg._lib.load()
    cfg = op_config()
    sm = pkg.SpectralMesh(cfg)
    col = pkg.FSInelasticVHSCollision(cfg, sm, precision="mixed", with_loss=True, batch_max=NX, device=local)
    if args.no_autotune:
        tuning = col.plan.tuning
    else:
        tune_ms, tuning = col.plan.autotune(NX)  # kernel choices for this batch, timed on the device
    f0_host = sod_state(sm.v_center)
    sol = pkg.Solution({"dim_x": 1, "dim_v": 3, "xmin": 0.0, "xmax": 1.0, "l": sm.L, "nx": NX, "nv": NV},
                       device=local)
    sol.state.f.copy_(torch.as_tensor(f0_host))
    solver = pkg.BoltzmannSolver1D(KN, collision_operator=col)
    solver.all_bcs = pkg.BC.extrap
    solver.time_integrator = "PFE"
    solver.inner_steps = [K_INNER]
    solver.inner_dt = [DT0]
    solver.dt = DT
    solver.setup(sol)

    def step():
        solver.step(sol, False, 0.0, DT)

    for _ in range(args.warmup):
        step()
    stream = solver._get_stream(device)
    torch.cuda.synchronize()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)  # > 129 MB L2

    # ---------------- timed region: device time of K macro-steps -------------
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = lib.pii_kernel_launches()
    evs = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()  # L2 flush between timed steps (outside the event pair)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            evs.append((a, b))
    torch.cuda.synchronize()
    launches = lib.pii_kernel_launches() - launches0
    if dist:
        dist.barrier()
    ck = clocks.stop()
    total_s = sum(a.elapsed_time(b) for a, b in evs) / 1e3
    value, total_s = replica_aggregate(total_s, CELL_EVALS_PER_STEP * args.steps, dist, device)
    ms_per_step = total_s / args.steps * 1e3

    # ---------------- e2e: host f in, host f out, through the solver API -------
    pin_in = torch.empty(sol.f.shape, dtype=torch.float64).pin_memory()
    pin_out = torch.empty_like(pin_in).pin_memory()
    pin_in.copy_(torch.as_tensor(f0_host))
    e2e_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sol.state.f.copy_(pin_in, non_blocking=True)
        step()
        pin_out.copy_(sol.state.f, non_blocking=True)
        torch.cuda.current_stream().synchronize()
    e2e_s = time.perf_counter() - t0
    _, e2e_s = replica_aggregate(e2e_s, CELL_EVALS_PER_STEP * e2e_steps, dist, device)
    nbytes = sol.f.numel() * 8
    e2e = {"value": world * CELL_EVALS_PER_STEP * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": nbytes,
           "d2h_bytes_per_step": nbytes,
           "path": "pinned host f -> device, BoltzmannSolver1D.step (PFE macro-step), device f -> pinned host"}

    # ---------------- attribution: per-kernel CUDA-event timing ---------------
    plan = col.plan
    lib.pii_plan_profile(plan.handle, 1)
    with torch.cuda.stream(stream):
        step()
    ms = (pkg._lib.ctypes.c_double * pkg._lib.NSTAGES)()
    cnt = (pkg._lib.ctypes.c_int64 * pkg._lib.NSTAGES)()
    lib.pii_plan_profile_read(plan.handle, ms, cnt)
    lib.pii_plan_profile(plan.handle, 0)
    stages = {pkg._lib.STAGES[i]: {"ms": ms[i], "launches": int(cnt[i])} for i in range(pkg._lib.NSTAGES) if cnt[i]}
    tot = sum(v["ms"] for v in stages.values())
    for v in stages.values():
        v["share"] = v["ms"] / tot if tot else None
    dom = max(stages, key=lambda k: stages[k]["ms"])
    # the packed gain path is two kernels (the a-parity pass over antipodal
    # pairs and its Nyquist correction): the gain term's time is their sum
    gain_ms = stages[dom]["ms"] + (stages["nyq_corr"]["ms"] if dom == "gain_parity" and "nyq_corr" in stages else 0.0)
    # algorithmic FLOPs: one 1D pass over a grid = 5 N log2(n); items = (cell, pair)
    N = NV**3
    items_per_collide = NX * NR * NS
    pass_flops = 5.0 * N * math.log2(NV)
    # per (cell, pair) item; the fused kernel does the whole pair (direct-method term 2*5N log2 N + 16 N)
    per_item = {"pair_plane": 4 * pass_flops + 2 * N, "col_pstart": pass_flops + 12 * N,
                "col_pend": pass_flops + 14 * N, "reduce": 2 * N,
                "gain_cluster": 2 * 5.0 * N * math.log2(N) + 16 * N,
                "gain_parity": 2 * 5.0 * N * math.log2(N) + 16 * N}
    collides = K_INNER
    if dom in per_item:
        flops_total = per_item[dom] * items_per_collide * collides
    else:
        flops_total = None
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    n_sms = int(torch.cuda.get_device_properties(local).multi_processor_count)
    fp32_peak = n_sms * 128 * 2 * sm_max * 1e6 / 1e12  # TFLOP/s, FP32 FMA lanes x clock
    roof = {"kernel": dom, "bound": "fp32", "unit": "TFLOP/s", "peak": fp32_peak,
            "peak_source": f"{n_sms} SMs (device query) x 128 FP32 lanes x 2 flop x sm_max_mhz={sm_max:.0f} "
                           "(MEASURED_PEAKS.json); MEASURED_PEAKS.json has no FP32 CUDA-core figure",
            "launches_per_step": stages[dom]["launches"], "avg_launch_ms": stages[dom]["ms"] / stages[dom]["launches"]}
    if flops_total:
        per_launch = flops_total / stages[dom]["launches"]
        roof["achieved"] = per_launch / (gain_ms / stages[dom]["launches"] / 1e3) / 1e12
        roof["frac"] = roof["achieved"] / fp32_peak
        roof["algorithmic_flops_per_launch"] = per_launch
        if gain_ms != stages[dom]["ms"]:
            roof["timed_kernels"] = "gain_parity + nyq_corr (the gain term)"
            roof["note"] = ("algorithmic FLOPs of the direct method (2 * 5 N log2 N + 16 N per (cell, pair)); the "
                            "packed path evaluates antipodal pairs together and performs about half of them")
            # the same work counted as executed: one pass per antipodal pair
            # (half the pairs) plus the Nyquist correction's 12 FMA per
            # (output point, input-point pair, cell), about 1.5 n^2 Nq of them
            nq = 3 * NV * NV - 3 * NV + 1
            exe = per_launch / 2 + 2 * 12 * 1.5 * NV * NV * nq * NX
            roof["executed_flops_per_launch"] = exe
            roof["executed_frac"] = exe / (gain_ms / stages[dom]["launches"] / 1e3) / 1e12 / fp32_peak
    else:
        roof["achieved"] = roof["frac"] = None
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    roof["traffic"] = None
    if os.path.exists(tfile):
        tr = json.load(open(tfile))
        tkey = "gain_packed" if gain_ms != stages[dom]["ms"] else dom  # packed: both kernels of the gain term
        if tkey in tr:
            roof["traffic"] = tr[tkey].get("dram_bytes_per_launch")
            roof["traffic_source"] = tr[tkey].get("source")
    # whole-step FLOP rate (algorithmic F = (2Q + n_r + 2) 5N log2 N + 16 Q N per cell-eval) for context
    F_cell = (2 * NR * NS + NR + 2) * 5 * N * math.log2(N) + 16 * NR * NS * N
    roof["step_algorithmic_tflops"] = F_cell * value / world / 1e12
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "precision": "FP32 FFTs and quadrature sums; FP64 state, increments, extrapolation",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "cells": NX, "n_v": NV, "n_r": NR, "n_sigma": NS,
                   "cell_evals_per_step": CELL_EVALS_PER_STEP, "l2": "flushed (256 MB write) between timed steps",
                   "graph": "each macro-step replayed as one CUDA graph", "parallelism": f"replicas x{world}",
                   "tuning": tuning},
        "clocks": ck, "e2e": e2e, "gpu_launches": int(launches), "roofline": roof,
        "kernels": stages, "hbm_peak_gbs": hbm_peak,
    }

    # ---------------- comparators (rank 0, N = 1 legs) -------------------------
    if rank == 0 and not args.no_fp64:
        f_dev = sol.state.f.new_tensor(f0_host)
        dbl = pkg.FSInelasticVHSCollision(cfg, sm, precision="double", with_loss=True, batch_max=NX, device=local)
        qm = col.collide(f_dev, with_loss=True)
        q64 = dbl.collide(f_dev, with_loss=True)
        err = (qm - q64).abs().amax(dim=(1, 2, 3)) / q64.abs().amax(dim=(1, 2, 3))
        line["rel_linf_err_vs_fp64"] = float(err.max())
        plan64 = dbl.plan
        q = torch.empty_like(f_dev)
        cells64 = 16
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        st = lib.pii_collide(plan64.handle, f_dev.data_ptr(), q.data_ptr(), cells64, 1, 0.0, 0,
                             torch.cuda.current_stream().cuda_stream)
        b.record()
        torch.cuda.synchronize()
        pkg._lib.check(st, "pii_collide fp64")
        pii64 = cells64 / (a.elapsed_time(b) / 1e3)
        dbl.close()
        try:
            torch64 = time_torch_fp64(sm, f_dev, 4, device)
        except Exception as ex:  # noqa: BLE001
            torch64 = None
            line["fp64_torch_error"] = str(ex)[:200]
        collide_rate = None
        # collide-only throughput of the mixed path on the full batch (device time)
        qm2 = torch.empty_like(f_dev)
        torch.cuda.synchronize()
        a.record()
        for _ in range(3):
            lib.pii_collide(col.plan.handle, f_dev.data_ptr(), qm2.data_ptr(), NX, 1, 0.0, 0,
                            torch.cuda.current_stream().cuda_stream)
        b.record()
        torch.cuda.synchronize()
        collide_rate = 3 * NX / (a.elapsed_time(b) / 1e3)
        line["fp64_gpu"] = {
            "torch_fft_complex128": torch64,
            "pii_fp64_kernels": pii64,
            "unit": UNIT,
            "what": "Q(f,f) gain - loss on the workload's cells: the reference's broadcast method in "
                    "torch.fft complex128 (4 cells), and this library's kernels in FP64 (16 cells)",
        }
        line["mixed_collide_only"] = collide_rate
        if torch64:
            line["speedup_vs_fp64_gpu"] = collide_rate / torch64
    if rank == 0 and not args.no_n64:
        line["n64"] = measure_n64(pkg, device)
    if rank == 0 and not args.no_c3:
        line["c3"] = measure_c3(pkg, device)
    if rank == 0 and not args.no_c4:
        line["c4"] = measure_c4(pkg, device, args.c4_steps, args.c4_fp64_steps)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
