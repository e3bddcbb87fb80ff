"""Time the reference's own operator on this machine's cores beside the oracle port.

The CPU baseline that ``bench.py`` reports runs the oracle (the FP64
NumPy/SciPy restatement in ``oracle/fs_inelastic.py``), because the reference
cannot travel to the benchmark host.  This script measures, on one machine
where the reference checkout is present, how the reference's own
``FSInelasticVHSCollision.collide`` (``src/collision/inelastic_collisions.py:139-172,
208-227``: broadcast tables, pyfftw plans over the (n_r, n_sigma, n^3) arrays)
compares with the port on the same cores and the same cells: the benchmark
workload's operator (n = 32 on [-8, 8]^3, 32 Gauss-Legendre radial x 32-point
design, hard spheres, e = e0 = 0.8, Q = gain - loss) on the Sod state's left
and right cells, one cell per call.

The reference runs under the shims of ``ref_shim.py`` (pyfftw's builders
mapped onto scipy.fft with ``workers`` threads; the reference's own setting is
``NUM_THREADS = 8``).  Results agree to FP64 rounding, which the script checks.

Run from the repository root (needs the reference checkout):
``PII_REFERENCE_ROOT=<checkout> python tests/golden/time_reference_cpu.py [cells] [workers]``
Prints one JSON line.  GPU test runs and ``bench.py`` never execute it.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import bench  # noqa: E402  (workload constants and the Sod state)
from oracle import fs_inelastic as fo  # noqa: E402
from ref_shim import load_reference  # noqa: E402


def main(cells=4, workers=None):
    workers = workers or os.cpu_count() or 1
    ref = load_reference(workers)
    cfg = bench.op_config()
    t0 = time.perf_counter()
    sm = ref.spectral_mesh.SpectralMesh(cfg)
    col = ref.inelastic.FSInelasticVHSCollision(cfg, sm)
    t_ref_setup = time.perf_counter() - t0
    f = bench.sod_state(sm.v_center)
    picks = [f[0], f[-1]]
    col(picks[0])  # the public call: builds the plans and broadcast kernels for one cell (n, n, n)
    col.collide(picks[0], with_loss=True)  # warm-up
    t0 = time.perf_counter()
    q_ref = [col.collide(picks[k % 2], with_loss=True) for k in range(cells)]
    t_ref = time.perf_counter() - t0

    m = fo.Mesh(bench.NV, bench.S_L8, bench.NR, bench.NS)
    op = fo.FSInelasticVHS(m, bench.E, bench.E, 1.0)
    op.collide_cell(picks[0], True, workers)  # warm-up
    t0 = time.perf_counter()
    q_port = [op.collide_cell(picks[k % 2], True, workers) for k in range(cells)]
    t_port = time.perf_counter() - t0
    err = max(float(np.abs(a - b).max() / np.abs(b).max()) for a, b in zip(q_port, q_ref))
    print(json.dumps({
        "workload": "Q(f,f) gain - loss, n=32^3 on [-8,8]^3, 32 GL radial x 32 design, e=e0=0.8, Sod cells",
        "cells": cells, "workers": workers, "cpu": os.uname().machine,
        "reference_cell_evals_per_s": cells / t_ref, "reference_setup_s": t_ref_setup,
        "port_cell_evals_per_s": cells / t_port, "port_over_reference": t_ref / t_port,
        "rel_linf_port_vs_reference": err,
    }))


if __name__ == "__main__":
    a = sys.argv[1:]
    main(int(a[0]) if a else 4, int(a[1]) if len(a) > 1 else None)
