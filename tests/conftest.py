import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

L8_S = 16.0 / (3.0 + math.sqrt(2.0))  # velocity-mesh "s" giving L = 8


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name))

    return load


def op_config(nv, s, nr, nsphr, e, e0, gamma):
    return {
        "velocity-mesh": {"nv": int(nv), "s": float(s), "nr": int(nr)},
        "spherical-design-rule": {"ssrule": "womersley", "nsphr": int(nsphr)},
        "collision-model": {"dim": 3, "type": "vhs", "e": float(e), "e0": float(e0), "gamma": float(gamma)},
    }


def maxwellian(v, rho, u, T):
    V = np.meshgrid(v, v, v, indexing="ij")
    d2 = (V[0] - u[0]) ** 2 + (V[1] - u[1]) ** 2 + (V[2] - u[2]) ** 2
    return rho / (2 * math.pi * T) ** 1.5 * np.exp(-d2 / (2 * T))


def rel_linf(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
