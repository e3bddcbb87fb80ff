"""GB300-native fast-spectral inelastic collision operator and projective steps.

Drop-in for the hot path of Mayuyu/proj-int-inelastic: the operator classes of
``src/collision`` and the step interface of ``src/solver.py`` /
``src/boltzmann.py`` / ``src/iter_solver.py``, evaluated by hand-written
sm_103a CUDA kernels in ``libpii_gb300.so`` (C ABI: ``include/pii_gb300.h``).
"""
from . import _lib
from .collision import FSInelasticVHSCollision, Plan, SpectralMesh, get_sphrquadrule
from .ensemble import Ensemble
from .solver import (BC, BoltzmannFastSweep, BoltzmannSolver, BoltzmannSolver0D, BoltzmannSolver1D, Grid,
                     IterativeBoltzmannSolver, Solution, Solver, State, maxwellian)

__all__ = [
    "BC", "BoltzmannFastSweep", "BoltzmannSolver", "Ensemble", "BoltzmannSolver0D", "BoltzmannSolver1D", "FSInelasticVHSCollision",
    "Grid", "IterativeBoltzmannSolver", "Plan", "Solution", "Solver", "SpectralMesh", "State", "get_sphrquadrule",
    "maxwellian",
]
