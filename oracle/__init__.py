"""CPU oracle for the fast-spectral inelastic collision operator and its solver.

TEST INFRASTRUCTURE, NOT PRODUCT CODE.  This package is a plain NumPy / SciPy
FP64 restatement of the reference's algorithm for the hot path
(Mayuyu/proj-int-inelastic):

* ``fs_inelastic`` -- velocity mesh, quadratures, kernel tables and
  ``collide`` (``src/collision/spectral_mesh.py``,
  ``src/collision/inelastic_collisions.py``);
* ``transport``    -- second-order upwind + minmod TVD flux in x with the
  extrapolation / periodic ghost cells (``src/boltzmann.py:177-205``,
  ``src/solver.py:59-105``, ``src/riemann/advection_1D.py``,
  ``src/limiters/tvd.py``);
* ``integrators``  -- forward Euler, projective forward Euler and the 2- and
  3-level telescopic projective steps (``src/boltzmann.py:82-164``), plus the
  FP64 3D-velocity moments.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import it, and only as the
checker or the timed CPU baseline -- never as the thing measured or shipped.

Parity pin: the restatement is checked against fixtures produced by running
the reference itself (``tests/golden/make_golden.py``) -- the reference ships
no tests or golden vectors of its own.
"""
