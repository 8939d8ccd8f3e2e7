"""CPU oracle for the GPE time-stepping hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
package: only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline``
leg / ``--impl reference`` arm of ``bench.py`` use it, and there only as the
checker or as the timed CPU baseline.

The oracle restates, in plain FP64 NumPy, the reference's own CPU algorithms:

* ``oracle.philox``  -- Philox-4x32-10, counter layout, Box-Muller normals and
  the truncated-Wigner increment (``polarism/noise/philox.py``,
  ``polarism/noise/stochastic.py``).
* ``oracle.gpe``     -- the finite-difference right-hand side, the stage-coupled
  RK4 step (``rk4-fdm``), both Strang orderings of the split-step method, the
  Lawson IFRK step with the embedded DP5 error norm, and the FP64 observables.

Parity is pinned by ``tests/test_oracle_golden.py`` against fixtures in
``tests/golden/`` that were produced by running the reference itself
(``tests/golden/make_golden.py``) plus the reference's own known-answer vectors.
"""
