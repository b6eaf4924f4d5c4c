"""CPU oracle for the BP / FFBP path.

TEST INFRASTRUCTURE ONLY.  Nothing in ``bp_project_gb300`` imports this
package; it is used by ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` to check and time the product.

* ``oracle.cpp`` restates the reference's FP64 Numba kernels
  (``fast_bp/ffbp.py``) in C++/OpenMP.
* ``plan.py`` restates the reference's FP64 FFBP planner
  (``fast_bp/gpu_backend.py:121-224`` / ``fast_bp/ffbp.py:124-177``) in numpy.
* ``reference.py`` wraps both with the reference's function names.

Parity pin: ``tests/golden/`` holds outputs of the reference itself
(``fast_bp/ffbp.py`` and ``build_ffbp_plan`` imported with a no-op numba
shim) on seeded inputs; ``tests/test_oracle_golden.py`` checks this oracle
against them.
"""
