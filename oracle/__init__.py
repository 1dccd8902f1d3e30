"""TEST INFRASTRUCTURE ONLY — the oracle.

A CPU restatement of NuTo's element-assembly path (``nuto_oracle.hpp``, compiled to
``oracle/_build/liboracle.so``) plus a Python restatement of the quasistatic Newton driver
(``quasistatic.py``). Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package; the product library never does.

Parity status: the reference cannot be compiled in this environment (Eigen3, Boost and MUMPS are not
installed), so the restatement is pinned against the reference's own golden vectors and known-answer
tests (``tests/golden/`` and ``tests/test_oracle_*.py``).
"""

from .core import (  # noqa: F401
    build,
    lib,
    Mesh,
    Problem,
    Integrand,
    QUAD4,
    HEX8,
    HEX20,
    PLANE_STRESS,
    PLANE_STRAIN,
    FULL,
    UNILATERAL,
    MB_LINEAR_ELASTIC,
    MB_LOCAL_DAMAGE,
    GRADIENT_DAMAGE,
)
