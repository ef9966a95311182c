"""CPU parity oracle for incompact3d_gb300 (test infrastructure only).

The product library never imports this package.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it, as
the checker.  ``x3d_oracle.cpp`` restates the reference's FP64 arithmetic for
the per-timestep path (compact schemes, filters, staggered operators, periodic
Poisson solve, incompressible step); see the file:line citations there.
"""
from .oracle import Oracle, build, OP_DER1, OP_DER2, OP_FIL, OP_DVP, OP_IVP, OP_DPV, OP_IPV  # noqa: F401
