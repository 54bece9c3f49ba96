"""GB300-native operator-split step of ReSEACT (SSPRK43 PPM transport + Rosenbrock23 chemistry).

The compute path is libreseact_gb300.so (C ABI, include/reseact_gb300.h), hand-written CUDA
for sm_103a.  Python here is the host mirror of the reference's driver interface:
``op_split.lie_trotter_solve{,_bisect}``, the .esm mechanism front end, and workload builders.
"""
from . import abi, mechanism, workloads  # noqa: F401
from ._lib import RsError, Solver, load  # noqa: F401
from .build import build as build_library  # noqa: F401
from .op_split import lie_trotter_solve, lie_trotter_solve_bisect  # noqa: F401
