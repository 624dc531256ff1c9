"""GB300 (sm_103a) Vertex Block Descent and XPBD for SPG scenes.

The solver is the CUDA library ``libspgx.so`` behind the C ABI in ``include/spgx.h``;
``spg_gb300.native`` holds its ctypes bindings and ``spg_gb300.scenes`` the scene builders.
"""
from spg_gb300.native import (ANCHOR, BENDING, SNH, SPRING, STVK, SpgxError, VbdSolver, XpbdSolver,  # noqa: F401
                              eval_constraints, eval_vertex_blocks, lib)
