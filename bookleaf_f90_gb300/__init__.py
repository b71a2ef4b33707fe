"""GB300 (sm_103a) implementation of BookLeaf's per-step hydro hot path.

  abi      ctypes mirror of include/bookleaf_gb300.h
  solver   Solver: inf_solver_getdt / inf_solver_lagstep / inf_solver_alestep
           on the device, and the device-resident time loop
  batch    BatchSolver: many independent problems advanced together
  closure  the learned mixed-cell closure: its network (tensor-core
           kernels), sub-cell training data from refined runs, training
  setup    host-side control-file reader, mesh generator, initial conditions
  build    nvcc build of the in-tree shared library
"""
from . import abi  # noqa: F401
from .solver import Solver, SolverError  # noqa: F401
from .batch import BatchSolver  # noqa: F401
from .setup import Problem, configs  # noqa: F401

__all__ = ["abi", "closure", "Solver", "SolverError", "BatchSolver", "Problem", "configs"]
