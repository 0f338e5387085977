"""GB300-native Jacobi Poisson solver backend for fpie.

The package provides the fpie solver plugin classes ``EquSolver`` and
``GridSolver`` (``partition`` / ``reset`` / ``sync`` / ``step``) over a C-ABI
shared library of hand-written sm_103a CUDA kernels, plus processors that
mirror ``fpie.process`` and select the backend by name.
"""

__version__ = "0.1.0"
