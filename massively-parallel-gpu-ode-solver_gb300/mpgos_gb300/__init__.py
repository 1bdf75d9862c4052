"""GB300-native ensemble explicit Runge-Kutta integrator (host side).

The numerical work runs in sm_103a kernels behind the C-ABI of
``include/mpgos.h``; this package builds the native libraries in-tree
(``build``), binds the C-ABI (``capi``) and mirrors the reference's host
object ``ProblemSolver`` (``solver``).
"""
from .capi import Algorithm, MpgosError, Option, Variable  # noqa: F401
from .solver import ProblemSolver  # noqa: F401
