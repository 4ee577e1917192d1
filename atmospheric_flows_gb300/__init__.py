"""GB300-native hot path of an IMEX-DG dynamical core.

sm_103a CUDA kernels behind a C ABI (``include/atm_gb300.h``) replace the
matrix-free ``EULEROperator`` and the stage solvers of
GiuseppeOrlando878776/Atmospheric_Flows.  Python is the test and bench
harness; the time loop runs in the library.
"""
from .hill import HillParams, HillCase, build_case  # noqa: F401

__all__ = ["HillParams", "HillCase", "build_case", "EULEROperator", "MatrixFreeStorage",
           "EulerSolver"]


def __getattr__(name):
    if name in ("EULEROperator", "MatrixFreeStorage"):
        from . import euler_operator

        return getattr(euler_operator, name)
    if name == "EulerSolver":
        from .euler_solver import EulerSolver

        return EulerSolver
    raise AttributeError(name)
