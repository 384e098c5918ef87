"""GB300-native (sm_103a) DG/DGSEM residual and SSP Runge-Kutta update for
the 3D Euler equations: a drop-in for miniCFD's mini::spatial / mini::temporal
hot path (pvcStillInGradSchool/pvcRiemannSolvers).

The compute path is the C-ABI library ``libmcfd.so`` (include/mcfd.h) built
from ``csrc/`` for sm_103a; this package is its host-side mirror of the
reference interface.  There is no CPU fallback: constructing a system without
the built library or without a GPU raises.
"""
from . import capi, cases, mesh
from .system import Ensemble, General, Lobatto, MovingSplit, ObliqueSplit, RungeKutta, base64_encode, write_vtu_arrays

__all__ = ["capi", "cases", "mesh", "Ensemble", "General", "Lobatto", "MovingSplit", "ObliqueSplit", "RungeKutta",
           "base64_encode", "write_vtu_arrays"]
