"""fv2d_gb300: GB300-native (sm_103a) residual-and-update step of the fv2d 2-D unstructured
finite-volume Euler/Navier-Stokes solver (drop-in for Avery-Hantla/CFD-2D-NS-FV's solver step).

The directory name contains dashes, so load it with ``load_package()`` from the repository root
(``__graft_entry__``, ``bench.py`` and the tests do) or put this directory's parent on sys.path
and import it under the name ``fv2d_gb300`` through importlib.
"""
from . import build, meshgen  # noqa: F401
from .fv2d import (FP32, FP64, Batch, Case, Fv2dError, HostMesh, Solver, case_from_dict, library,  # noqa: F401
                   read_inputs)
