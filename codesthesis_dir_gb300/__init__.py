"""GB300-native (CUDA sm_103a) implementation of the time-step hot path of
M. King's rotating-annulus / Rayleigh-Benard convection codes
(martin-king/codesthesis_dir): the velocity / streamfunction multigrid
Poisson solves and the compact-scheme Dufort-Frankel transport of vorticity
and temperature with its wall boundary conditions, behind a C ABI that the
Fortran drivers can call (include/gb300_convection.h).
"""
from .lib import (BATCH_FP64, BATCH_MIXED, FIELDS, GBError, SMOOTHER_LEX, SMOOTHER_ZEBRA,  # noqa: F401
                  load)

__all__ = ["load", "GBError", "FIELDS", "SMOOTHER_LEX", "SMOOTHER_ZEBRA", "BATCH_FP64", "BATCH_MIXED"]
