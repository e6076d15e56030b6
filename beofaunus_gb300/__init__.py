"""GB300-native Metropolis energy-change path for Faunus (bjornstenqvist/beoFaunus).

Python front end over the C-ABI library ``libfaunus_gb300.so`` (CUDA kernels
for sm_103a plus the C++ host runtime). See include/faunus_gb300.h.
"""
from .params import (FG_MAX_TYPES, FG_MODEL_DH_LJ, FG_MODEL_EWALD_WCA, FG_MODEL_MULTIPOLE_RF,
                     FgParams, make_params)

__all__ = ["FgParams", "make_params", "FG_MODEL_EWALD_WCA", "FG_MODEL_DH_LJ",
           "FG_MODEL_MULTIPOLE_RF", "FG_MAX_TYPES"]
