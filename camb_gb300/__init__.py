"""GB300-native CAMB scalar-perturbation path (flat, adiabatic, scalar C_l).

The hot path -- per-k Einstein-Boltzmann evolution with Dormand-Prince 5(4) stepping,
line-of-sight projection onto spherical Bessel functions and the k-integral for the
C_l -- runs as CUDA kernels for sm_103a in libcambgpu.so; the Python surface mirrors
the reference's camb.get_results / CAMBdata power-spectrum calls.
"""
from ._lib import CAMBError, Tables, load
from .model import AccuracyParams, CAMBparams, set_params
from .results import (CAMBdata, get_matter_power_interpolator, get_results, get_results_batch,
                      get_results_batch_shared, get_results_stream, get_transfer_functions, get_transfer_functions_batch)

__all__ = ["CAMBError", "Tables", "load", "AccuracyParams", "CAMBparams", "set_params", "CAMBdata",
           "get_matter_power_interpolator", "get_results", "get_results_batch", "get_results_batch_shared", "get_results_stream", "get_transfer_functions",
           "get_transfer_functions_batch"]
