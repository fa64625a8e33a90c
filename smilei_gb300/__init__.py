"""smilei_gb300 -- GB300-native (sm_103a) PIC-step hot path with Smilei's operator interfaces.

The compute path is libsmileigb300.so (hand-written CUDA behind the C ABI in
include/smilei_gb300.h).  ``operators`` mirrors the reference's operator
classes on one patch's arrays; ``simulation`` runs whole resident timesteps;
``namelist`` executes Smilei namelists against them.
"""
from ._lib import SmileiGPUError, lib, last_error  # noqa: F401

__version__ = "0.1.0"
