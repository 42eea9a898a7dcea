"""GB300-native monodomain time step of cardiacFoam.

The compute path is libcardiac_gpu.so (hand-written sm_103a CUDA behind the C
ABI in include/cardiac_gpu.h); this package holds its Python bindings, the
mesh builder, the build driver and the cellML2foam-to-CUDA emitter.
"""
from .lib import (PRECISION_FP64, PRECISION_MIXED, FIELD_VM, FIELD_IION, FIELD_ACTIVATION,
                  FIELD_SOURCE, FIELD_VM_OLD, CfgError)

__all__ = ["PRECISION_FP64", "PRECISION_MIXED", "FIELD_VM", "FIELD_IION", "FIELD_ACTIVATION",
           "FIELD_SOURCE", "FIELD_VM_OLD", "CfgError"]
