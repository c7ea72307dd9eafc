"""GB300-native (sm_103a) Single-Decoupling (SDM) two-state force.

Public surface:
  * :mod:`.capi`     ctypes binding of the C ABI (include/sdm_capi.h)
  * :class:`SDMForce` host mirror of the reference's SDM parameter API
  * :class:`LangevinIntegratorSDM` host mirror of the reference integrator
    (fused stochastic-dynamics step on the GPU)
  * :class:`SDMUtils` host mirror of the reference's restraint helpers
    (group-1 centroid and alignment restraints, evaluated on the GPU)
  * :mod:`.systems`  seeded synthetic systems
  * :mod:`.build`    in-tree build of the CUDA library
"""
from . import systems  # noqa: F401
from .capi import Handle, SdmError, load_library  # noqa: F401
from .force import LangevinIntegratorSDM, SDMForce, SDMUtils, force_from_system, integrator_from_system  # noqa: F401

__all__ = ["systems", "Handle", "SdmError", "load_library", "SDMForce", "LangevinIntegratorSDM", "SDMUtils",
           "force_from_system", "integrator_from_system"]
