"""mallocmc_gb300 — a GB300-native (sm_103a) ScatterAlloc device heap.

The heap and every kernel live in libmallocmc_gb300.so (C ABI:
include/mallocmc_gb300.h; device API: include/mallocMC/scatter_device.cuh).
This package is the host-side mirror of mallocMC's Allocator/policy interface
(src/include/mallocMC/allocator.hpp) over that ABI.
"""
from .allocator import Allocator, HeapInfo
from .policies import AlignmentPolicies, CreationPolicies, DistributionPolicies, OOMPolicies, ReservePoolPolicies

__all__ = ["Allocator", "HeapInfo", "AlignmentPolicies", "CreationPolicies", "DistributionPolicies", "OOMPolicies",
           "ReservePoolPolicies"]
__version__ = "2.6.0"
