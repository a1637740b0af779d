"""The reference's policy classes as Python values.

Names and parameters follow src/include/mallocMC/ (creationPolicies/,
distributionPolicies/, oOMPolicies/, reservePoolPolicies/, alignmentPolicies/);
the namespaces are classes so `DistributionPolicies.Noop` and
`AlignmentPolicies.Noop` stay distinct as in C++.
"""
from __future__ import annotations

from dataclasses import dataclass

from . import _lib as L


class CreationPolicies:
    @dataclass(frozen=True)
    class Scatter:
        """Scatter<HeapConfig, HashConfig> (creationPolicies/Scatter.hpp:56-85, 106-207).
        reference_quirks keeps the reference's exact-pagesize free and page-based
        underflow behaviour (default); False selects the fixed behaviour."""

        pagesize: int = 4096
        accessblocksize: int = 2 * 1024 * 1024 * 1024
        regionsize: int = 16
        wastefactor: int = 2
        resetfreedpages: bool = False
        hashingK: int = 38183
        hashingDistMP: int = 17497
        hashingDistWP: int = 1
        hashingDistWPRel: int = 1
        reference_quirks: bool = True
        providesAvailableSlots = True  # Scatter.hpp:117

        @staticmethod
        def classname() -> str:
            return "Scatter"


class DistributionPolicies:
    @dataclass(frozen=True)
    class XMallocSIMD:
        """XMallocSIMD<Config> (distributionPolicies/XMallocSIMD.hpp:76-185)."""

        pagesize: int = 4096
        code = L.MMC_DIST_XMALLOCSIMD

    @dataclass(frozen=True)
    class Noop:
        """distributionPolicies/Noop.hpp:46-72."""

        code = L.MMC_DIST_NOOP


class OOMPolicies:
    @dataclass(frozen=True)
    class ReturnNull:
        """oOMPolicies/ReturnNull.hpp:44-57."""

        code = L.MMC_OOM_RETURNNULL

    @dataclass(frozen=True)
    class BadAllocException:
        """oOMPolicies/BadAllocException.hpp:50-74. On the device the reference
        asserts; here the failure sets MMC_DEVERR_OOM (read with
        Allocator.error_flags) and the call returns NULL, so no kernel traps."""

        code = L.MMC_OOM_FLAG


class ReservePoolPolicies:
    @dataclass(frozen=True)
    class AlpakaBuf:
        """reservePoolPolicies/AlpakaBuf.hpp:38-61: the heap owns a cudaMalloc'd pool."""


class AlignmentPolicies:
    @dataclass(frozen=True)
    class Shrink:
        """Shrink<Config> (alignmentPolicies/Shrink.hpp:80-146)."""

        dataAlignment: int = 16

        def __post_init__(self):
            a = self.dataAlignment
            if a == 0 or (a & (a - 1)) != 0:
                raise ValueError("dataAlignment must also be a power of 2")  # Shrink.hpp:103-106

        def applyPadding(self, n: int) -> int:
            clear = self.dataAlignment - 1
            return ((n & 0xFFFFFFFF) + clear) & ~clear & 0xFFFFFFFF

    @dataclass(frozen=True)
    class Noop:
        """alignmentPolicies/Noop.hpp:47-65."""

        dataAlignment = 1

        @staticmethod
        def applyPadding(n: int) -> int:
            return n & 0xFFFFFFFF


def make_config(creation, distribution, oom, alignment) -> L.MmcConfig:
    """Combine policies into the C config; enforces PolicyCheck2
    (mallocMC_constraints.hpp:84-88): Scatter and XMallocSIMD share a pagesize."""
    if not isinstance(creation, CreationPolicies.Scatter):
        raise TypeError("only CreationPolicies.Scatter is implemented on the GPU heap")
    if isinstance(distribution, DistributionPolicies.XMallocSIMD) and distribution.pagesize != creation.pagesize:
        raise ValueError("Pagesize must be the same when combining Scatter and XMallocSIMD")
    c = L.MmcConfig()
    c.pagesize = creation.pagesize
    c.regionsize = creation.regionsize
    c.wastefactor = creation.wastefactor
    c.resetfreedpages = int(creation.resetfreedpages)
    c.accessblocksize = creation.accessblocksize
    c.hashingK = creation.hashingK
    c.hashingDistMP = creation.hashingDistMP
    c.hashingDistWP = creation.hashingDistWP
    c.hashingDistWPRel = creation.hashingDistWPRel
    c.dataAlignment = alignment.dataAlignment
    c.distribution = distribution.code
    c.oom_policy = oom.code
    c.reference_quirks = int(creation.reference_quirks)
    return c
