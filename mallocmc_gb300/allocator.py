"""Host-side mirror of mallocMC::Allocator (src/include/mallocMC/allocator.hpp:97-242)
over the C ABI. Device memory for the workload helpers comes from torch
(plumbing only); every heap operation runs in libmallocmc_gb300.so.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .policies import AlignmentPolicies, CreationPolicies, DistributionPolicies, OOMPolicies, ReservePoolPolicies
from .policies import make_config


@dataclass
class HeapInfo:
    """allocator.hpp:77-81"""

    p: int
    size: int


def _stream_ptr(stream) -> int:
    if stream is None:
        import torch

        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Allocator:
    """Allocator<CreationPolicy, DistributionPolicy, OOMPolicy, ReservePoolPolicy, AlignmentPolicy>.

    Construction allocates the pool and initialises the heap (allocator.hpp:136-159,
    179-183; default size 8 MiB); close() or garbage collection frees it (:185-189).
    """

    def __init__(self, creation=None, distribution=None, oom=None, reserve_pool=None, alignment=None,
                 size: int = 8 * 1024 * 1024, device: int = 0, stream=None):
        self.creation = creation or CreationPolicies.Scatter()
        self.distribution = distribution or DistributionPolicies.XMallocSIMD(self.creation.pagesize)
        self.oom = oom or OOMPolicies.ReturnNull()
        self.reserve_pool = reserve_pool or ReservePoolPolicies.AlpakaBuf()
        self.alignment = alignment or AlignmentPolicies.Shrink()
        self.device = device
        self._cfg = make_config(self.creation, self.distribution, self.oom, self.alignment)
        self._h = ctypes.c_void_p()
        L.check(L.lib().mmc_heap_create(ctypes.byref(self._cfg), size, device, _stream_ptr(stream),
                                        ctypes.byref(self._h)), "Allocator")

    # -- lifetime -------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            L.lib().mmc_heap_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def destructiveResize(self, size: int, stream=None):
        """allocator.hpp:195-200"""
        L.check(L.lib().mmc_heap_destructive_resize(self._h, size, _stream_ptr(stream)), "destructiveResize")

    # -- reference API --------------------------------------------------------
    def getAllocatorHandle(self) -> L.MmcDeviceHandle:
        """allocator.hpp:202-206: the by-value device handle kernels receive."""
        d = L.MmcDeviceHandle()
        L.check(L.lib().mmc_heap_device_handle(self._h, ctypes.byref(d)), "getAllocatorHandle")
        return d

    def getAvailableSlots(self, slotSize: int, stream=None) -> int:
        """allocator.hpp:227-233 (pads, counts, waits)."""
        out = ctypes.c_uint()
        L.check(L.lib().mmc_available_slots(self._h, slotSize, _stream_ptr(stream), ctypes.byref(out)),
                "getAvailableSlots")
        return out.value

    def getAvailableSlotsAsync(self, slotSize: int, out_dev_ptr: int, stream=None):
        """Stream-ordered count into device memory (no host synchronisation)."""
        L.check(L.lib().mmc_available_slots_async(self._h, slotSize, _stream_ptr(stream), out_dev_ptr),
                "getAvailableSlotsAsync")

    def getHeapLocations(self):
        """allocator.hpp:235-241"""
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        L.check(L.lib().mmc_heap_locations(self._h, ctypes.byref(p), ctypes.byref(n)), "getHeapLocations")
        return [HeapInfo(p.value or 0, n.value)]

    def info(self, linebreak: str = " ") -> str:
        """allocator.hpp:214-223"""
        buf = ctypes.create_string_buffer(2048)
        L.check(L.lib().mmc_heap_info(self._h, buf, len(buf)), "info")
        return buf.value.decode().replace("\n", linebreak)

    # -- introspection --------------------------------------------------------
    @property
    def handle_ptr(self):
        return self._h

    def geometry(self) -> L.MmcGeometry:
        g = L.MmcGeometry()
        L.check(L.lib().mmc_heap_geometry(self._h, ctypes.byref(g)), "geometry")
        return g

    def error_flags(self, clear: bool = False, stream=None) -> int:
        f = ctypes.c_uint32()
        L.check(L.lib().mmc_heap_error(self._h, _stream_ptr(stream), ctypes.byref(f), int(clear)), "error_flags")
        return f.value

    def snapshot(self, stream=None):
        """(ptes[numpages, 3], regions, masks[numpages, maxOnPageMasks], header dict)."""
        g = self.geometry()
        ptes = np.zeros((g.numpages, 3), dtype=np.uint32)
        regions = np.zeros(g.numregions, dtype=np.uint32)
        masks = np.zeros((g.numpages, max(1, g.maxOnPageMasks)), dtype=np.uint32)
        hdr = np.zeros(3, dtype=np.uint32)
        L.check(L.lib().mmc_snapshot_metadata(self._h, _stream_ptr(stream), ptes.ctypes.data, regions.ctypes.data,
                                              masks.ctypes.data if g.maxOnPageMasks else None, hdr.ctypes.data),
                "snapshot")
        return ptes, regions, masks[:, : g.maxOnPageMasks], {
            "firstFreePageBased": int(hdr[0]), "firstfreeblock": int(hdr[1]), "pagebasedMutex": int(hdr[2])}

    def freemap(self, stream=None) -> np.ndarray:
        """The free-page bitmap as one bool per page (True: the bit is set,
        i.e. the page counts as free for the concurrent multi-page search)."""
        g = self.geometry()
        words = np.zeros((g.numpages + 31) // 32, dtype=np.uint32)
        L.check(L.lib().mmc_snapshot_freemap(self._h, _stream_ptr(stream), words.ctypes.data), "snapshot_freemap")
        bits = np.unpackbits(words.view(np.uint8), bitorder="little")
        return bits[: g.numpages].astype(bool)
