"""ctypes binding of libmallocmc_gb300.so (the C ABI in include/mallocmc_gb300.h).

The library is required: there is no CPU or eager fallback. Importing the
binding without the built library raises with the build command.
"""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libmallocmc_gb300.so")

MMC_OK, MMC_ERR_CONFIG, MMC_ERR_CUDA, MMC_ERR_TIMEOUT, MMC_ERR_OOM, MMC_ERR_ARG = range(6)
MMC_DIST_NOOP, MMC_DIST_XMALLOCSIMD = 0, 1
MMC_OOM_RETURNNULL, MMC_OOM_FLAG = 0, 1
MMC_DEVERR_TIMEOUT, MMC_DEVERR_BADFREE, MMC_DEVERR_OOM, MMC_DEVERR_BADCMD, MMC_DEVERR_PAGEBASED = 0x1, 0x2, 0x4, 0x8, 0x10
MMC_SERVE_FREE, MMC_SERVE_LIVE, MMC_SERVE_DONE = 0, 1, 2

u32, u64, i64, vp = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int64, ctypes.c_void_p


class MmcConfig(ctypes.Structure):
    _fields_ = [
        ("pagesize", u32), ("regionsize", u32), ("wastefactor", u32), ("resetfreedpages", u32),
        ("accessblocksize", u64), ("hashingK", u32), ("hashingDistMP", u32), ("hashingDistWP", u32),
        ("hashingDistWPRel", u32), ("dataAlignment", u32), ("distribution", u32), ("oom_policy", u32),
        ("reference_quirks", u32),
    ]


class MmcDeviceHandle(ctypes.Structure):
    _fields_ = [
        ("state", vp), ("pages", vp), ("chunksize", vp), ("count", vp), ("bitmask", vp), ("regions", vp),
        ("freemap", vp), ("numpages", u32), ("numregions", u32), ("accessblocks", u32), ("pagesperblock", u32),
        ("pagesize", u32), ("regionsize", u32), ("wastefactor", u32), ("resetfreedpages", u32),
        ("hashingK", u32), ("hashingDistMP", u32), ("hashingDistWP", u32), ("hashingDistWPRel", u32),
        ("dataAlignment", u32), ("distribution", u32), ("oom_policy", u32), ("reference_quirks", u32),
        ("hierarchyThreshold", u32), ("minChunkSize", u32), ("paddedMinChunkSize", u32), ("maxOnPageMasks", u32),
    ]


class MmcGeometry(ctypes.Structure):
    _fields_ = [
        ("memsize", u64), ("numpages", u32), ("numregions", u32), ("accessblocks", u32), ("pagesperblock", u32),
        ("maxOnPageMasks", u32), ("hierarchyThreshold", u32), ("ptes_offset", u64), ("regions_offset", u64),
    ]


class MmcStressParams(ctypes.Structure):
    _fields_ = [
        ("blocks", u32), ("threads_per_block", u32), ("rounds", u32), ("lo", u32), ("hi", u32), ("step", u32),
        ("seed", u64), ("write_pattern", u32), ("reserved", u32),
    ]


class MmcJob(ctypes.Structure):
    _fields_ = [("threads", u32), ("item_begin", u32), ("seed", u64), ("mean_size", u32), ("max_size", u32),
                ("min_cycles", u32), ("max_cycles", u32)]


class MmcServeSlot(ctypes.Structure):
    _fields_ = [("id", u32), ("final_len", u32), ("len", u32), ("nchunks", u32), ("seed", u64), ("state", u32),
                ("failed", u32), ("checksum", u64)]


class MmcServeCmd(ctypes.Structure):
    _fields_ = [("kind", u32), ("slot", u32), ("id", u32), ("final_len", u32), ("seed", u64)]


class MmcFragParams(ctypes.Structure):
    _fields_ = [("blocks", u32), ("threads_per_block", u32), ("seed", u64), ("first_request", u64),
                ("small_lo", u32), ("small_hi", u32), ("large_lo", u32), ("large_hi", u32),
                ("large_permille", u32), ("waves", u32)]


# name -> (restype, argtypes); every function declared in include/mallocmc_gb300.h
SIGNATURES = {
    "mmc_config_default": (None, [ctypes.POINTER(MmcConfig)]),
    "mmc_heap_create": (ctypes.c_int, [ctypes.POINTER(MmcConfig), ctypes.c_size_t, ctypes.c_int, vp,
                                       ctypes.POINTER(vp)]),
    "mmc_heap_create_on_pool": (ctypes.c_int, [ctypes.POINTER(MmcConfig), vp, ctypes.c_size_t, ctypes.c_int, vp,
                                               ctypes.POINTER(vp)]),
    "mmc_heap_destroy": (ctypes.c_int, [vp]),
    "mmc_heap_destructive_resize": (ctypes.c_int, [vp, ctypes.c_size_t, vp]),
    "mmc_heap_device_handle": (ctypes.c_int, [vp, ctypes.POINTER(MmcDeviceHandle)]),
    "mmc_heap_locations": (ctypes.c_int, [vp, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_size_t)]),
    "mmc_heap_geometry": (ctypes.c_int, [vp, ctypes.POINTER(MmcGeometry)]),
    "mmc_heap_info": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_size_t]),
    "mmc_available_slots": (ctypes.c_int, [vp, ctypes.c_size_t, vp, ctypes.POINTER(ctypes.c_uint)]),
    "mmc_available_slots_async": (ctypes.c_int, [vp, ctypes.c_size_t, vp, vp]),
    "mmc_available_slots_noalloc": (ctypes.c_int, [ctypes.POINTER(MmcDeviceHandle), ctypes.c_size_t, ctypes.c_uint,
                                                   vp, vp]),
    "mmc_heap_error": (ctypes.c_int, [vp, vp, ctypes.POINTER(u32), ctypes.c_int]),
    "mmc_snapshot_metadata": (ctypes.c_int, [vp, vp, vp, vp, vp, vp]),
    "mmc_snapshot_freemap": (ctypes.c_int, [vp, vp, vp]),
    "mmc_heap_stats": (ctypes.c_int, [vp, vp, vp, ctypes.c_int]),
    "mmc_last_error": (ctypes.c_char_p, []),
    "mmc_run_program": (ctypes.c_int, [vp, vp, vp, i64, vp, vp]),
    "mmc_run_stress": (ctypes.c_int, [vp, ctypes.POINTER(MmcStressParams), vp, vp, vp]),
    "mmc_run_verify": (ctypes.c_int, [vp, u32, u32, vp, u32, vp, vp, vp]),
    "mmc_run_alloc_offsets": (ctypes.c_int, [vp, u32, u32, vp, u32, vp, vp]),
    "mmc_run_free_offsets": (ctypes.c_int, [vp, u32, u32, vp, u32, vp, vp, vp]),
    "mmc_oldmalloc_set_heap": (ctypes.c_int, [ctypes.c_size_t, ctypes.c_int]),
    "mmc_run_stress_oldmalloc": (ctypes.c_int, [ctypes.POINTER(MmcStressParams), vp, vp, vp]),
    "mmc_batch_create": (ctypes.c_int, [vp, ctypes.POINTER(MmcJob), u32, u32, ctypes.c_int, vp, ctypes.POINTER(vp)]),
    "mmc_batch_run": (ctypes.c_int, [vp, vp]),
    "mmc_batch_run_plain": (ctypes.c_int, [vp, vp]),
    "mmc_batch_stats": (ctypes.c_int, [vp, vp, vp, ctypes.c_int]),
    "mmc_batch_info": (ctypes.c_int, [vp, ctypes.POINTER(u32), ctypes.POINTER(u32), ctypes.POINTER(u64)]),
    "mmc_batch_destroy": (ctypes.c_int, [vp]),
    "mmc_serve_create": (ctypes.c_int, [vp, u32, u32, u32, u32, ctypes.POINTER(vp)]),
    "mmc_serve_queue": (ctypes.c_int, [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp),
                                       ctypes.POINTER(vp)]),
    "mmc_serve_tick": (ctypes.c_int, [vp, ctypes.c_int]),
    "mmc_serve_check_queue": (ctypes.c_int, [vp, u32, u32, u32]),
    "mmc_serve_pipeline": (ctypes.c_int, [vp, ctypes.c_int] + [ctypes.POINTER(vp)] * 6),
    "mmc_serve_launch": (ctypes.c_int, [vp, ctypes.c_int]),
    "mmc_serve_wait": (ctypes.c_int, [vp]),
    "mmc_serve_wait_buffer": (ctypes.c_int, [vp, ctypes.c_int]),
    "mmc_serve_destroy": (ctypes.c_int, [vp]),
    "mmc_run_fill": (ctypes.c_int, [vp, ctypes.POINTER(MmcFragParams), vp, vp, u64, vp, vp]),
    "mmc_run_free_list": (ctypes.c_int, [vp, vp, vp, vp, u64, vp, vp]),
    "mmc_run_verify_list": (ctypes.c_int, [vp, vp, vp, u64, vp, vp]),
    "mmc_atomic_peak": (ctypes.c_int, [vp, u64, u32, u32, u32, ctypes.c_int, ctypes.c_int, vp, vp]),
}

_lib = None
_stats_lib = None
STATS_LIB_PATH = os.path.join(PKG, "libmallocmc_gb300_stats.so")


class MallocMCError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"mallocMC status {status}: {msg}")
        self.status = status


def lib() -> ctypes.CDLL:
    """The loaded C-ABI library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is not built: run `python -m mallocmc_gb300.build` "
                               "(or __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def stats_lib() -> ctypes.CDLL:
    """The same C ABI built with the device event counters (MMC_DEVICE_STATS):
    mmc_heap_stats reports the MMC_STAT_* counts of heaps created through it."""
    global _stats_lib
    if _stats_lib is None:
        if not os.path.exists(STATS_LIB_PATH):
            raise RuntimeError(f"{STATS_LIB_PATH} is not built: run `python -m mallocmc_gb300.build`")
        L = ctypes.CDLL(STATS_LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _stats_lib = L
    return _stats_lib


def check(status: int, what: str = ""):
    if status != MMC_OK:
        msg = lib().mmc_last_error().decode(errors="replace")
        if status == MMC_ERR_CONFIG:
            raise ValueError(f"{what}: {msg}")
        raise MallocMCError(status, f"{what}: {msg}")
