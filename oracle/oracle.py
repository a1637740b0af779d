"""ctypes front end of the oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: the CPU restatement of the reference's Scatter heap
(src/include/mallocMC/creationPolicies/Scatter.hpp) that the CUDA heap is
checked against. Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg import this module; the product package never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")


class OcConfig(ctypes.Structure):
    _fields_ = [
        ("pagesize", ctypes.c_uint32),
        ("regionsize", ctypes.c_uint32),
        ("wastefactor", ctypes.c_uint32),
        ("resetfreedpages", ctypes.c_uint32),
        ("accessblocksize", ctypes.c_uint64),
        ("hashingK", ctypes.c_uint32),
        ("hashingDistMP", ctypes.c_uint32),
        ("hashingDistWP", ctypes.c_uint32),
        ("hashingDistWPRel", ctypes.c_uint32),
        ("dataAlignment", ctypes.c_uint32),
        ("reference_quirks", ctypes.c_uint32),
    ]


@dataclass(frozen=True)
class HeapConfig:
    """Scatter/Shrink template parameters as runtime values (Scatter.hpp:56-85,
    Shrink.hpp:62-65). data_alignment 0 selects AlignmentPolicies::Noop;
    xmallocsimd selects the XMallocSIMD distribution policy (1) or Noop (0)."""

    pagesize: int = 4096
    accessblocksize: int = 2 << 30
    regionsize: int = 16
    wastefactor: int = 2
    resetfreedpages: bool = False
    hashingK: int = 38183
    hashingDistMP: int = 17497
    hashingDistWP: int = 1
    hashingDistWPRel: int = 1
    data_alignment: int = 16
    xmallocsimd: bool = True
    reference_quirks: bool = True

    def to_oc(self) -> OcConfig:
        return OcConfig(self.pagesize, self.regionsize, self.wastefactor, int(self.resetfreedpages),
                        self.accessblocksize, self.hashingK, self.hashingDistMP, self.hashingDistWP,
                        self.hashingDistWPRel, self.data_alignment, int(self.reference_quirks))


# The configurations the reference harness is instantiated for (names match
# oracle/ref_harness.cpp and the tests/golden fixtures).
REF_CONFIGS = {
    "p4k_ab8m_r16_w2": HeapConfig(4096, 8 << 20, 16, 2, False),
    "p4k_ab8m_r16_w2_reset": HeapConfig(4096, 8 << 20, 16, 2, True),
    "p4k_ab4m_r8_w4_noop": HeapConfig(4096, 4 << 20, 8, 4, False, 7919, 101, 3, 2, 0, False),
    "p16k_ab16m_r8_w2": HeapConfig(16384, 16 << 20, 8, 2, False),
    "p64k_ab32m_r4_w2_reset": HeapConfig(65536, 32 << 20, 4, 2, True),
    "p1k_ab1m_r32_w1_a8": HeapConfig(1024, 1 << 20, 32, 1, False, data_alignment=8),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"oracle library missing: {LIB_PATH} (run `make -C oracle`)")
        L = ctypes.CDLL(LIB_PATH)
        vp, u32, u64, i64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int64
        L.oc_heap_create.argtypes = [ctypes.POINTER(OcConfig), u64, ctypes.POINTER(vp)]
        L.oc_heap_create.restype = ctypes.c_int
        L.oc_heap_destroy.argtypes = [vp]
        L.oc_malloc.argtypes = [vp, u64]
        L.oc_malloc.restype = vp
        L.oc_free.argtypes = [vp, vp]
        L.oc_available_slots.argtypes = [vp, u64]
        L.oc_available_slots.restype = u32
        L.oc_available_slots_accelerator.argtypes = [vp, u64]
        L.oc_available_slots_accelerator.restype = u32
        for name in ("oc_numpages", "oc_accessblocks", "oc_numregions", "oc_max_on_page_masks",
                     "oc_hierarchy_threshold"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = u32
        L.oc_pool.argtypes = [vp]
        L.oc_pool.restype = vp
        L.oc_header.argtypes = [vp, vp]
        L.oc_snapshot_ptes.argtypes = [vp, vp]
        L.oc_snapshot_regions.argtypes = [vp, vp]
        L.oc_snapshot_masks.argtypes = [vp, vp]
        L.oc_load_state.argtypes = [vp, vp, vp, vp]
        L.oc_run_program.argtypes = [vp, vp, vp, i64, vp]
        L.oc_mix64.argtypes = [u64, u64, u64]
        L.oc_mix64.restype = u64
        L.oc_run_stress.argtypes = [vp, u64, u32, u64, u32, u32, u32, ctypes.c_int,
                                    ctypes.POINTER(u64), ctypes.POINTER(u64), ctypes.POINTER(ctypes.c_double)]
        L.oc_run_stress.restype = u64
        L.oc_frag_size.argtypes = [u64, u64, u32, u32, u32, u32, u32]
        L.oc_frag_size.restype = u32
        L.oc_run_fragmentation.argtypes = [vp, u64, u32, u32, u32, u32, u32, vp]
        _lib = L
    return _lib


class OracleHeap:
    """One Scatter heap restated on the CPU (see oracle/scatter_oracle.h)."""

    def __init__(self, cfg: HeapConfig, heap_bytes: int):
        self.cfg = cfg
        self.heap_bytes = heap_bytes
        h = ctypes.c_void_p()
        rc = lib().oc_heap_create(ctypes.byref(cfg.to_oc()), heap_bytes, ctypes.byref(h))
        if rc != 0:
            raise ValueError(f"oracle heap create failed (code {rc})")
        self._h = h

    def close(self):
        if self._h:
            lib().oc_heap_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def numpages(self) -> int:
        return lib().oc_numpages(self._h)

    @property
    def accessblocks(self) -> int:
        return lib().oc_accessblocks(self._h)

    @property
    def numregions(self) -> int:
        return lib().oc_numregions(self._h)

    @property
    def max_on_page_masks(self) -> int:
        return lib().oc_max_on_page_masks(self._h)

    @property
    def hierarchy_threshold(self) -> int:
        return lib().oc_hierarchy_threshold(self._h)

    def pool(self) -> int:
        return lib().oc_pool(self._h)

    def malloc(self, n: int) -> int:
        """Pool offset of the allocation, or -1 (ReturnNull)."""
        p = lib().oc_malloc(self._h, n)
        return -1 if not p else p - self.pool()

    def free_offset(self, off: int):
        if off >= 0:
            lib().oc_free(self._h, self.pool() + off)

    def available_slots(self, n: int) -> int:
        return lib().oc_available_slots(self._h, n)

    def available_slots_accelerator(self, n: int) -> int:
        return lib().oc_available_slots_accelerator(self._h, n)

    def run_program(self, kinds: bytes, args) -> np.ndarray:
        k = np.frombuffer(kinds, dtype=np.uint8).copy()
        a = np.asarray(args, dtype=np.uint64)
        out = np.zeros(len(k), dtype=np.int64)
        lib().oc_run_program(self._h, k.ctypes.data, a.ctypes.data, len(k), out.ctypes.data)
        return out

    def header(self):
        out = np.zeros(3, dtype=np.uint32)
        lib().oc_header(self._h, out.ctypes.data)
        return {"firstFreePageBased": int(out[0]), "firstfreeblock": int(out[1]), "pagebasedMutex": int(out[2])}

    def snapshot(self):
        """(ptes[numpages,3], regions[numregions], masks[numpages, maxOnPageMasks])."""
        n = self.numpages
        ptes = np.zeros((n, 3), dtype=np.uint32)
        lib().oc_snapshot_ptes(self._h, ptes.ctypes.data)
        regions = np.zeros(self.numregions, dtype=np.uint32)
        lib().oc_snapshot_regions(self._h, regions.ctypes.data)
        masks = np.zeros((n, max(self.max_on_page_masks, 1)), dtype=np.uint32)
        if self.max_on_page_masks:
            lib().oc_snapshot_masks(self._h, masks.ctypes.data)
        return ptes, regions, masks[:, : self.max_on_page_masks]

    def load_state(self, ptes, regions=None, masks=None):
        ptes = np.ascontiguousarray(ptes, dtype=np.uint32)
        r = None if regions is None else np.ascontiguousarray(regions, dtype=np.uint32)
        m = None if masks is None else np.ascontiguousarray(masks, dtype=np.uint32)
        lib().oc_load_state(self._h, ptes.ctypes.data, None if r is None else r.ctypes.data,
                            None if m is None else m.ctypes.data)

    def run_fragmentation(self, seed: int, small=(16, 2048), large=(8192, 1 << 20), large_permille: int = 100):
        """The reference's fill / free-half / refill on this heap (see scatter_oracle.h)."""
        out = np.zeros(6, dtype=np.uint64)
        lib().oc_run_fragmentation(self._h, seed, small[0], small[1], large[0], large[1], large_permille,
                                   out.ctypes.data)
        keys = ("phase1_allocs", "phase1_live_bytes", "freed", "phase2_allocs", "final_live_bytes", "micros")
        return {k: int(v) for k, v in zip(keys, out)}

    def run_stress(self, vthreads: int, rounds: int, seed: int, lo: int, hi: int, step: int, workers: int):
        nulls, bad, secs = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_double()
        pairs = lib().oc_run_stress(self._h, vthreads, rounds, seed, lo, hi, step, workers,
                                    ctypes.byref(nulls), ctypes.byref(bad), ctypes.byref(secs))
        return {"pairs": int(pairs), "nulls": int(nulls.value), "bad": int(bad.value), "seconds": secs.value}


def mix64(seed: int, a, b):
    """numpy twin of oc_mix64 (SplitMix64 finaliser over a counter)."""
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) + np.asarray(a, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
             + np.asarray(b, dtype=np.uint64) * np.uint64(0xD1B54A32D192ED03))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def run_reference(config_name: str, heap_bytes: int, program_text: str) -> dict:
    """Run the reference harness (oracle/_ref, built only where the reference
    sources exist) on an op program; returns its JSON document."""
    import json

    if not os.path.exists(REF_HARNESS):
        raise RuntimeError("reference harness not built (oracle/_ref/ref_harness)")
    r = subprocess.run([REF_HARNESS, config_name, str(heap_bytes)], input=program_text, capture_output=True,
                       text=True, check=True)
    return json.loads(r.stdout)
