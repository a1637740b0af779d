"""Batched uneven allocation jobs (one persistent, graph-captured launch) over
the C ABI's mmc_batch_* entry points."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L
from .allocator import Allocator, _stream_ptr


def make_jobs(njobs: int = 512, seed: int = 3, tmin: int = 32, tmax: int = 65536, mean_size: int = 64,
              max_size: int = 4096, min_cycles: int = 1, max_cycles: int = 16):
    """The uneven-job workload: thread counts log-uniform in [tmin, tmax],
    geometric sizes (mean mean_size, cap max_size), cycles uniform per thread."""
    rng = np.random.default_rng(seed)
    threads = np.exp(rng.uniform(np.log(tmin), np.log(tmax), size=njobs)).astype(np.int64)
    jobs = (L.MmcJob * njobs)()
    for i in range(njobs):
        jobs[i].threads = int(threads[i])
        jobs[i].seed = int(rng.integers(1, 2**63))
        jobs[i].mean_size = mean_size
        jobs[i].max_size = max_size
        jobs[i].min_cycles = min_cycles
        jobs[i].max_cycles = max_cycles
    return jobs


def expected_pairs(jobs) -> np.ndarray:
    """Pairs each job performs (the cycle draws of the kernels, on the host)."""
    from .seeds import mix64

    out = np.zeros(len(jobs), dtype=np.int64)
    for i, j in enumerate(jobs):
        t = np.arange(j.threads, dtype=np.uint64)
        span = np.uint64(j.max_cycles - j.min_cycles + 1)
        cyc = j.min_cycles + ((mix64(j.seed, t, 0xC1C1E) >> np.uint64(32)) % span).astype(np.int64)
        out[i] = int(cyc.sum())
    return out


class Batch:
    def __init__(self, alloc: Allocator, jobs, persistent_blocks: int = 0, use_graph: bool = True, stream=None):
        self.alloc = alloc
        self.njobs = len(jobs)
        self._b = ctypes.c_void_p()
        L.check(L.lib().mmc_batch_create(alloc.handle_ptr, jobs, self.njobs, persistent_blocks, int(use_graph),
                                         _stream_ptr(stream), ctypes.byref(self._b)), "batch_create")

    def run(self, stream=None):
        L.check(L.lib().mmc_batch_run(self._b, _stream_ptr(stream)), "batch_run")

    def run_plain(self, stream=None):
        L.check(L.lib().mmc_batch_run_plain(self._b, _stream_ptr(stream)), "batch_run_plain")

    def stats(self, clear: bool = True, stream=None) -> np.ndarray:
        out = np.zeros((self.njobs, 4), dtype=np.uint64)
        L.check(L.lib().mmc_batch_stats(self._b, _stream_ptr(stream), out.ctypes.data, int(clear)), "batch_stats")
        return out

    def info(self):
        items, blocks, threads = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint64()
        L.check(L.lib().mmc_batch_info(self._b, ctypes.byref(items), ctypes.byref(blocks), ctypes.byref(threads)),
                "batch_info")
        return {"items": items.value, "blocks": blocks.value, "threads": threads.value}

    def close(self):
        if getattr(self, "_b", None):
            L.lib().mmc_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
