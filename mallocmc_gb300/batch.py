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


def main(argv=None):
    """Run the uneven-job workload (make_jobs) on a fresh heap of the given size
    and geometry (default: autotune.GB300_TUNED), check every job's pair count,
    nulls and pattern errors, and print the milliseconds of each run.
    `--no-graph` launches the persistent kernel directly instead of replaying
    its graph (so a profiler sees a plain launch), `--plain` one launch per job."""
    import argparse
    import json
    import time

    import torch

    from .autotune import GB300_TUNED, _accessblock
    from .policies import AlignmentPolicies, CreationPolicies, DistributionPolicies

    ap = argparse.ArgumentParser(prog="python -m mallocmc_gb300.batch")
    ap.add_argument("--jobs", type=int, default=512)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--heap-gib", type=int, default=16)
    ap.add_argument("--runs", type=int, default=2)
    ap.add_argument("--pagesize", type=int, default=GB300_TUNED.pagesize)
    ap.add_argument("--regionsize", type=int, default=GB300_TUNED.regionsize)
    ap.add_argument("--hashingK", type=int, default=GB300_TUNED.hashingK)
    ap.add_argument("--hashingDistMP", type=int, default=GB300_TUNED.hashingDistMP)
    ap.add_argument("--accessblock-fraction", type=int, default=GB300_TUNED.accessblock_fraction)
    ap.add_argument("--blocks-per-sm", type=int, default=GB300_TUNED.blocks_per_sm)
    form = ap.add_mutually_exclusive_group()
    form.add_argument("--no-graph", action="store_true")
    form.add_argument("--plain", action="store_true")
    a = ap.parse_args(argv)

    heap_bytes = a.heap_gib << 30
    jobs = make_jobs(a.jobs, seed=a.seed)
    want = expected_pairs(jobs)
    creation = CreationPolicies.Scatter(pagesize=a.pagesize, regionsize=a.regionsize,
                                        accessblocksize=_accessblock(heap_bytes, a.pagesize, a.accessblock_fraction),
                                        hashingK=a.hashingK, hashingDistMP=a.hashingDistMP)
    alloc = Allocator(creation, DistributionPolicies.XMallocSIMD(a.pagesize), None, None,
                      AlignmentPolicies.Shrink(16), size=heap_bytes)
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    b = Batch(alloc, jobs, persistent_blocks=sms * a.blocks_per_sm, use_graph=not a.no_graph)
    ms = []
    for _ in range(a.runs):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.run_plain() if a.plain else b.run()
        torch.cuda.synchronize()
        ms.append(1e3 * (time.perf_counter() - t0))
    st = b.stats(clear=True)
    ok = (np.array_equal(st[:, 0].astype(np.int64), a.runs * want) and int(st[:, 1].sum()) == 0
          and int(st[:, 2].sum()) == 0)
    b.close()
    alloc.close()
    print(json.dumps({"ok": ok, "pairs_per_run": int(want.sum()), "ms_per_run_host": ms}))
    return 0 if ok else 1


if __name__ == "__main__":
    raise SystemExit(main())
