"""Fragmentation and large-allocation mix: fill until the first NULL, free a
seeded half of the live blocks, refill until the next NULL; report the fill
fraction (live requested bytes / heap bytes) and the throughput."""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _lib as L
from .allocator import Allocator, _stream_ptr


def frag_params(blocks, threads_per_block, seed, first_request=0, small=(16, 2048), large=(8192, 1 << 20),
                large_permille=100, waves=8):
    p = L.MmcFragParams()
    p.blocks, p.threads_per_block, p.seed, p.first_request = blocks, threads_per_block, seed, first_request
    p.small_lo, p.small_hi = small
    p.large_lo, p.large_hi = large
    p.large_permille, p.waves = large_permille, waves
    return p


def algorithmic_atomics(sizes, freed, pagesize: int) -> int:
    """Minimum global atomics of a fragmentation run's operations under the
    reference algorithm, for the successful mallocs of `sizes` and the frees of
    the entries `freed` indexes: a chunked malloc 3 (CAS chunk size, add count,
    or mask), a k-page malloc k CASes and the hint CAS; a chunked free 2 (3 on a
    hierarchical chunk, whose on-page mask is cleared too), a k-page free k
    CASes and the hint max. A malloc that fails is counted with none."""
    sizes = np.asarray(sizes, dtype=np.int64)
    freed = np.asarray(freed, dtype=np.int64)
    pages = -(-sizes // pagesize)
    atomics = int(np.where(sizes <= pagesize, 3, pages + 1).sum())
    fs = sizes[freed[freed < len(sizes)]]
    ht = (pagesize - 8) // 33
    atomics += int(np.where(fs <= pagesize, np.where(fs <= ht, 3, 2), -(-fs // pagesize) + 1).sum())
    return atomics


def mean_request_bytes(small=(16, 2048), large=(8192, 1 << 20), large_permille=100) -> float:
    """Expected size of one request: uniform small sizes, log-uniform large ones."""
    import math

    ms = (small[0] + small[1]) / 2.0
    ml = (large[1] - large[0]) / math.log(large[1] / large[0])
    return (1000 - large_permille) / 1000.0 * ms + large_permille / 1000.0 * ml


def run_fragmentation(alloc: Allocator, seed: int, blocks: int, threads_per_block: int = 256,
                      capacity: int = 1 << 22, small=(16, 2048), large=(8192, 1 << 20), large_permille=100,
                      stream=None, waves_per_call: int = 8, max_waves: int = 1 << 20, release: bool = False,
                      wave_fraction: float | None = 0.5, min_wave: int = 32) -> dict:
    """Phase 1 fills from request 0 in waves of concurrent requests until a
    wave meets a NULL; a seeded half of the live blocks is freed; phase 2
    continues with the next unused request index until the next NULL. Returns
    fill fractions, counts, timings and the tag-error count. With release,
    every block still live is then freed (its tags checked first).

    Wave sizes: with wave_fraction (the default), each wave is admitted by
    free memory, as the serving loop admits requests: it holds as many
    requests as wave_fraction of the heap's free bytes is expected to take
    (mean_request_bytes), at least min_wave and at most
    blocks * threads_per_block, rounded up to whole warps. Waves are large
    while the heap is empty and shrink as it fills, so the requests that meet
    the first NULL go out a few at a time, as in a serial run. With
    wave_fraction None every wave is blocks * threads_per_block requests."""
    import torch

    lib = L.lib()
    dev = torch.device("cuda", alloc.device)
    s = _stream_ptr(stream)
    ptrs = torch.zeros(capacity, dtype=torch.int64, device=dev)
    sizes = torch.zeros(capacity, dtype=torch.int32, device=dev)
    ctr = torch.zeros(8, dtype=torch.int64, device=dev)
    heap_bytes = alloc.getHeapLocations()[0].size
    out = {"heap_bytes": heap_bytes}

    T = blocks * threads_per_block
    per_request = mean_request_bytes(small, large, large_permille)

    def fill(first):
        """Waves from request `first` until the stop flag; returns (seconds,
        waves, requests issued)."""
        ctr[4] = 0
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        waves = issued = 0
        while waves < max_waves:
            if wave_fraction is None:
                p = frag_params(blocks, threads_per_block, seed, first + issued, small, large, large_permille,
                                waves_per_call)
                n, waves = waves_per_call * T, waves + waves_per_call
            else:
                free = max(0, heap_bytes - int(ctr[1].item()))
                n = min(T, max(min_wave, int(wave_fraction * free / per_request)))
                tpb = threads_per_block if n >= threads_per_block else 32
                nb = -(-n // tpb)
                n = nb * tpb
                p = frag_params(nb, tpb, seed, first + issued, small, large, large_permille, 1)
                waves += 1
            L.check(lib.mmc_run_fill(alloc.handle_ptr, ctypes.byref(p), ptrs.data_ptr(), sizes.data_ptr(),
                                     capacity, ctr.data_ptr(), s), "fill")
            issued += n
            if int(ctr[4].item()) != 0:
                break
        torch.cuda.synchronize(dev)
        return time.perf_counter() - t0, waves, issued

    t1, w1, issued1 = fill(0)
    c = ctr.cpu().numpy().view(np.uint64)
    n1, live1, req1 = int(c[0]), int(c[1]), int(c[2])
    out.update(phase1_allocs=n1, phase1_requests=req1, phase1_live_bytes=live1, phase1_fill=live1 / heap_bytes,
               phase1_seconds=t1)
    half = np.random.default_rng(seed).permutation(min(n1, capacity))[: n1 // 2].astype(np.uint32)
    idx = torch.from_numpy(half.view(np.int32)).to(dev)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    L.check(lib.mmc_run_free_list(alloc.handle_ptr, ptrs.data_ptr(), sizes.data_ptr(), idx.data_ptr(), len(half),
                                  ctr.data_ptr(), s), "free_list")
    torch.cuda.synchronize(dev)
    tf = time.perf_counter() - t0
    t2, w2, issued2 = fill(issued1)
    c = ctr.cpu().numpy().view(np.uint64)
    n_total, live2, req_total = int(c[0]), int(c[1]), int(c[2])
    L.check(lib.mmc_run_verify_list(alloc.handle_ptr, ptrs.data_ptr(), sizes.data_ptr(), min(n_total, capacity),
                                    ctr.data_ptr(), s), "verify_list")
    torch.cuda.synchronize(dev)
    c = ctr.cpu().numpy().view(np.uint64)
    ops = req_total + len(half)
    got = sizes[: min(n_total, capacity)].cpu().numpy().astype(np.int64)
    atomics = algorithmic_atomics(got, half, int(alloc.getAllocatorHandle().pagesize))
    out.update(freed=len(half), phase2_allocs=n_total - n1, final_live_bytes=live2, final_fill=live2 / heap_bytes,
               algorithmic_atomics=atomics, atomics_per_second=atomics / (t1 + tf + t2),
               tag_errors=int(c[3]), free_seconds=tf, phase2_seconds=t2,
               ops_per_second=ops / (t1 + tf + t2), list_overflow=n_total > capacity, max_wave_requests=T,
               waves=(w1, w2), requests_issued=(issued1, issued2),
               wave_sizing=("admitted by free memory: %g of the free bytes per wave, %d to %d requests"
                            % (wave_fraction, min_wave, T)) if wave_fraction is not None else "fixed")
    if release:
        n = min(n_total, capacity)
        every = torch.arange(n, dtype=torch.int32, device=dev)
        L.check(lib.mmc_run_free_list(alloc.handle_ptr, ptrs.data_ptr(), sizes.data_ptr(), every.data_ptr(), n,
                                      ctr.data_ptr(), s), "free_list")
        torch.cuda.synchronize(dev)
        c = ctr.cpu().numpy().view(np.uint64)
        out.update(released_live_bytes=int(c[1]), tag_errors=int(c[3]))
    return out


def main(argv=None):
    """Run the fragmentation workload once on a fresh heap (pagesize 4096,
    regionsize 16, wastefactor 2, the fill-tuned hash distances of
    autotune.GB300_FRAG_TUNED unless given) and print its fills, times and
    check results as one JSON line; exit status 1 if a tag was damaged or a
    block was not given back."""
    import argparse
    import json

    import torch

    from .autotune import GB300_FRAG_TUNED, FragConfig, frag_allocator

    ap = argparse.ArgumentParser(prog="python -m mallocmc_gb300.fragmentation")
    ap.add_argument("--heap-gib", type=float, default=32.0)
    ap.add_argument("--accessblock-mib", type=int, default=256)
    ap.add_argument("--seed", type=int, default=42)
    ap.add_argument("--blocks-per-sm", type=int, default=2, help="a wave holds at most SMs x this x 256 requests")
    ap.add_argument("--hash", default=None, help="hashingDistMP,WP,WPRel (default: the tuned distances)")
    a = ap.parse_args(argv)

    cfg = FragConfig(*[int(x) for x in a.hash.split(",")]) if a.hash else GB300_FRAG_TUNED
    heap_bytes = int(a.heap_gib * (1 << 30))
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    alloc = frag_allocator(heap_bytes, a.accessblock_mib << 20, cfg)
    try:
        r = run_fragmentation(alloc, a.seed, sms * a.blocks_per_sm, 256, capacity=1 << 23, release=True)
    finally:
        alloc.close()
    ok = r["tag_errors"] == 0 and r["released_live_bytes"] == 0 and not r["list_overflow"]
    keys = ("phase1_fill", "final_fill", "phase1_seconds", "phase2_seconds", "ops_per_second", "waves", "tag_errors")
    print(json.dumps({"ok": ok, **{k: r[k] for k in keys}}))
    return 0 if ok else 1


if __name__ == "__main__":
    raise SystemExit(main())
