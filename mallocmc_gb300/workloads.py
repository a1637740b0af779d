"""Python drivers of the workload kernels exported by libmallocmc_gb300.so.

Device buffers come from torch (plumbing); the kernels are the library's.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L
from .allocator import Allocator, _stream_ptr


def _torch():
    import torch

    return torch


def program_arrays(ops):
    """Encode [(kind, arg)] with 'f' args as malloc indices into (kinds u8,
    args u64) with 'f' args as op indices, as mmc_run_program expects."""
    kinds = np.zeros(len(ops), dtype=np.uint8)
    args = np.zeros(len(ops), dtype=np.uint64)
    malloc_ops = []
    for i, (k, a) in enumerate(ops):
        kinds[i] = ord(k)
        if k == "m":
            malloc_ops.append(i)
            args[i] = a
        elif k == "f":
            args[i] = malloc_ops[a] if a < len(malloc_ops) else np.uint64(0xFFFFFFFFFFFFFFFF)
        else:
            args[i] = a
    return kinds, args


def run_program(alloc: Allocator, ops, stream=None) -> np.ndarray:
    """Replay an op program in one device thread with the reference CPU-serial
    thread ids. Returns per-op results (offset / -1 for 'm', counts for 's'/'d')."""
    torch = _torch()
    kinds, args = program_arrays(ops)
    dev = torch.device("cuda", alloc.device)
    dk = torch.from_numpy(kinds).to(dev)
    da = torch.from_numpy(args.view(np.int64)).to(dev)
    out = torch.zeros(len(ops), dtype=torch.int64, device=dev)
    L.check(L.lib().mmc_run_program(alloc.handle_ptr, dk.data_ptr(), da.data_ptr(), len(ops), out.data_ptr(),
                                    _stream_ptr(stream)), "run_program")
    torch.cuda.synchronize(dev)
    return out.cpu().numpy()


PATTERN_THREAD, PATTERN_WARP = 1, 2


def stress_params(blocks, threads_per_block, rounds, lo=16, hi=1024, step=16, seed=1, write_pattern=PATTERN_THREAD):
    """write_pattern: PATTERN_THREAD (each thread writes and verifies its own
    block) or PATTERN_WARP (the warp does its lanes' blocks together, coalesced)."""
    p = L.MmcStressParams()
    p.blocks, p.threads_per_block, p.rounds = blocks, threads_per_block, rounds
    p.lo, p.hi, p.step, p.seed = lo, hi, step, seed
    p.write_pattern = int(write_pattern)
    return p


def launch_stress(alloc: Allocator, params, sizes_dev_ptr, stats_dev_ptr, stream=None):
    L.check(L.lib().mmc_run_stress(alloc.handle_ptr, ctypes.byref(params), sizes_dev_ptr, stats_dev_ptr,
                                   _stream_ptr(stream)), "run_stress")


def run_stress(alloc: Allocator, blocks, threads_per_block, rounds, lo=16, hi=1024, step=16, seed=1,
               write_pattern=PATTERN_THREAD, sizes=None, stream=None) -> dict:
    torch = _torch()
    dev = torch.device("cuda", alloc.device)
    stats = torch.zeros(4, dtype=torch.int64, device=dev)
    sz = None
    if sizes is not None:
        sz = torch.as_tensor(np.ascontiguousarray(sizes, dtype=np.uint16).view(np.int16)).to(dev)
    p = stress_params(blocks, threads_per_block, rounds, lo, hi, step, seed, write_pattern)
    launch_stress(alloc, p, sz.data_ptr() if sz is not None else None, stats.data_ptr(), stream)
    torch.cuda.synchronize(dev)
    s = stats.cpu().numpy().view(np.uint64)
    return {"pairs": int(s[0]), "nulls": int(s[1]), "bad": int(s[2]), "checksum": int(s[3])}


def run_verify(alloc: Allocator, blocks, threads_per_block, sizes, seed, stream=None):
    torch = _torch()
    dev = torch.device("cuda", alloc.device)
    n = blocks * threads_per_block
    ds = torch.as_tensor(np.ascontiguousarray(sizes, dtype=np.uint32).view(np.int32)).to(dev)
    offs = torch.full((n,), -2, dtype=torch.int64, device=dev)
    err = torch.zeros(1, dtype=torch.int64, device=dev)
    L.check(L.lib().mmc_run_verify(alloc.handle_ptr, blocks, threads_per_block, ds.data_ptr(), seed, offs.data_ptr(),
                                   err.data_ptr(), _stream_ptr(stream)), "run_verify")
    torch.cuda.synchronize(dev)
    return offs.cpu().numpy(), int(err.item())


def alloc_offsets(alloc: Allocator, blocks, threads_per_block, sizes, seed, stream=None):
    torch = _torch()
    dev = torch.device("cuda", alloc.device)
    n = blocks * threads_per_block
    ds = torch.as_tensor(np.ascontiguousarray(sizes, dtype=np.uint32).view(np.int32)).to(dev)
    offs = torch.full((n,), -2, dtype=torch.int64, device=dev)
    L.check(L.lib().mmc_run_alloc_offsets(alloc.handle_ptr, blocks, threads_per_block, ds.data_ptr(), seed,
                                          offs.data_ptr(), _stream_ptr(stream)), "alloc_offsets")
    torch.cuda.synchronize(dev)
    return ds, offs


def free_offsets(alloc: Allocator, blocks, threads_per_block, ds, offs, seed, stream=None) -> int:
    torch = _torch()
    err = torch.zeros(1, dtype=torch.int64, device=offs.device)
    L.check(L.lib().mmc_run_free_offsets(alloc.handle_ptr, blocks, threads_per_block, ds.data_ptr(), seed,
                                         offs.data_ptr(), err.data_ptr(), _stream_ptr(stream)), "free_offsets")
    torch.cuda.synchronize(offs.device)
    return int(err.item())


def atomic_peak(buf_dev_ptr, words, blocks, threads_per_block, iters, returning, contended, sink_dev_ptr,
                stream=None):
    L.check(L.lib().mmc_atomic_peak(buf_dev_ptr, words, blocks, threads_per_block, iters, int(returning),
                                    int(contended), sink_dev_ptr, _stream_ptr(stream)), "atomic_peak")
