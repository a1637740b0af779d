"""The free-slot count that allocates nothing (mmc_available_slots_noalloc).

Callers that cannot call cudaMalloc (code inside a framework whose device
memory belongs to its own pool allocator, a plugin handed only the device
handle, a latency-bound host loop that cannot take cudaMalloc's device-wide
synchronisation) count free slots through this entry point, whose scan
scratch is a fixed 32 KiB device array instead of heap-owned memory.
Its counts must equal those of the regular entry point (mmc_available_slots) on
the same heap state, exactly, on two calls in a row. This file is named so
pytest collects it last; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_slot_count_matches_regular_entry_point():
    import torch

    from mallocmc_gb300 import _lib as L
    from mallocmc_gb300.workloads import alloc_offsets
    from oracle.oracle import REF_CONFIGS
    from tests.test_parity_gpu import gpu_allocator

    lib = L.lib()
    cfg = REF_CONFIGS["p4k_ab8m_r16_w2"]
    rng = np.random.default_rng(21)
    sizes = rng.choice([16, 48, 100, 256, 1000, 3000, 4096, 9000, 20000], size=16 * 256).astype(np.uint32)
    with gpu_allocator(cfg, 64 << 20) as alloc:
        alloc_offsets(alloc, 16, 256, sizes, 5)  # a fragmented, partly used heap
        handle = alloc.getAllocatorHandle()
        stream = torch.cuda.current_stream().cuda_stream
        out = torch.zeros(2, dtype=torch.int32, device="cuda")
        for slot in (0, 16, 100, 1000, 4096, 12288, 1 << 20):
            want = alloc.getAvailableSlots(slot)
            for k in range(2):  # two calls in a row share the static scratch
                st = lib.mmc_available_slots_noalloc(ctypes.byref(handle), slot, 0, stream, out.data_ptr() + 4 * k)
                assert st == L.MMC_OK, lib.mmc_last_error()
            torch.cuda.synchronize()
            got = out.cpu().numpy().view(np.uint32)
            assert int(got[0]) == want and int(got[1]) == want, (slot, got.tolist(), want)
        # an explicit scan width within the limit gives the same count; one beyond it is refused
        st = lib.mmc_available_slots_noalloc(ctypes.byref(handle), 16, 2048, stream, out.data_ptr())
        assert st == L.MMC_OK
        torch.cuda.synchronize()
        assert int(out.cpu().numpy().view(np.uint32)[0]) == alloc.getAvailableSlots(16)
        st = lib.mmc_available_slots_noalloc(ctypes.byref(handle), 16, 2049, stream, out.data_ptr())
        assert st == L.MMC_ERR_ARG
        assert b"exceeds the static scratch" in lib.mmc_last_error()
