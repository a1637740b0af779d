"""The device event counters (MMC_STAT_*), read through mmc_heap_stats of the
library built with MMC_DEVICE_STATS (libmallocmc_gb300_stats.so). The counts
follow from the workloads: one chunked allocation per thread of a verify run
without XMallocSIMD, one multi-page allocation per thread asking for more than
a page, failures counted once the heap is full; the regular library keeps
every counter at zero."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CHUNKED, FIRST_PAGE, WALK_PAGES, REGION_FAIL, REGION_SKIP, SIZE_MISMATCH, PAGE_FULL, CHUNKED_FAIL = range(8)
PAGE_BASED, PAGE_SCAN, PAGE_LOST, PAGE_BASED_FAIL = 8, 9, 10, 11


def _heap(lib, heap_bytes, accessblock, distribution):
    from mallocmc_gb300 import _lib as L

    cfg = L.MmcConfig()
    lib.mmc_config_default(ctypes.byref(cfg))
    cfg.accessblocksize = accessblock
    cfg.distribution = distribution
    h = ctypes.c_void_p()
    assert lib.mmc_heap_create(ctypes.byref(cfg), heap_bytes, 0, None, ctypes.byref(h)) == L.MMC_OK, \
        lib.mmc_last_error()
    return h


def _stats(lib, h, clear=True):
    out = np.zeros(16, dtype=np.uint64)
    assert lib.mmc_heap_stats(h, None, out.ctypes.data, int(clear)) == 0
    return out


def _verify(lib, h, blocks, tpb, sizes, seed):
    import torch

    ds = torch.as_tensor(np.ascontiguousarray(sizes, dtype=np.uint32).view(np.int32)).cuda()
    offs = torch.zeros(blocks * tpb, dtype=torch.int64, device="cuda")
    err = torch.zeros(1, dtype=torch.int64, device="cuda")
    assert lib.mmc_run_verify(h, blocks, tpb, ds.data_ptr(), seed, offs.data_ptr(), err.data_ptr(), None) == 0
    torch.cuda.synchronize()
    return offs.cpu().numpy(), int(err.item())


def test_counters_follow_the_workload():
    from mallocmc_gb300 import _lib as L

    lib = L.stats_lib()
    h = _heap(lib, 64 << 20, 8 << 20, L.MMC_DIST_NOOP)
    try:
        _stats(lib, h)
        rng = np.random.default_rng(3)
        n = 4 * 256
        offs, bad = _verify(lib, h, 4, 256, rng.choice([16, 32, 64, 128], size=n), 7)
        s = _stats(lib, h)
        assert bad == 0 and np.all(offs >= 0)
        assert s[CHUNKED] == n and s[CHUNKED_FAIL] == 0
        assert 0 < s[FIRST_PAGE] <= n
        assert s[PAGE_BASED] == 0 and s[PAGE_SCAN] == 0
        # multi-page requests: one page-based allocation each, each search reads page words
        offs, bad = _verify(lib, h, 1, 64, np.full(64, 3 * 4096 + 16), 8)
        s = _stats(lib, h)
        assert bad == 0 and np.all(offs >= 0)
        assert s[PAGE_BASED] == 64 and s[PAGE_BASED_FAIL] == 0 and s[PAGE_SCAN] >= 64 * 4
        assert s[CHUNKED] == 0
        # more 1 MiB requests than the 64 MiB heap holds: the failures are counted
        offs, bad = _verify(lib, h, 1, 96, np.full(96, 1 << 20), 9)
        s = _stats(lib, h)
        assert int((offs < 0).sum()) == int(s[PAGE_BASED_FAIL]) > 0
        assert s[PAGE_BASED] == 96
    finally:
        lib.mmc_heap_destroy(h)


def test_regular_library_keeps_counters_at_zero():
    from mallocmc_gb300 import _lib as L

    lib = L.lib()
    h = _heap(lib, 64 << 20, 8 << 20, L.MMC_DIST_NOOP)
    try:
        _verify(lib, h, 2, 128, np.full(256, 64), 1)
        assert int(_stats(lib, h).sum()) == 0
    finally:
        lib.mmc_heap_destroy(h)
