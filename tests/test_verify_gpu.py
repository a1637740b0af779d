"""verify_heap-style checks of concurrent GPU runs (reference: tests/verify_heap.cpp).

Concurrent placements depend on %smid/%warpid, so parity here is by
properties: every returned block lies inside the page area, honours the
alignment, overlaps no other live block, holds its per-thread pattern intact;
freeing everything returns the page-table counts and bitmasks and the on-page
masks to zero exactly; getAvailableSlots equals the oracle's count on the same
heap state (and, with resetfreedpages, its pre-run value).
"""
import numpy as np
import pytest

from oracle.oracle import HeapConfig, OracleHeap, mix64
from tests.test_parity_gpu import gpu_allocator

pytestmark = pytest.mark.gpu


def check_live_blocks(offs, sizes, numpages, pagesize, align=16):
    ok = offs >= 0
    o = offs[ok]
    s = ((sizes[ok].astype(np.int64) + align - 1) // align) * align
    assert np.all(o % align == 0), "misaligned block"
    assert np.all(o + s <= numpages * pagesize), "block outside the page area"
    order = np.argsort(o, kind="stable")
    o, s = o[order], s[order]
    assert np.all(o[:-1] + s[:-1] <= o[1:]), "overlapping live blocks"
    return int(ok.sum())


def used_mask_words(ptes, masks, pagesize=4096):
    """The on-page mask words in use: the last `segments` words of each page
    formatted with a chunk size <= HierarchyThreshold (Scatter.hpp:397-421);
    elsewhere the page tail is payload."""
    ht = (pagesize - 8) // 33
    n = masks.shape[1]
    out = []
    for c in np.unique(ptes[:, 0]):
        c = int(c)
        if c == 0 or c > ht:
            continue
        seg = c * 32 + 4
        full = min(32, pagesize // seg)
        add = min(31, ((pagesize - full * seg - 4) & 0xFFFFFFFF) // c) if full != 32 else 0
        segments = full + (1 if add > 0 else 0)
        rows = masks[ptes[:, 0] == c]
        out.append(rows[:, n - segments:])
    return np.concatenate([o.ravel() for o in out]) if out else np.zeros(0, dtype=np.uint32)


def assert_all_free(snap, pagesize=4096):
    ptes, regions, masks, hdr = snap
    assert int(ptes[:, 1].max(initial=0)) == 0, "page fill counts not back to zero"
    assert int(ptes[:, 2].max(initial=0)) == 0, "page bitmasks not back to zero"
    assert int(used_mask_words(ptes, masks, pagesize).max(initial=0)) == 0, "on-page masks not back to zero"
    assert hdr["pagebasedMutex"] == 0


@pytest.mark.parametrize("reset", [False, True])
def test_verify_workload_4x256(reset):
    """The plain verify run: 64 MiB, pagesize 4096, access block 8 MiB, XMallocSIMD,
    ReturnNull, Shrink<16>; 4 blocks x 256 threads; sizes from {16,32,64,128}."""
    from mallocmc_gb300.workloads import alloc_offsets, free_offsets

    cfg = HeapConfig(4096, 8 << 20, 16, 2, reset)
    seed = 12345
    n = 4 * 256
    sizes = (16 << (mix64(seed, np.arange(n), 0) % np.uint64(4)).astype(np.int64)).astype(np.uint32)
    with gpu_allocator(cfg, 64 << 20) as alloc:
        g = alloc.geometry()
        before = alloc.getAvailableSlots(16)
        ds, offs_t = alloc_offsets(alloc, 4, 256, sizes, seed)
        offs = offs_t.cpu().numpy()
        assert np.all(offs >= 0)
        check_live_blocks(offs, sizes, g.numpages, 4096)
        errors = free_offsets(alloc, 4, 256, ds, offs_t, seed)
        assert errors == 0
        snap = alloc.snapshot()
        assert_all_free(snap)
        after = alloc.getAvailableSlots(16)
        assert alloc.error_flags() == 0
    if reset:
        assert after == before
    else:
        oh = OracleHeap(cfg, 64 << 20)
        oh.load_state(snap[0], snap[1], snap[2])
        assert after == oh.available_slots(16)


def test_single_kernel_verify_and_damage_negative():
    """mmc_run_verify in one kernel, then the reference's negative test
    (verify_heap.cpp:399-405, 676-688): a corrupted word must be detected."""
    import torch

    from mallocmc_gb300.workloads import alloc_offsets, free_offsets, run_verify

    cfg = HeapConfig(4096, 8 << 20, 16, 2, False)
    n = 64 * 128
    rng = np.random.default_rng(3)
    sizes = (16 * rng.integers(1, 65, size=n)).astype(np.uint32)
    with gpu_allocator(cfg, 256 << 20) as alloc:
        offs, errors = run_verify(alloc, 64, 128, sizes, 99)
        assert errors == 0 and np.all(offs >= 0)
        ds, offs_t = alloc_offsets(alloc, 64, 128, sizes, 99)
        pool = alloc.getHeapLocations()[0].p
        victim = int(offs_t[1].item())

        class _Word:  # one u32 of the second block, seen through the CUDA array interface
            __cuda_array_interface__ = {"shape": (1,), "typestr": "<u4", "data": (pool + victim, False),
                                        "version": 3}

        torch.as_tensor(_Word(), device="cuda").fill_(5 * 750 - 1)
        torch.cuda.synchronize()
        assert free_offsets(alloc, 64, 128, ds, offs_t, 99) == 1
        assert_all_free(alloc.snapshot())


def test_stress_full_grid_small_heap():
    """Many rounds of malloc/write/verify/free from a full GPU grid."""
    import torch

    from mallocmc_gb300.workloads import run_stress

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    cfg = HeapConfig(4096, 64 << 20, 16, 2, False)
    with gpu_allocator(cfg, 1 << 30) as alloc:
        st = run_stress(alloc, sms * 4, 256, 20, 16, 1024, 16, seed=1)
        assert st["pairs"] == sms * 4 * 256 * 20
        assert st["nulls"] == 0 and st["bad"] == 0
        assert_all_free(alloc.snapshot())
        assert alloc.error_flags() == 0


def test_xmallocsimd_coalesces_in_lane_order():
    """All 32 lanes request 16 B: one chunk of 16 + 32*16 bytes per warp, the
    lane count at its head, lane k at base + 16 + 16k (XMallocSIMD.hpp:118-176)."""
    from mallocmc_gb300.workloads import alloc_offsets, free_offsets

    cfg = HeapConfig(4096, 8 << 20, 16, 2, False)
    n = 8 * 128
    sizes = np.full(n, 16, dtype=np.uint32)
    with gpu_allocator(cfg, 64 << 20) as alloc:
        ds, offs_t = alloc_offsets(alloc, 8, 128, sizes, 1)
        offs = offs_t.cpu().numpy().reshape(-1, 32)
        base = offs[:, :1] - 16
        assert np.array_equal(offs - base, np.tile(16 + 16 * np.arange(32), (offs.shape[0], 1)))
        ptes = alloc.snapshot()[0]
        # each warp's chunk is one fill slot of a page formatted for 16 + 512 bytes
        assert int(ptes[:, 1].sum()) == offs.shape[0]
        assert set(np.unique(ptes[ptes[:, 1] > 0, 0])) <= {528, 544}
        assert free_offsets(alloc, 8, 128, ds, offs_t, 1) == 0
        assert_all_free(alloc.snapshot())


def test_noop_distribution_does_not_coalesce():
    from mallocmc_gb300.workloads import alloc_offsets, free_offsets

    cfg = HeapConfig(4096, 8 << 20, 16, 2, False, xmallocsimd=False)
    n = 4 * 128
    sizes = np.full(n, 16, dtype=np.uint32)
    with gpu_allocator(cfg, 64 << 20) as alloc:
        ds, offs_t = alloc_offsets(alloc, 4, 128, sizes, 1)
        offs = offs_t.cpu().numpy()
        check_live_blocks(offs, sizes, alloc.geometry().numpages, 4096)
        assert int(alloc.snapshot()[0][:, 1].sum()) == n
        assert free_offsets(alloc, 4, 128, ds, offs_t, 1) == 0
        assert_all_free(alloc.snapshot())


def test_page_based_allocations_concurrent():
    """Multi-page requests from many threads (global mutex path, Scatter.hpp:824-866)."""
    from mallocmc_gb300.workloads import alloc_offsets, free_offsets

    cfg = HeapConfig(4096, 16 << 20, 16, 2, False)
    n = 8 * 64
    rng = np.random.default_rng(8)
    sizes = (16 * rng.integers(260, 1400, size=n)).astype(np.uint32)  # 4 KiB .. 22 KiB
    with gpu_allocator(cfg, 128 << 20) as alloc:
        g = alloc.geometry()
        ds, offs_t = alloc_offsets(alloc, 8, 64, sizes, 4)
        offs = offs_t.cpu().numpy()
        assert np.all(offs >= 0)
        check_live_blocks(offs, sizes, g.numpages, 4096)
        assert free_offsets(alloc, 8, 64, ds, offs_t, 4) == 0
        ptes, regions, masks, hdr = alloc.snapshot()
        assert int(ptes[:, 0].max()) <= 4096  # every multi-page run released
        assert_all_free((ptes, regions, masks, hdr))
        assert alloc.error_flags() == 0


def test_page_based_runs_above_256_pages_mixed_with_chunks():
    """Full warps whose lanes ask for 1-3 MiB runs (256-768 pages: the warp's
    claim spans several 256-page groups) next to lanes asking for 64-byte
    chunks: no overlap, patterns intact, everything released."""
    from mallocmc_gb300.workloads import alloc_offsets, free_offsets

    cfg = HeapConfig(4096, 256 << 20, 16, 2, False)
    n = 4 * 64
    rng = np.random.default_rng(11)
    big = (16 * rng.integers((1 << 20) // 16, (3 << 20) // 16, size=n)).astype(np.uint32)
    sizes = np.where(np.arange(n) % 2 == 0, big, 64).astype(np.uint32)
    with gpu_allocator(cfg, 1 << 30) as alloc:
        g = alloc.geometry()
        ds, offs_t = alloc_offsets(alloc, 4, 64, sizes, 12)
        offs = offs_t.cpu().numpy()
        assert np.all(offs >= 0)
        check_live_blocks(offs, sizes, g.numpages, 4096)
        assert free_offsets(alloc, 4, 64, ds, offs_t, 12) == 0
        ptes, regions, masks, hdr = alloc.snapshot()
        assert int(ptes[:, 0].max()) <= 4096
        assert_all_free((ptes, regions, masks, hdr))
        assert alloc.error_flags() == 0


def test_stress_warp_pattern_mode():
    """The warp-cooperative pattern mode writes and verifies every lane's whole
    block (512 bytes per instruction); counts and cleanliness as in the per-thread mode."""
    import torch

    from mallocmc_gb300.workloads import PATTERN_WARP, run_stress

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    cfg = HeapConfig(4096, 256 << 20, 16, 2, False)
    with gpu_allocator(cfg, 1 << 30) as alloc:
        st = run_stress(alloc, sms * 4, 256, 20, 16, 1024, 16, seed=9, write_pattern=PATTERN_WARP)
        assert st["pairs"] == sms * 4 * 256 * 20
        assert st["nulls"] == 0 and st["bad"] == 0
        assert_all_free(alloc.snapshot())
        assert alloc.error_flags() == 0


def _warp_pattern_checksum(sizes, seed, nthreads):
    """What the warp pattern's read-back adds up: lane l of a warp reads units
    l, l + 32, ... of every lane's block, sums (v.x ^ v.y) over them (u64, with
    wrap) across all rounds; the lanes' sums are XORed within the warp and the
    warps' results XORed together."""
    from mallocmc_gb300.seeds import mix64

    rounds = sizes.shape[0]
    total = np.uint64(0)
    with np.errstate(over="ignore"):
        for w in range(nthreads // 32):
            lane_sums = np.zeros(32, dtype=np.uint64)
            for r in range(rounds):
                t = np.arange(w * 32, w * 32 + 32, dtype=np.uint64)
                m = mix64(seed, t, r)
                for k in range(32):
                    i = np.arange(int(sizes[r, w * 32 + k]) // 16, dtype=np.uint64)
                    vx = m[k] + np.uint64(2) * i
                    np.add.at(lane_sums, (i % np.uint64(32)).astype(np.int64), vx ^ (vx + np.uint64(1)))
            x = np.uint64(0)
            for v in lane_sums:
                x ^= v
            total ^= x
    return int(total)


def test_stress_warp_pattern_reads_back_every_unit():
    """The warp pattern's read-back (staged through shared memory) sees every
    16-byte unit it wrote: the kernel's checksum of the values read equals the
    one computed from the sizes and seeds on the host."""
    from mallocmc_gb300.workloads import PATTERN_WARP, run_stress

    blocks, tpb, rounds, seed = 8, 256, 5, 77
    n = blocks * tpb
    rng = np.random.default_rng(5)
    sizes = (rng.integers(1, 65, size=(rounds, n)) * 16).astype(np.uint16)
    cfg = HeapConfig(4096, 64 << 20, 16, 2, False)
    with gpu_allocator(cfg, 256 << 20) as alloc:
        st = run_stress(alloc, blocks, tpb, rounds, 16, 1024, 16, seed=seed, write_pattern=PATTERN_WARP,
                        sizes=sizes.ravel())
        assert st["pairs"] == n * rounds and st["nulls"] == 0 and st["bad"] == 0
        assert st["checksum"] == _warp_pattern_checksum(sizes, seed, n)


@pytest.mark.parametrize("size,xmalloc", [(256, True), (1024, True), (4096, True), (48, False), (2000, False)])
def test_warp_uniform_sizes(size, xmalloc):
    """Every lane of every warp asks for the same size, the case the same-size
    group claim serves (one lane reserves and claims for the warp): patterns
    intact, every pair counted, everything free afterwards; small sizes under
    the Noop distribution keep the one-lane claim (hierarchical pages). Run
    with the reference's exact-pagesize leak fixed (reference_quirks off):
    with it, a 4096-byte block is never given back (the leak itself is
    pinned by the golden fixtures)."""
    import torch

    from mallocmc_gb300.workloads import PATTERN_WARP, run_stress

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    cfg = HeapConfig(4096, 256 << 20, 16, 2, False, xmallocsimd=xmalloc, reference_quirks=False)
    with gpu_allocator(cfg, 1 << 30) as alloc:
        st = run_stress(alloc, sms * 2, 256, 10, size, size, 16, seed=21, write_pattern=PATTERN_WARP)
        assert st["pairs"] == sms * 2 * 256 * 10, st
        assert st["nulls"] == 0 and st["bad"] == 0, st
        assert_all_free(alloc.snapshot())
        assert alloc.error_flags() == 0


def test_stress_full_size_steps_no_corruption():
    """The benchmark workload (8 GiB heap, SMs x 8 x 256 threads, 100 rounds of
    malloc / u64 pattern / verify / free) three times back to back: no block may
    ever be handed out twice (a pattern error), none may fail, and everything
    must be free afterwards."""
    import torch

    from mallocmc_gb300.workloads import run_stress

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    cfg = HeapConfig(4096, 2 << 30, 16, 2, False)
    with gpu_allocator(cfg, 8 << 30) as alloc:
        for step in range(3):
            st = run_stress(alloc, sms * 8, 256, 100, 16, 1024, 16, seed=100 + step)
            assert st["pairs"] == sms * 8 * 256 * 100, st
            assert st["nulls"] == 0 and st["bad"] == 0, st
        snap = alloc.snapshot()
        assert_all_free(snap)
        assert alloc.error_flags() == 0


@pytest.mark.parametrize("quirks", [True, False])
def test_page_based_hint_after_a_run_at_page_zero(quirks):
    """Multi-page runs allocated one after another by real thread ids (the
    lock-free search) fill a 64 MiB heap top-down, the last run ending at page
    0; one run is freed and the next multi-page malloc tries again. The
    reference stores page - 1 as the next search start, which wraps for a run
    at page 0 (Scatter.hpp:800-804) and no later free can lower it again
    (deallocPageBased's atomicMax, :885): the reference's mode reproduces the
    failing malloc, the fixed mode (reference_quirks = 0) serves it from the
    freed run. Every offset equals the oracle's serial run in the same mode."""
    from mallocmc_gb300.workloads import alloc_offsets, free_offsets, program_arrays

    cfg = HeapConfig(4096, 8 << 20, 16, 2, False, reference_quirks=quirks)
    heap = 64 << 20
    size = 232 * 4096  # 16240 pages = 70 runs of 232
    with gpu_allocator(cfg, heap) as alloc:
        g = alloc.geometry()
        runs = g.numpages // 232
        assert runs * 232 == g.numpages
        got = []
        for i in range(runs):
            ds, offs_t = alloc_offsets(alloc, 1, 1, np.array([size], dtype=np.uint32), i)
            got.append((ds, offs_t, i))
        offs = np.array([int(o.cpu().item()) for _, o, _ in got])
        assert np.all(offs >= 0) and offs[-1] == 0
        hint = alloc.snapshot()[3]["firstFreePageBased"]
        assert hint == (0xFFFFFFFF if quirks else 0)
        ds, offs_t, seed = got[9]
        assert free_offsets(alloc, 1, 1, ds, offs_t, seed) == 0
        _, again_t = alloc_offsets(alloc, 1, 1, np.array([size], dtype=np.uint32), 99)
        again = int(again_t.cpu().item())
        if quirks:
            assert again == -1
        else:
            assert again == int(offs[9])
        oh = OracleHeap(cfg, heap)
        ops = [("m", size)] * runs + [("f", 9), ("m", size)]
        kinds, args = program_arrays(ops)
        want = oh.run_program(kinds.tobytes(), args)
        oh.close()
        assert want[:runs].tolist() == offs.tolist()
        assert int(want[-1]) == again
        assert alloc.error_flags() == 0


def assert_freemap_consistent(alloc, max_false_positive=0.001):
    """The free-page bitmap against the page table: every page whose chunk size
    is 0 has its bit (a missed free page would hide runs from the multi-page
    search); a set bit on a used page (a free's late set) is allowed, rarely."""
    ptes = alloc.snapshot()[0]
    bits = alloc.freemap()
    free = ptes[:, 0] == 0
    assert not np.any(free & ~bits), f"{int((free & ~bits).sum())} free pages without their bit"
    assert int((bits & ~free).sum()) <= max(2, max_false_positive * len(free))


def test_freemap_tracks_the_page_table():
    """After chunked allocations (which format pages), concurrent multi-page
    allocations, their frees and a fill to out-of-memory, the bitmap the
    concurrent search reads agrees with the chunk sizes; after everything is
    freed, every page is free in both."""
    from mallocmc_gb300.workloads import alloc_offsets, free_offsets

    cfg = HeapConfig(4096, 16 << 20, 16, 2, False)
    rng = np.random.default_rng(5)
    with gpu_allocator(cfg, 128 << 20) as alloc:
        g = alloc.geometry()
        assert np.all(alloc.freemap())
        n = 8 * 128
        sizes = np.where(rng.random(n) < 0.5, 16 * rng.integers(1, 200, size=n),
                         16 * rng.integers(300, 20000, size=n)).astype(np.uint32)
        ds, offs_t = alloc_offsets(alloc, 8, 128, sizes, 3)
        offs = offs_t.cpu().numpy()
        check_live_blocks(offs, sizes, g.numpages, 4096)
        assert_freemap_consistent(alloc)
        assert free_offsets(alloc, 8, 128, ds, offs_t, 3) == 0
        assert_freemap_consistent(alloc)
        ptes = alloc.snapshot()[0]
        assert int(np.count_nonzero(ptes[:, 0] > 4096)) == 0
        # multi-page runs only, more than fit: some fail; then free what was allocated
        big = (16 * rng.integers(4096 // 16, (1 << 20) // 16, size=512)).astype(np.uint32)
        ds, offs_t = alloc_offsets(alloc, 4, 128, big, 4)
        offs = offs_t.cpu().numpy()
        assert (offs < 0).any() and (offs >= 0).any()
        check_live_blocks(offs, big, g.numpages, 4096)
        assert_freemap_consistent(alloc)
        assert free_offsets(alloc, 4, 128, ds, offs_t, 4) == 0
        assert_freemap_consistent(alloc)
        assert alloc.error_flags() == 0


def test_freemap_with_page_resets():
    """resetfreedpages: pages return to chunk size 0 when their last chunk is
    freed, and their bits come back."""
    from mallocmc_gb300.workloads import alloc_offsets, free_offsets

    cfg = HeapConfig(4096, 16 << 20, 16, 2, True)
    rng = np.random.default_rng(6)
    with gpu_allocator(cfg, 64 << 20) as alloc:
        for rnd in range(3):
            n = 16 * 256
            sizes = (16 * rng.integers(1, 128, size=n)).astype(np.uint32)
            ds, offs_t = alloc_offsets(alloc, 16, 256, sizes, rnd)
            assert_freemap_consistent(alloc)
            assert free_offsets(alloc, 16, 256, ds, offs_t, rnd) == 0
            assert_freemap_consistent(alloc)
        ptes = alloc.snapshot()[0]
        assert int(np.count_nonzero(ptes[:, 0])) == 0
        assert np.all(alloc.freemap())


def test_free_orders_the_threads_accesses_before_reuse():
    """Sixteen full-grid runs of per-thread write / verify / free on a 1 GiB
    heap: no thread may read another owner's data in its own block. Before the
    free issued a release fence, a thread's verify reads could be served after
    the next owner's writes (1 to 6 of 25 such runs found mismatches)."""
    import torch

    from mallocmc_gb300.workloads import PATTERN_THREAD, run_stress

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    cfg = HeapConfig(4096, 64 << 20, 16, 2, False)
    bad = 0
    for rep in range(16):
        with gpu_allocator(cfg, 1 << 30) as alloc:
            st = run_stress(alloc, sms * 4, 256, 20, 16, 1024, 16, seed=100 + rep, write_pattern=PATTERN_THREAD)
            assert st["pairs"] == sms * 4 * 256 * 20 and st["nulls"] == 0
            bad += st["bad"]
    assert bad == 0
