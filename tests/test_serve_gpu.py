"""The continuous-batching request loop on the device-resident heap.

Every request's checksum (over all its elements, read back before its chunks
are freed) must equal the host's formula, whether it ran alone or in a mix of
requests admitted while others were on the GPU, in the batched (one graph
launch per tick) and in the per-request form. Afterwards the heap is clean."""
import numpy as np
import pytest

from oracle.oracle import HeapConfig
from tests.test_parity_gpu import gpu_allocator
from tests.test_verify_gpu import assert_all_free

pytestmark = pytest.mark.gpu


def _server_heap():
    return gpu_allocator(HeapConfig(65536, 512 << 20, 16, 2, False), 2 << 30)


def test_mix_and_alone_checksums_equal():
    from mallocmc_gb300.serve import Server, expected_checksum, make_requests

    arrivals, lengths, seeds = make_requests(96, rate=1e9, seed=7)
    want = np.array([expected_checksum(int(s), int(n)) for s, n in zip(seeds, lengths)], dtype=np.uint64)
    with _server_heap() as alloc:
        srv = Server(alloc, slots=64, max_chunks=128, step=64, queue_cap=256)
        mix = srv.run(arrivals, lengths, seeds, batched=True, realtime=False)
        assert mix["completed"] == len(arrivals)
        assert np.array_equal(mix["checksum"], want)
        per = srv.run(arrivals, lengths, seeds, batched=False, realtime=False)
        assert per["completed"] == len(arrivals)
        assert np.array_equal(per["checksum"], want)
        piped = srv.run(arrivals, lengths, seeds, batched=True, realtime=False, pipelined=True)
        assert piped["completed"] == len(arrivals)
        assert np.array_equal(piped["checksum"], want)
        for i in (0, 5, 17):
            alone = srv.run(arrivals[i:i + 1], lengths[i:i + 1], seeds[i:i + 1], batched=True, realtime=False)
            assert alone["checksum"][0] == want[i]
        srv.close()
        assert_all_free(alloc.snapshot(), pagesize=65536)
        assert alloc.error_flags() == 0


def test_tick_free_count_equals_get_available_slots():
    """A tick's free-chunk count (the fused count kernel: block sums totalled by
    the last block to finish) equals getAvailableSlots(16 KiB) on the same heap
    state, for the synchronous and the pipelined tick, on a heap that other
    blocks of several sizes (formatted pages of other chunk sizes, multi-page
    runs) partly fill; and again once they are freed."""
    from mallocmc_gb300.serve import Server
    from mallocmc_gb300.workloads import alloc_offsets, free_offsets

    rng = np.random.default_rng(12)
    n = 16 * 128
    sizes = rng.choice([64, 1024, 4096, 16384, 65536, 3 * 65536], size=n).astype(np.uint32)
    with gpu_allocator(HeapConfig(65536, 64 << 20, 16, 2, False), 512 << 20) as alloc:
        srv = Server(alloc, slots=64, max_chunks=16, step=64, queue_cap=128)
        ds, offs = alloc_offsets(alloc, 16, 128, sizes, 3)
        for rep in range(2):
            want = alloc.getAvailableSlots(16384)
            srv.queue_len[0] = 0
            srv.tick(batched=True)
            srv.wait()
            assert int(srv.free_chunks[0]) == want
            for b in (0, 1):
                srv._pipe[b]["qlen"][0] = 0
                srv.launch(b)
                srv.wait_buffer(b)
                assert int(srv._pipe[b]["free"][0]) == want
            if rep == 0:
                assert free_offsets(alloc, 16, 128, ds, offs, 3) == 0
        srv.close()
        assert alloc.error_flags() == 0


@pytest.mark.parametrize("pipelined", [False, True])
def test_admission_waits_for_free_chunks(pipelined):
    """A heap too small for all requests at once: admission must hold requests
    back until completions return chunks, and every request still completes."""
    from mallocmc_gb300.serve import Server, expected_checksum, make_requests

    arrivals, lengths, seeds = make_requests(40, rate=1e9, seed=8, median=8192, sigma=0.3)
    want = np.array([expected_checksum(int(s), int(n)) for s, n in zip(seeds, lengths)], dtype=np.uint64)
    with gpu_allocator(HeapConfig(65536, 8 << 20, 16, 2, False), 16 << 20) as alloc:
        srv = Server(alloc, slots=64, max_chunks=128, step=256, queue_cap=128)
        res = srv.run(arrivals, lengths, seeds, batched=True, realtime=False, pipelined=pipelined)
        assert res["completed"] == len(arrivals)
        assert np.array_equal(res["checksum"], want)
        # never more chunks promised than the heap held: some requests had to wait
        assert np.nanmax(res["admit"]) > 0.0
        srv.close()


def test_cut_short_run_drains_before_the_next():
    """A run stopped by its time limit with requests still growing drains them
    (their chunks freed, their slots released) before returning, so the next
    run starts on an empty slot table: its checksums are right and the heap
    ends clean."""
    from mallocmc_gb300.serve import Server, expected_checksum, make_requests

    arrivals, lengths, seeds = make_requests(64, rate=1e9, seed=9, median=16384, sigma=0.2)
    want = np.array([expected_checksum(int(s), int(n)) for s, n in zip(seeds, lengths)], dtype=np.uint64)
    with _server_heap() as alloc:
        srv = Server(alloc, slots=64, max_chunks=128, step=16, queue_cap=128)
        first = srv.run(arrivals, lengths, seeds, batched=True, realtime=False, max_seconds=0.002)
        assert first["completed"] < len(arrivals)
        assert not (srv.slots["state"] != 0).any()  # every slot free again
        again = srv.run(arrivals, lengths, seeds, batched=True, realtime=False)
        assert again["completed"] == len(arrivals)
        assert np.array_equal(again["checksum"], want)
        srv.close()
        assert_all_free(alloc.snapshot(), pagesize=65536)
        assert alloc.error_flags() == 0


def test_tick_refuses_a_bad_queue():
    """A tick whose host-written queue is out of range (length beyond the
    queue's capacity, a slot beyond the table, an unknown kind, an admission
    longer than a slot's chunks hold) is refused
    with MMC_ERR_ARG before anything is launched, in the synchronous and the
    pipelined form; a valid queue then ticks normally."""
    from mallocmc_gb300 import _lib as L
    from mallocmc_gb300.serve import Server

    with _server_heap() as alloc:
        srv = Server(alloc, slots=8, max_chunks=16, step=64, queue_cap=4)
        lib = L.lib()
        for batched in (1, 0):
            srv.queue_len[0] = 5
            assert lib.mmc_serve_tick(srv._s, batched) == L.MMC_ERR_ARG
            srv.queue_len[0] = 1
            srv.queue[0] = (1, 8, 0, 100, 1)
            assert lib.mmc_serve_tick(srv._s, batched) == L.MMC_ERR_ARG
            srv.queue[0] = (3, 0, 0, 100, 1)
            assert lib.mmc_serve_tick(srv._s, batched) == L.MMC_ERR_ARG
            srv.queue[0] = (1, 0, 0, 16 * 256 + 1, 1)  # longer than the slot's 16 chunks hold
            assert lib.mmc_serve_tick(srv._s, batched) == L.MMC_ERR_ARG
        pq = srv._pipe[0]["q"]
        pql = srv._pipe[0]["qlen"]
        pql[0] = 1
        pq["kind"][0], pq["slot"][0] = 1, 9
        assert lib.mmc_serve_launch(srv._s, 0) == L.MMC_ERR_ARG
        pq["slot"][0], pq["final_len"][0] = 1, 16 * 256 + 1
        assert lib.mmc_serve_launch(srv._s, 0) == L.MMC_ERR_ARG
        pql[0] = 0
        srv.queue[0] = (1, 2, 0, 100, 1)
        assert lib.mmc_serve_tick(srv._s, 1) == L.MMC_OK
        assert int(srv.slots["state"][2]) in (L.MMC_SERVE_LIVE, L.MMC_SERVE_DONE)
        srv.queue_len[0] = 0
        while int(srv.slots["state"][2]) != L.MMC_SERVE_DONE:
            assert lib.mmc_serve_tick(srv._s, 1) == L.MMC_OK
        srv.queue_len[0] = 1
        srv.queue[0] = (2, 2, 0, 0, 0)
        assert lib.mmc_serve_tick(srv._s, 1) == L.MMC_OK
        srv.close()
        assert alloc.error_flags() == 0


def test_serving_on_a_16_gib_heap_at_a_realistic_rate():
    """The serving configuration's shape on a 16 GiB heap of 64 KiB pages:
    Poisson arrivals at 20 k requests/s (simulated clock), lognormal lengths
    (median 1024, sigma 1, cap 32768), 4096 slots, pipelined graph ticks.
    Every request completes with the checksum it has alone, each of a few
    requests run alone matches, and the heap is empty afterwards."""
    from mallocmc_gb300 import AlignmentPolicies, Allocator, CreationPolicies, DistributionPolicies
    from mallocmc_gb300.serve import Server, expected_checksum, make_requests

    heap = 16 << 30
    creation = CreationPolicies.Scatter(pagesize=65536, accessblocksize=4 << 30, regionsize=16)
    arrivals, lengths, seeds = make_requests(4000, rate=20000, seed=20000)
    want = np.array([expected_checksum(int(s), int(n)) for s, n in zip(seeds, lengths)], dtype=np.uint64)
    with Allocator(creation, DistributionPolicies.XMallocSIMD(65536), None, None, AlignmentPolicies.Shrink(16),
                   size=heap) as alloc:
        srv = Server(alloc, slots=4096, max_chunks=128, step=64, queue_cap=8192)
        mix = srv.run(arrivals, lengths, seeds, batched=True, realtime=False, pipelined=True)
        assert mix["completed"] == len(arrivals)
        assert np.array_equal(mix["checksum"], want)
        for i in (0, 123, 3999):
            alone = srv.run(arrivals[i:i + 1], lengths[i:i + 1], seeds[i:i + 1], batched=True, realtime=False)
            assert alone["checksum"][0] == want[i] == mix["checksum"][i]
        srv.close()
        assert_all_free(alloc.snapshot(), pagesize=65536)
        assert alloc.error_flags() == 0


def test_command_line_serves_every_request():
    """python -m mallocmc_gb300.serve at 2 k requests/s for 0.2 s on a 4 GiB
    heap: every request completes with its checksum (exit status 0)."""
    from mallocmc_gb300.serve import main

    assert main(["--rate", "2000", "--seconds", "0.2", "--heap-gib", "4"]) == 0
