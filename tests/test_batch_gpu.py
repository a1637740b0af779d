"""Batched uneven jobs: one persistent, graph-captured launch against one
plain launch per job. Every job's result (pairs, nulls, pattern errors and the
XOR checksum of everything it read back) must be the same in both forms, i.e.
the same alone and in the mix, and the pairs must equal the host's count of the
cycle draws."""
import numpy as np
import pytest

from oracle.oracle import HeapConfig
from tests.test_parity_gpu import gpu_allocator
from tests.test_verify_gpu import assert_all_free

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_matches_plain_launches(use_graph):
    from mallocmc_gb300.batch import Batch, expected_pairs, make_jobs

    jobs = make_jobs(njobs=48, seed=11, tmin=32, tmax=8192)
    want = expected_pairs(jobs)
    cfg = HeapConfig(4096, 256 << 20, 16, 2, False)
    with gpu_allocator(cfg, 1 << 30) as alloc:
        b = Batch(alloc, jobs, persistent_blocks=0, use_graph=use_graph)
        b.run_plain()
        plain = b.stats()
        b.run()
        b.run()
        batched = b.stats()
        b.close()
        assert np.array_equal(plain[:, 0].astype(np.int64), want)
        assert int(plain[:, 1].sum()) == 0 and int(plain[:, 2].sum()) == 0
        assert np.array_equal(batched[:, 0].astype(np.int64), 2 * want)
        assert int(batched[:, 1].sum()) == 0 and int(batched[:, 2].sum()) == 0
        # two runs XOR their (identical) checksums away; one plain run keeps it
        assert int(batched[:, 3].astype(np.uint64).max()) == 0
        assert_all_free(alloc.snapshot())
        assert alloc.error_flags() == 0


def test_batch_checksums_equal_across_forms():
    from mallocmc_gb300.batch import Batch, make_jobs

    jobs = make_jobs(njobs=32, seed=12, tmin=32, tmax=4096)
    cfg = HeapConfig(16384, 256 << 20, 8, 2, False)
    with gpu_allocator(cfg, 1 << 30) as alloc:
        b = Batch(alloc, jobs, persistent_blocks=152 * 2, use_graph=True)
        b.run_plain()
        plain = b.stats()
        b.run()
        batched = b.stats()
        b.close()
        assert np.array_equal(plain, batched)


def test_batch_jobs_of_one_thread_and_zero_cycles():
    """Jobs of a single thread, thread counts off the 256-thread item grid, and
    threads with no cycles at all: the persistent form skips padding slots and
    empty threads and still matches the plain launches job by job."""
    from mallocmc_gb300.batch import Batch, expected_pairs, make_jobs

    jobs = make_jobs(njobs=40, seed=13, tmin=1, tmax=700, min_cycles=0, max_cycles=3)
    jobs[0].threads = 1
    jobs[7].threads = 257
    want = expected_pairs(jobs)
    cfg = HeapConfig(4096, 256 << 20, 16, 2, False)
    with gpu_allocator(cfg, 1 << 30) as alloc:
        b = Batch(alloc, jobs, persistent_blocks=152, use_graph=True)
        b.run_plain()
        plain = b.stats()
        b.run()
        batched = b.stats()
        b.close()
        assert np.array_equal(plain[:, 0].astype(np.int64), want)
        assert np.array_equal(plain, batched)
        assert_all_free(alloc.snapshot())
        assert alloc.error_flags() == 0


def test_batch_beyond_the_shared_job_table():
    """3000 jobs do not fit the per-block job columns in shared memory: the
    persistent form then flushes every thread's counters to the global table
    and still matches the plain launches job by job."""
    from mallocmc_gb300.batch import Batch, expected_pairs, make_jobs

    jobs = make_jobs(njobs=3000, seed=14, tmin=1, tmax=64, max_cycles=4)
    want = expected_pairs(jobs)
    cfg = HeapConfig(4096, 256 << 20, 16, 2, False)
    with gpu_allocator(cfg, 1 << 30) as alloc:
        b = Batch(alloc, jobs, persistent_blocks=304, use_graph=True)
        b.run_plain()
        plain = b.stats()
        b.run()
        batched = b.stats()
        b.close()
        assert np.array_equal(plain[:, 0].astype(np.int64), want)
        assert np.array_equal(plain, batched)
        assert alloc.error_flags() == 0


def test_full_size_batched_workload():
    """The bench's batched workload at its full size: 512 jobs (thread counts
    log-uniform in [32, 65536], 3.9 M job threads), one 16 GiB heap on the
    autotuned geometry. Every job's pair count equals the host's count of its
    cycle draws, no allocation fails, no pattern breaks, the persistent graph
    launch and the per-job launches give each job the same checksum, and the
    heap is empty afterwards."""
    from mallocmc_gb300 import AlignmentPolicies, Allocator, CreationPolicies, DistributionPolicies
    from mallocmc_gb300.autotune import GB300_TUNED as cfg
    from mallocmc_gb300.autotune import _accessblock
    from mallocmc_gb300.batch import Batch, expected_pairs, make_jobs

    heap = 16 << 30
    jobs = make_jobs(512, seed=3)
    want = expected_pairs(jobs)
    creation = CreationPolicies.Scatter(pagesize=cfg.pagesize, regionsize=cfg.regionsize,
                                        accessblocksize=_accessblock(heap, cfg.pagesize, cfg.accessblock_fraction),
                                        hashingK=cfg.hashingK, hashingDistMP=cfg.hashingDistMP)
    with Allocator(creation, DistributionPolicies.XMallocSIMD(cfg.pagesize), None, None,
                   AlignmentPolicies.Shrink(16), size=heap) as alloc:
        b = Batch(alloc, jobs, persistent_blocks=152 * cfg.blocks_per_sm, use_graph=True)
        b.run_plain()
        plain = b.stats()
        b.run()
        graph = b.stats()
        b.close()
        assert np.array_equal(plain[:, 0].astype(np.int64), want)
        assert int(plain[:, 1].sum()) == 0 and int(plain[:, 2].sum()) == 0
        assert np.array_equal(plain, graph)
        assert_all_free(alloc.snapshot(), pagesize=cfg.pagesize)
        assert alloc.error_flags() == 0
