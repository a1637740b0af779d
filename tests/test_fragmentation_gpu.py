"""Fragmentation and large-allocation mix on the device heap: fill until the
first NULL, free a seeded half, refill until the next NULL (a mix of chunked
and multi-page requests). The fill fraction at out-of-memory must reach the
oracle's (the reference's algorithm run serially on the same seed and heap
geometry), every block must keep its tags, and freeing everything must leave
the page table empty."""
import numpy as np
import pytest

from oracle.oracle import HeapConfig, OracleHeap
from tests.test_verify_gpu import assert_all_free

pytestmark = pytest.mark.gpu

SEED = 42


def _allocator(heap, ab, mp, wp, wprel):
    from mallocmc_gb300 import AlignmentPolicies, Allocator, CreationPolicies, DistributionPolicies

    creation = CreationPolicies.Scatter(pagesize=4096, accessblocksize=ab, hashingDistMP=mp, hashingDistWP=wp,
                                        hashingDistWPRel=wprel)
    return Allocator(creation, DistributionPolicies.XMallocSIMD(4096), None, None, AlignmentPolicies.Shrink(16),
                     size=heap)


@pytest.mark.parametrize("heap,ab,blocks,tpb", [(1 << 30, 256 << 20, 152, 64), (1 << 30, 64 << 20, 304, 256)])
def test_fill_reaches_the_oracle(heap, ab, blocks, tpb):
    """Hash distances for fill (hashingDistMP 1, WP 0): starts of one size class
    stay within a few hundred pages, so chunk pages stay clustered the way the
    serial run's are; the oracle's serial fill does not depend on them."""
    from mallocmc_gb300.fragmentation import run_fragmentation

    want = OracleHeap(HeapConfig(4096, ab, 16, 2, False), heap).run_fragmentation(SEED)
    with _allocator(heap, ab, 1, 0, 0) as alloc:
        r = run_fragmentation(alloc, SEED, blocks, tpb, release=True)
        assert r["tag_errors"] == 0 and not r["list_overflow"]
        assert alloc.error_flags() == 0
        assert r["released_live_bytes"] == 0
        assert_all_free(alloc.snapshot())
        ptes = alloc.snapshot()[0]
        # no page-based run is left claimed: a page is either unformatted or a formatted chunk page
        assert int(np.count_nonzero(ptes[:, 0] > 4096)) == 0
    assert r["final_fill"] >= want["final_live_bytes"] / heap
    assert r["phase1_fill"] >= 0.97 * want["phase1_live_bytes"] / heap


def test_default_hash_keeps_tags_and_frees_everything():
    from mallocmc_gb300.fragmentation import run_fragmentation

    with _allocator(512 << 20, 64 << 20, 17497, 1, 1) as alloc:
        r = run_fragmentation(alloc, SEED + 1, 304, 256, release=True)
        assert r["tag_errors"] == 0 and r["released_live_bytes"] == 0
        assert r["phase1_allocs"] > 0 and r["phase2_allocs"] > 0
        assert alloc.error_flags() == 0
        assert_all_free(alloc.snapshot())
        assert int(np.count_nonzero(alloc.snapshot()[0][:, 0] > 4096)) == 0
