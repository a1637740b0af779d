"""The bench's algorithmic-atomics model (bench.warp_atomics and the two
workloads built on it) against a lane-by-lane restatement of the same rules:
XMallocSIMD groups the active lanes below pagesize/32 when there are at least
two (malloc 3 atomics, free one subtraction per lane plus 3 on a hierarchical
chunk or 2), every other lane pays 3 + 3 or 3 + 2."""
import numpy as np

import bench


def _by_lanes(w, act, pagesize):
    ht = (pagesize - 8) // 33
    total = 0
    for sizes, on in zip(w.reshape(-1, 32), act.reshape(-1, 32)):
        co = [int(s) for s, a in zip(sizes, on) if a and s < pagesize // 32]
        grouped = len(co) >= 2
        if grouped:
            total += 3 + (3 if 16 + sum(co) <= ht else 2) + len(co)
        for s, a in zip(sizes, on):
            if not a or (grouped and s < pagesize // 32):
                continue
            total += 3 + (3 if max(int(s), 16) <= ht else 2)
    return total


def test_warp_atomics_matches_lane_by_lane():
    rng = np.random.default_rng(4)
    for pagesize in (4096, 16384):
        w = (16 * rng.integers(1, 80, size=(6, 5, 32))).astype(np.int64)
        act = rng.random((6, 5, 32)) < 0.7
        assert bench.warp_atomics(w, act, pagesize) == _by_lanes(w, act, pagesize)


def test_stress_model_counts_every_pair():
    sizes = bench.size_table(3, 256)
    work = bench.algorithmic_work(sizes)
    assert work["pairs"] == 3 * 256
    assert work["atomics"] == _by_lanes(sizes.astype(np.int64), np.ones(sizes.shape, bool), 4096)
    assert work["payload_bytes"] == 2 * int(sizes.astype(np.int64).sum())


def test_batched_model_counts_the_jobs_pairs():
    from mallocmc_gb300.batch import expected_pairs, make_jobs

    jobs = make_jobs(njobs=6, seed=5, tmin=1, tmax=300)
    w = bench.batched_algorithmic_atomics(jobs, 16384)
    assert w["pairs"] == int(expected_pairs(jobs).sum())
    assert 1.0 < w["atomics_per_pair"] < 7.0


def test_fragmentation_atomics_by_operation():
    """The fragmentation run's atomic count, operation by operation: 4 KiB
    pages, hierarchical chunks up to (4096 - 8) // 33 = 123 bytes."""
    from mallocmc_gb300.fragmentation import algorithmic_atomics

    sizes = [64, 2048, 4096, 8192, 12289]  # hierarchical, chunk, whole page, 2 pages, 4 pages
    assert algorithmic_atomics(sizes, [], 4096) == 3 + 3 + 3 + (2 + 1) + (4 + 1)
    # frees: 64 B (hierarchical: 3), 4096 B (a chunk of the page size: 2), the 4-page run (4 + 1)
    assert algorithmic_atomics(sizes, [0, 2, 4], 4096) == 17 + 3 + 2 + 5
    # an index past the successful mallocs is ignored
    assert algorithmic_atomics(sizes, [99], 4096) == 17
