"""Parity of the CUDA heap with the reference, through the C ABI.

1. Every golden fixture (produced by the unmodified reference, see
   tests/golden/gen_golden.py) is replayed by mmc_run_program: one device
   thread with the reference CPU backend's thread ids. Offsets, slot counts
   and metadata snapshots must be bit-identical.
2. Seeded random programs larger than the fixtures are compared with the
   oracle (oracle/scatter_oracle.c) op by op and snapshot by snapshot.
3. getAvailableSlots (host API, two-pass device scan) equals the oracle's
   count for the same heap state, including states produced on the GPU.
"""
import os

import numpy as np
import pytest

from oracle.oracle import REF_CONFIGS, HeapConfig, OracleHeap
from tests.golden_util import digest, fixture_paths, load

pytestmark = pytest.mark.gpu

CASES = [os.path.basename(p)[:-5] for p in fixture_paths()]


def gpu_allocator(cfg: HeapConfig, heap_bytes: int):
    from mallocmc_gb300 import Allocator, AlignmentPolicies, CreationPolicies, DistributionPolicies

    creation = CreationPolicies.Scatter(
        pagesize=cfg.pagesize, accessblocksize=cfg.accessblocksize, regionsize=cfg.regionsize,
        wastefactor=cfg.wastefactor, resetfreedpages=cfg.resetfreedpages, hashingK=cfg.hashingK,
        hashingDistMP=cfg.hashingDistMP, hashingDistWP=cfg.hashingDistWP, hashingDistWPRel=cfg.hashingDistWPRel,
        reference_quirks=cfg.reference_quirks)
    dist = DistributionPolicies.XMallocSIMD(cfg.pagesize) if cfg.xmallocsimd else DistributionPolicies.Noop()
    align = AlignmentPolicies.Shrink(cfg.data_alignment) if cfg.data_alignment > 1 else AlignmentPolicies.Noop()
    return Allocator(creation, dist, None, None, align, size=heap_bytes)


def snapshot_matches(snap, want):
    ptes, regions, masks, hdr = snap
    assert hdr["firstFreePageBased"] == want["firstFreePageBased"]
    assert hdr["firstfreeblock"] == want["firstfreeblock"]
    assert hdr["pagebasedMutex"] == want["pagebasedMutex"]
    assert int(np.count_nonzero(ptes.any(axis=1))) == want["n_nonzero_ptes"]
    assert digest(ptes) == want["ptes_sha256"]
    assert digest(regions) == want["regions_sha256"]
    assert digest(masks) == want["masks_sha256"]


@pytest.mark.parametrize("name", CASES)
def test_golden_fixture_bit_exact(name):
    from mallocmc_gb300.workloads import run_program

    case = load(os.path.join(os.path.dirname(__file__), "golden", name + ".json"))
    cfg = REF_CONFIGS[case["config"]]
    ops = [(k, a) for k, a in case["ops"]]
    snap_points = [i for i, (k, _) in enumerate(ops) if k == "S"]
    # the full program: every result
    with gpu_allocator(cfg, case["heap_bytes"]) as alloc:
        g = alloc.geometry()
        assert (g.numpages, g.accessblocks) == (case["numpages"], case["accessblocks"])
        out = run_program(alloc, ops)
        if snap_points and snap_points[-1] == len(ops) - 1:
            snapshot_matches(alloc.snapshot(), case["snapshots"][-1])
            assert alloc.error_flags() == 0
    exp = case["results"]
    mism = [(i, ops[i], int(out[i]), exp[i]) for i in range(len(ops)) if exp[i] is not None and int(out[i]) != exp[i]]
    assert not mism, f"{len(mism)} mismatches, first: {mism[:5]}"
    # intermediate snapshots: replay the prefix on a fresh heap
    for k, pos in enumerate(snap_points[:-1] if snap_points and snap_points[-1] == len(ops) - 1 else snap_points):
        with gpu_allocator(cfg, case["heap_bytes"]) as alloc:
            run_program(alloc, ops[:pos])
            snapshot_matches(alloc.snapshot(), case["snapshots"][k])


def _random_ops(rng, P, n):
    ops, live, nm = [], [], 0
    for _ in range(n):
        r = rng.random()
        if r < 0.4 and live:
            ops.append(("f", live.pop(int(rng.integers(len(live))))))
        elif r < 0.42:
            ops.append(("d" if rng.random() < 0.5 else "s", int(rng.choice([16, 48, 200, P // 2, P, 3 * P]))))
        else:
            c = rng.random()
            sz = int(rng.integers(1, P // 8)) if c < 0.6 else int(rng.integers(P // 8, P + 1)) if c < 0.92 else \
                int(rng.integers(P + 1, 5 * P))
            ops.append(("m", sz))
            live.append(nm)
            nm += 1
    return ops


@pytest.mark.parametrize("cfg_name,heap,seed,n", [
    ("p4k_ab8m_r16_w2", 48 << 20, 11, 20000),
    ("p4k_ab8m_r16_w2_reset", 32 << 20, 12, 20000),
    ("p16k_ab16m_r8_w2", 64 << 20, 13, 8000),
    ("p4k_ab4m_r8_w4_noop", 8 << 20, 14, 12000),
])
def test_random_programs_match_oracle(cfg_name, heap, seed, n):
    from mallocmc_gb300.workloads import run_program

    cfg = REF_CONFIGS[cfg_name]
    ops = _random_ops(np.random.default_rng(seed), cfg.pagesize, n)
    oh = OracleHeap(cfg, heap)
    want = []
    offs = []
    for k, a in ops:
        if k == "m":
            o = oh.malloc(a)
            offs.append(o)
            want.append(o)
        elif k == "f":
            oh.free_offset(offs[a])
            want.append(0)
        elif k == "s":
            want.append(oh.available_slots(a))
        else:
            want.append(oh.available_slots_accelerator(a))
    with gpu_allocator(cfg, heap) as alloc:
        out = run_program(alloc, ops)
        snap = alloc.snapshot()
    mism = np.nonzero(out != np.array(want, dtype=np.int64))[0]
    assert len(mism) == 0, [(int(i), ops[i], int(out[i]), want[i]) for i in mism[:5]]
    ptes, regions, masks = oh.snapshot()
    assert np.array_equal(snap[0], ptes)
    assert np.array_equal(snap[1], regions)
    assert np.array_equal(snap[2], masks)
    assert snap[3] == oh.header()


SLOT_SIZES = [0, 1, 15, 16, 17, 48, 100, 123, 124, 128, 1000, 2047, 2048, 4095, 4096, 4097, 8192, 12288, 40000,
              1 << 20]


@pytest.mark.parametrize("cfg_name,heap", [("p4k_ab8m_r16_w2", 64 << 20), ("p16k_ab16m_r8_w2", 64 << 20),
                                           ("p1k_ab1m_r32_w1_a8", 8 << 20), ("p64k_ab32m_r4_w2_reset", 96 << 20)])
def test_available_slots_fresh_heap(cfg_name, heap):
    cfg = REF_CONFIGS[cfg_name]
    oh = OracleHeap(cfg, heap)
    with gpu_allocator(cfg, heap) as alloc:
        for s in SLOT_SIZES:
            assert alloc.getAvailableSlots(s) == oh.available_slots(s), s


@pytest.mark.parametrize("mix", ["mixed", "warp_uniform"])
def test_available_slots_on_fragmented_state(mix):
    """A GPU-made, fragmented state (concurrent allocations with real thread
    ids) counted by the GPU scan and by the oracle on the same snapshot; in
    the warp-uniform case every warp's lanes ask for one size, so their chunks
    come from same-size group claims."""
    from mallocmc_gb300.workloads import alloc_offsets

    cfg = REF_CONFIGS["p4k_ab8m_r16_w2"]
    heap = 64 << 20
    rng = np.random.default_rng(5)
    n = 16 * 256
    choices = [16, 32, 48, 64, 128, 256, 600, 1000, 2048, 4096, 6000, 20000]
    if mix == "mixed":
        sizes = rng.choice(choices, size=n).astype(np.uint32)
    else:
        sizes = np.repeat(rng.choice([256, 600, 1000, 2048], size=n // 32), 32).astype(np.uint32)
    with gpu_allocator(cfg, heap) as alloc:
        alloc_offsets(alloc, 16, 256, sizes, 7)
        ptes, regions, masks, hdr = alloc.snapshot()
        got = {s: alloc.getAvailableSlots(s) for s in SLOT_SIZES}
    oh = OracleHeap(cfg, heap)
    oh.load_state(ptes, regions, masks)
    for s in SLOT_SIZES:
        assert got[s] == oh.available_slots(s), s
