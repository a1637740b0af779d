"""The oracle (oracle/scatter_oracle.c) against the reference's own outputs.

Every fixture in tests/golden was produced by the unmodified reference
(alpaka CPU-serial) via tests/golden/gen_golden.py. The oracle must reproduce
each malloc offset, each getAvailableSlots value and each metadata snapshot
bit for bit before it may check the CUDA heap.
"""
import os

import numpy as np
import pytest

from oracle.oracle import REF_CONFIGS, OracleHeap
from tests.golden_util import digest, fixture_paths, load

CASES = [os.path.basename(p)[:-5] for p in fixture_paths()]


def replay(case):
    cfg = REF_CONFIGS[case["config"]]
    h = OracleHeap(cfg, case["heap_bytes"])
    assert h.numpages == case["numpages"]
    assert h.accessblocks == case["accessblocks"]
    assert h.max_on_page_masks == case["max_on_page_masks"]
    results, snaps, ptrs = [], [], []
    for kind, arg in case["ops"]:
        if kind == "m":
            off = h.malloc(arg)
            ptrs.append(off)
            results.append(off)
        elif kind == "f":
            h.free_offset(ptrs[arg])
            results.append(None)
        elif kind == "s":
            results.append(h.available_slots(arg))
        elif kind == "d":
            results.append(h.available_slots_accelerator(arg))
        elif kind == "S":
            ptes, regions, masks = h.snapshot()
            snaps.append((ptes, regions, masks, h.header()))
            results.append(None)
    return h, results, snaps


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    case = load(os.path.join(os.path.dirname(__file__), "golden", name + ".json"))
    _, results, snaps = replay(case)
    exp = case["results"]
    mism = [(i, case["ops"][i], results[i], exp[i]) for i in range(len(exp)) if exp[i] is not None and results[i] != exp[i]]
    assert not mism, f"{len(mism)} mismatches, first: {mism[:5]}"
    assert len(snaps) == len(case["snapshots"])
    for (ptes, regions, masks, hdr), want in zip(snaps, case["snapshots"]):
        assert hdr["firstFreePageBased"] == want["firstFreePageBased"]
        assert hdr["firstfreeblock"] == want["firstfreeblock"]
        assert hdr["pagebasedMutex"] == want["pagebasedMutex"]
        assert int(np.count_nonzero(ptes.any(axis=1))) == want["n_nonzero_ptes"]
        assert digest(ptes) == want["ptes_sha256"]
        assert digest(regions) == want["regions_sha256"]
        assert digest(masks) == want["masks_sha256"]


def test_known_answers_literal():
    """Hand-checked known answers (64 MiB heap, sizes 16..8192), independent of the fixture files."""
    h = OracleHeap(REF_CONFIGS["p4k_ab8m_r16_w2"], 64 << 20)
    assert h.numpages == 16240
    assert h.available_slots(16) == 4124960
    assert h.available_slots(4096) == 16240
    offs = [h.malloc(s) for s in (16, 32, 64, 128, 4096, 8192, 16, 1000)]
    assert offs == [3145728, 6291456, 3080192, 6160384, 7077888, 66510848, 3145744, 8126464]
    assert (h.available_slots(16), h.available_slots(4096), h.available_slots(8192)) == (4123306, 16232, 8113)


def test_heap_smaller_than_access_block_is_rejected():
    """The reference divides by zero here (Scatter.hpp:991-993); the oracle reports a config error."""
    with pytest.raises(ValueError):
        OracleHeap(REF_CONFIGS["p4k_ab8m_r16_w2"], 4 << 20)


def test_fragmentation_fixture_reproduces():
    """tests/golden/frag_fill.json (gen_frag_golden.py) holds the oracle's fill on
    the bench's fragmentation workload; the small geometry is recomputed here."""
    import json
    import os

    from oracle.oracle import HeapConfig, OracleHeap

    doc = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "frag_fill.json")))
    g = next(x for x in doc["geometries"] if x["heap_bytes"] == 1 << 30)
    h = OracleHeap(HeapConfig(g["pagesize"], g["accessblocksize"], g["regionsize"], g["wastefactor"], False),
                   g["heap_bytes"])
    r = h.run_fragmentation(doc["seed"], tuple(doc["small"]), tuple(doc["large"]), doc["large_permille"])
    for k in ("phase1_allocs", "phase1_live_bytes", "freed", "phase2_allocs", "final_live_bytes"):
        assert r[k] == g[k], k
    assert {x["heap_bytes"] for x in doc["geometries"]} >= {1 << 30, 32 << 30}
