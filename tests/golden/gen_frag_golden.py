"""Generate tests/golden/frag_fill.json: the oracle's fill fractions for the
fragmentation workload (fill until the first NULL, free a seeded half, refill
until the next NULL) on the heap geometries the tests and the bench use.

The oracle (oracle/scatter_oracle.c, oc_run_fragmentation) is the CPU
restatement of the reference's Scatter heap, pinned to the reference's own
outputs by tests/golden/*.json. Serially, smid and warpid are 0, so the hash
distances hashingDistMP/WP/WPRel do not change these numbers; pagesize, access
block, region size and waste factor do. A 32 GiB heap takes about ten minutes
of one core, which is why the numbers are recorded here instead of being
recomputed by the bench.

Usage: python tests/golden/gen_frag_golden.py [--only-small]
"""
import json
import os
import sys
from concurrent.futures import ProcessPoolExecutor
from multiprocessing import get_context

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "frag_fill.json")

SEED = 42
SMALL = (16, 2048)
LARGE = (8192, 1 << 20)
LARGE_PERMILLE = 100
# (heap bytes, access block bytes); pagesize 4096, regionsize 16, wastefactor 2
GEOMETRIES = [(1 << 30, 256 << 20), (4 << 30, 256 << 20), (32 << 30, 256 << 20), (32 << 30, 1 << 30)]


def run(geom):
    sys.path.insert(0, ROOT)
    from oracle.oracle import HeapConfig, OracleHeap

    heap_bytes, ab = geom
    h = OracleHeap(HeapConfig(4096, ab, 16, 2, False), heap_bytes)
    r = h.run_fragmentation(SEED, SMALL, LARGE, LARGE_PERMILLE)
    h.close()
    return {"heap_bytes": heap_bytes, "pagesize": 4096, "accessblocksize": ab, "regionsize": 16, "wastefactor": 2,
            "phase1_allocs": r["phase1_allocs"], "phase1_live_bytes": r["phase1_live_bytes"],
            "freed": r["freed"], "phase2_allocs": r["phase2_allocs"], "final_live_bytes": r["final_live_bytes"],
            "phase1_fill": r["phase1_live_bytes"] / heap_bytes, "final_fill": r["final_live_bytes"] / heap_bytes,
            "oracle_seconds": r["micros"] / 1e6}


def main():
    geoms = [g for g in GEOMETRIES if g[0] <= (4 << 30)] if "--only-small" in sys.argv else GEOMETRIES
    # one at a time: the oracle touches every page of its pool (page tails are initialised)
    with ProcessPoolExecutor(max_workers=1, mp_context=get_context("spawn")) as ex:
        rows = list(ex.map(run, geoms))
    doc = {"seed": SEED, "small": list(SMALL), "large": list(LARGE), "large_permille": LARGE_PERMILLE,
           "generator": "oracle.oracle.OracleHeap.run_fragmentation", "geometries": rows}
    with open(OUT, "w") as f:
        json.dump(doc, f, indent=1)
    print(json.dumps(doc, indent=1))


if __name__ == "__main__":
    main()
