"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the UNMODIFIED reference headers (alpaka CPU-serial backend, built by
`make -C oracle ref REF=<reference tree>` into oracle/_ref/ref_harness) on seeded op programs and
stores the programs together with the reference's outputs: pool offsets of
every malloc, getAvailableSlots results (host and accelerator paths) and a
metadata snapshot (PTEs, region counters, on-page masks, header words).

Only this script needs the reference sources; the fixtures it writes are
committed so the tests run anywhere. Usage:  python tests/golden/gen_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.oracle import REF_CONFIGS, run_reference  # noqa: E402


def program_text(ops):
    lines = []
    for k, a in ops:
        lines.append("snap" if k == "S" else f"{k} {a}")
    return "\n".join(lines) + "\n"


def dense_snapshot(snap, numpages, numregions, nmask):
    ptes = np.zeros((numpages, 3), dtype=np.uint32)
    for i, c, n, b in snap["ptes"]:
        ptes[i] = (c, n, b)
    regions = np.zeros(numregions, dtype=np.uint32)
    for i, v in snap["regions"]:
        regions[i] = v
    masks = np.zeros((numpages, nmask), dtype=np.uint32)
    for i, back, v in snap["masks"]:
        masks[i, nmask - back] = v
    return ptes, regions, masks


def digest(arr: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(arr, dtype="<u4").tobytes()).hexdigest()


def random_program(rng, cfg, n_ops, live_cap=None):
    """A seeded mix of mallocs over every size class of the heap, frees of
    random live allocations and slot queries."""
    P = cfg.pagesize
    ht = (P - 8) // 33
    edge = [0, 1, 8, 15, 16, 17, 31, 32, 33, ht - 1, ht, ht + 1, P // 32 - 1, P // 32, P // 2, P - 16, P - 1, P,
            P + 1, 2 * P, 2 * P + 16]
    ops, live = [], []
    nm = 0
    for _ in range(n_ops):
        r = rng.random()
        if r < 0.33 and live:
            j = live.pop(int(rng.integers(len(live))))
            ops.append(("f", j))
        elif r < 0.36:
            q = int(rng.choice([16, 64, 128, 1000, P // 2, P, 2 * P, 3 * P + 5]))
            ops.append(("s" if rng.random() < 0.7 else "d", q))
        else:
            c = rng.random()
            if c < 0.45:
                sz = int(rng.integers(1, max(2, P // 16)))
            elif c < 0.70:
                sz = int(rng.integers(P // 16, P // 2))
            elif c < 0.80:
                sz = int(rng.integers(P // 2, P + 1))
            elif c < 0.90:
                sz = int(rng.integers(P + 1, 6 * P))
            else:
                sz = int(rng.choice(edge))
            ops.append(("m", sz))
            live.append(nm)
            nm += 1
    ops.append(("s", 16))
    ops.append(("s", P))
    ops.append(("S", 0))
    return ops


def fill_program(cfg, heap_bytes, seed, name):
    """Allocate until the first null (90% small, 10% multi-page), free a
    seeded 50% permutation of the live blocks, refill until the next null."""
    rng = np.random.default_rng(seed)
    P = cfg.pagesize

    def draw():
        if rng.random() < 0.9:
            return int(rng.integers(16, 2049))
        return int(np.exp(rng.uniform(np.log(2 * P), np.log(24 * P))))

    n1 = int(heap_bytes // 900) + 64
    phase1 = [("m", draw()) for _ in range(n1)]
    res = run_reference(name, heap_bytes, program_text(phase1 + [("s", 16)]))
    offs = [r[2] for r in res["results"] if r[0] == "m"]
    first_null = offs.index(-1) if -1 in offs else len(offs)
    phase1 = phase1[: first_null + 1]
    live = [i for i in range(first_null)]
    perm = rng.permutation(len(live))[: len(live) // 2]
    frees = [("f", live[int(i)]) for i in sorted(perm)]
    phase2 = [("m", draw()) for _ in range(n1 // 2 + 64)]
    head = phase1 + [("s", 16), ("s", 4 * P), ("S", 0)] + frees + [("s", 16)]
    # keep phase 2 up to 40 mallocs past its first null: every failing malloc
    # walks the whole heap, which is slow to replay in one device thread
    res = run_reference(name, heap_bytes, program_text(head + phase2))
    offs2 = [r[2] for r in res["results"][len(head):] if r[0] == "m"]
    cut = (offs2.index(-1) + 41) if -1 in offs2 else len(offs2)
    return head + phase2[:cut] + [("s", 16), ("s", 4 * P), ("S", 0)]


def make_case(name, cfg_name, heap_bytes, ops):
    cfg = REF_CONFIGS[cfg_name]
    res = run_reference(cfg_name, heap_bytes, program_text(ops))
    nmask = min(32, -(-cfg.pagesize // (32 * ((cfg.pagesize - 128) // 1024) + 4)))
    numpages = res["numpages"]
    numregions = numpages // cfg.regionsize
    snaps = []
    for s in res["snapshots"]:
        ptes, regions, masks = dense_snapshot(s, numpages, numregions, nmask)
        entry = {
            "ptes_sha256": digest(ptes),
            "regions_sha256": digest(regions),
            "masks_sha256": digest(masks),
            "n_nonzero_ptes": len(s["ptes"]),
            "firstFreePageBased": s["firstFreePageBased"],
            "firstfreeblock": s["firstfreeblock"],
            "pagebasedMutex": s["pagebasedMutex"],
        }
        if len(s["ptes"]) <= 400:
            entry["ptes_sparse"] = s["ptes"]
            entry["regions_sparse"] = s["regions"]
        snaps.append(entry)
    return {
        "name": name,
        "config": cfg_name,
        "heap_bytes": heap_bytes,
        "numpages": numpages,
        "accessblocks": res["accessblocks"],
        "numregions": numregions,
        "max_on_page_masks": nmask,
        "ops": [[k, int(a)] for k, a in ops],
        "results": [r[-1] if r[0] in ("m", "s", "d") else None for r in res["results"]],
        "snapshots": snaps,
    }


def main():
    cases = []
    # 1. the known-answer sequence (64 MiB, pagesize 4096, access block 8 MiB)
    ka = [("s", 16), ("s", 4096)] + [("m", s) for s in (16, 32, 64, 128, 4096, 8192, 16, 1000)] + \
         [("s", 16), ("s", 4096), ("s", 8192), ("d", 16), ("S", 0)]
    cases.append(make_case("known_answer", "p4k_ab8m_r16_w2", 64 << 20, ka))

    # 2. seeded random programs over every configuration
    heaps = {"p4k_ab8m_r16_w2": 64 << 20, "p4k_ab8m_r16_w2_reset": 64 << 20, "p4k_ab4m_r8_w4_noop": 16 << 20,
             "p16k_ab16m_r8_w2": 64 << 20, "p64k_ab32m_r4_w2_reset": 96 << 20, "p1k_ab1m_r32_w1_a8": 8 << 20}
    for i, (cfg_name, hb) in enumerate(heaps.items()):
        rng = np.random.default_rng(1000 + i)
        ops = random_program(rng, REF_CONFIGS[cfg_name], 3000)
        cases.append(make_case(f"random_{cfg_name}", cfg_name, hb, ops))

    # 3. the verify workload run serially: 1024 threads, each malloc(size in
    #    {16,32,64,128}) then free, slots(16) before and after (both reset settings)
    from oracle.oracle import mix64

    sizes = (16 * (1 << (mix64(12345, np.arange(1024), 0) % np.uint64(4)).astype(np.int64))).tolist()
    for cfg_name in ("p4k_ab8m_r16_w2", "p4k_ab8m_r16_w2_reset"):
        ops = [("s", 16)]
        for t, s in enumerate(sizes):
            ops += [("m", s), ("f", t)]
        ops += [("s", 16), ("S", 0)]
        cases.append(make_case(f"verify1024_{cfg_name}", cfg_name, 64 << 20, ops))

    # 4. exact-pagesize malloc/free cycles (the reference leaks one page per cycle)
    ops = [("s", 4096)] + sum([[("m", 4096), ("f", i)] for i in range(100)], []) + [("s", 4096), ("s", 16), ("S", 0)]
    cases.append(make_case("pagesize_cycles", "p4k_ab8m_r16_w2", 64 << 20, ops))

    # 5. size edge cases: zero, narrowing of sizes >= 2^32, larger than the heap
    ops = [("m", 0), ("m", (1 << 32) + 16), ("m", (1 << 32) - 1), ("m", 1 << 40), ("m", 80 << 20), ("m", 17),
           ("f", 1), ("f", 5), ("s", 0), ("d", 0), ("s", 1 << 32), ("S", 0)]
    cases.append(make_case("size_edges", "p4k_ab8m_r16_w2", 64 << 20, ops))

    # 6. fill until OOM, free half, refill (small heaps)
    for cfg_name, hb, seed in (("p4k_ab4m_r8_w4_noop", 12 << 20, 77), ("p4k_ab8m_r16_w2_reset", 24 << 20, 78),
                               ("p1k_ab1m_r32_w1_a8", 4 << 20, 79)):
        ops = fill_program(REF_CONFIGS[cfg_name], hb, seed, cfg_name)
        cases.append(make_case(f"fill_{cfg_name}", cfg_name, hb, ops))

    for c in cases:
        path = os.path.join(HERE, f"{c['name']}.json")
        with open(path, "w") as f:
            json.dump(c, f, separators=(",", ":"))
        print(f"{c['name']}: {len(c['ops'])} ops, numpages {c['numpages']}, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
