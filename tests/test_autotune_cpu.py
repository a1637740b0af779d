"""The autotuner's search, on a synthetic cost instead of GPU timings: the
multi-start coordinate descent must find a configuration that a descent from
the reference defaults alone misses, and must skip failed candidates."""
from dataclasses import replace

import mallocmc_gb300.autotune as at


def test_multistart_finds_the_other_pagesize_basin(monkeypatch):
    # From the defaults (4096) every single-parameter move at pagesize 16384 looks
    # worse, but 16384 with regionsize 32 and the (7919, 101) primes is best.
    def cost(c):
        if c.pagesize == 65536:
            return None  # a failed candidate
        base = 3.0 if c.pagesize == 4096 else 3.5
        if c.pagesize == 16384 and c.regionsize == 32:
            base -= 0.6
        if c.pagesize == 16384 and (c.hashingK, c.hashingDistMP) == (7919, 101):
            base -= 0.6
        return base + 0.01 * abs(c.blocks_per_sm - 8)

    monkeypatch.setattr(at, "measure", lambda c, *a, **k: cost(c))
    best, ms, trace = at.autotune(jobs=None, heap_bytes=16 << 30, sms=152)
    assert best.pagesize == 16384 and best.regionsize == 32
    assert (best.hashingK, best.hashingDistMP) == (7919, 101)
    assert abs(ms - cost(best)) < 1e-12
    single, single_ms, _ = at.autotune(jobs=None, heap_bytes=16 << 30, sms=152, starts=[at.TuneConfig()])
    assert single.pagesize == 4096 and single_ms > ms
    assert any(t["ms"] is None for t in trace)
