"""Serving-style request loop on the device-resident heap (continuous batching).

Requests arrive (Poisson), wait until the heap has enough free 16 KiB slots for
their expected chunks (the device's getAvailableSlots count, refreshed every
tick, minus the chunks already promised to live requests) and a server slot is
free, then grow on the device tick by tick; completed requests hand back their
checksum and their slot. Latency is admit-to-completion, measured on the host
clock at the ticks that admit and complete a request.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _lib as L
from .allocator import Allocator

ELEMS_PER_CHUNK = 256
SLOT_DTYPE = np.dtype([("id", "<u4"), ("final_len", "<u4"), ("len", "<u4"), ("nchunks", "<u4"), ("seed", "<u8"),
                       ("state", "<u4"), ("failed", "<u4"), ("checksum", "<u8")])
CMD_DTYPE = np.dtype([("kind", "<u4"), ("slot", "<u4"), ("id", "<u4"), ("final_len", "<u4"), ("seed", "<u8")])
DONE_DTYPE = np.dtype([("slot", "<u4"), ("reserved", "<u4"), ("checksum", "<u8")])


def make_requests(n: int, rate: float, seed: int = 5, median: int = 1024, sigma: float = 1.0, cap: int = 32768):
    """n requests: Poisson arrivals at `rate`/s (exponential gaps), final lengths
    lognormal (median, sigma) capped, per-request content seeds."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n))
    lengths = np.minimum(np.maximum(1, np.round(np.exp(rng.normal(np.log(median), sigma, size=n)))), cap)
    seeds = rng.integers(1, 2**62, size=n, dtype=np.int64)
    return arrivals, lengths.astype(np.int64), seeds


def expected_checksum(seed: int, length: int) -> int:
    """The checksum a request of `length` elements computes: sum of value x (index + 1)."""
    from .seeds import mix64

    e = np.arange(length, dtype=np.uint64)
    v = (mix64(seed, e, 0x5E7) & np.uint64(0xFFFF)).astype(np.uint64)
    return int((v * (e + np.uint64(1))).sum(dtype=np.uint64))


class Server:
    def __init__(self, alloc: Allocator, slots: int = 4096, max_chunks: int = 128, step: int = 64,
                 queue_cap: int = 8192):
        self.alloc = alloc
        self.nslots = slots
        self.max_chunks = max_chunks
        self.step = step
        self.queue_cap = queue_cap
        self._s = ctypes.c_void_p()
        L.check(L.lib().mmc_serve_create(alloc.handle_ptr, slots, max_chunks, step, queue_cap, ctypes.byref(self._s)),
                "serve_create")
        q, ql, sl, fr = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        L.check(L.lib().mmc_serve_queue(self._s, ctypes.byref(q), ctypes.byref(ql), ctypes.byref(sl),
                                        ctypes.byref(fr)), "serve_queue")
        self.queue = np.ctypeslib.as_array(ctypes.cast(q, ctypes.POINTER(ctypes.c_uint8)),
                                           shape=(queue_cap * CMD_DTYPE.itemsize,)).view(CMD_DTYPE)
        self.queue_len = np.ctypeslib.as_array(ctypes.cast(ql, ctypes.POINTER(ctypes.c_uint32)), shape=(1,))
        self.slots = np.ctypeslib.as_array(ctypes.cast(sl, ctypes.POINTER(ctypes.c_uint8)),
                                           shape=(slots * SLOT_DTYPE.itemsize,)).view(SLOT_DTYPE)
        self.free_chunks = np.ctypeslib.as_array(ctypes.cast(fr, ctypes.POINTER(ctypes.c_uint32)), shape=(1,))
        # field views made once (a structured-array field lookup costs a microsecond a time)
        self._state, self._nchunks, self._checksum = (self.slots[f] for f in ("state", "nchunks", "checksum"))
        self._q = {f: self.queue[f] for f in ("kind", "slot", "id", "final_len", "seed")}
        self._pipe = [self._pipe_views(b) for b in (0, 1)]

    def _pipe_views(self, b):
        """Host views of pipelined-tick buffer b: its command queue and the
        results its tick publishes (completions, chunks still to take, free count)."""
        ptrs = [ctypes.c_void_p() for _ in range(6)]
        L.check(L.lib().mmc_serve_pipeline(self._s, b, *[ctypes.byref(x) for x in ptrs]), "serve_pipeline")

        def arr(p, ctype, n):
            return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctype)), shape=(n,))

        queue = arr(ptrs[0], ctypes.c_uint8, self.queue_cap * CMD_DTYPE.itemsize).view(CMD_DTYPE)
        done = arr(ptrs[2], ctypes.c_uint8, self.nslots * DONE_DTYPE.itemsize).view(DONE_DTYPE)
        return {"q": {f: queue[f] for f in ("kind", "slot", "id", "final_len", "seed")},
                "qlen": arr(ptrs[1], ctypes.c_uint32, 1),
                "done_slot": done["slot"], "done_checksum": done["checksum"],
                "done_len": arr(ptrs[3], ctypes.c_uint32, 1),
                "remaining": arr(ptrs[4], ctypes.c_uint64, 1),
                "free": arr(ptrs[5], ctypes.c_uint32, 1)}

    def tick(self, batched: bool = True):
        L.check(L.lib().mmc_serve_tick(self._s, int(batched)), "serve_tick")

    def launch(self, buffer: int):
        L.check(L.lib().mmc_serve_launch(self._s, buffer), "serve_launch")

    def wait(self):
        L.check(L.lib().mmc_serve_wait(self._s), "serve_wait")

    def wait_buffer(self, buffer: int):
        L.check(L.lib().mmc_serve_wait_buffer(self._s, buffer), "serve_wait_buffer")

    def close(self):
        if getattr(self, "_s", None):
            L.lib().mmc_serve_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run_pipelined(self, arrivals, lengths, seeds, realtime: bool = True, max_seconds: float = 60.0):
        """run() with batched ticks in flight while the host works: tick i runs on
        buffer i % 2 with the queue the host built during tick i - 1, from the
        results tick i - 2 published in the same buffer; it is queued behind
        tick i - 1 before the host waits for that one, so the device runs tick
        after tick without a gap. The host never reads what a running tick
        writes, and a tick's period is the longer of the device's and the
        host's work instead of their sum.
        Admission counts against the free chunks of tick i - 2, less the chunks
        its live requests will yet take and the needs admitted in the queue of
        the tick in flight (completions of the tick in flight are not yet
        counted, so admission stays on the safe side)."""
        n = len(arrivals)
        arrivals = np.asarray(arrivals)
        lengths = np.asarray(lengths, dtype=np.int64)
        seeds = np.asarray(seeds, dtype=np.int64)
        need = -(-lengths // ELEMS_PER_CHUNK)
        admit_t = np.full(n, np.nan)
        done_t = np.full(n, np.nan)
        checksum = np.zeros(n, dtype=np.uint64)
        w_lo = 0
        free_slots = list(range(self.nslots - 1, -1, -1))
        slot_req = np.full(self.nslots, -1, dtype=np.int64)
        if self.queue_cap < self.nslots:
            raise ValueError("pipelined ticks need queue_cap >= slots (a tick may release every slot)")
        ticks = 0
        done = 0
        P = self._pipe
        # two empty ticks publish the starting free count into both buffers
        for b in (0, 1):
            P[b]["qlen"][0] = 0
            self.launch(b)
        self.wait()
        inflight_pending = 0
        released_inflight = []
        i = 0
        waited = 0.0  # host time blocked on the device
        t0 = time.perf_counter()
        while done < n:
            now = time.perf_counter() - t0
            if now > max_seconds:
                break
            nxt = n if not realtime else int(np.searchsorted(arrivals, now, side="right"))
            pb = P[i & 1]
            q = pb["q"]
            # completions published by tick i - 2 in this buffer: released by this tick's queue
            nd = int(pb["done_len"][0])
            cmds = 0
            released = []
            if nd:
                sl = pb["done_slot"][:nd].astype(np.int64)
                r = slot_req[sl]
                done_t[r] = now
                checksum[r] = pb["done_checksum"][:nd]
                done += nd
                slot_req[sl] = -1
                q["kind"][:nd] = 2
                q["slot"][:nd] = sl
                q["id"][:nd] = 0
                q["final_len"][:nd] = 0
                q["seed"][:nd] = 0
                cmds = nd
                released = sl.tolist()
            free_slots.extend(released_inflight)  # released by the queue of the tick in flight
            available = int(pb["free"][0]) - int(pb["remaining"][0]) - inflight_pending
            pending = 0
            k = min(nxt - w_lo, len(free_slots), self.queue_cap - cmds)
            if k > 0:
                k = int(np.searchsorted(np.cumsum(need[w_lo:w_lo + k]), available, side="right"))
            if k > 0:
                reqs = np.arange(w_lo, w_lo + k)
                taken = np.asarray(free_slots[len(free_slots) - k:][::-1], dtype=np.int64)
                del free_slots[len(free_slots) - k:]
                slot_req[taken] = reqs
                sl = slice(cmds, cmds + k)
                q["kind"][sl] = 1
                q["slot"][sl] = taken
                q["id"][sl] = reqs
                q["final_len"][sl] = lengths[reqs]
                q["seed"][sl] = seeds[reqs].astype(np.uint64)
                admit_t[reqs] = now
                pending = int(need[reqs].sum())
                cmds += k
                w_lo += k
            pb["qlen"][0] = cmds
            # queue tick i behind tick i - 1 (no gap on the device), then wait
            # for tick i - 1, whose buffer the next pass reads and rewrites
            self.launch(i & 1)
            tw = time.perf_counter()
            self.wait_buffer((i - 1) & 1)
            waited += time.perf_counter() - tw
            ticks += 1
            i += 1
            inflight_pending = pending
            released_inflight = released
        self.wait()
        seconds = time.perf_counter() - t0
        if done < n:
            self._drain(slot_req)
        return {"admit": admit_t, "done": done_t, "checksum": checksum, "ticks": ticks, "seconds": seconds,
                "completed": done, "wait_seconds": waited}

    def run(self, arrivals, lengths, seeds, batched: bool = True, realtime: bool = True, max_seconds: float = 60.0,
            pipelined: bool = False):
        """Serve the requests; returns a dict of per-request admit / done times
        (seconds from start), checksums, and loop counters. With realtime=False
        every request is treated as arrived at the start (used by tests).

        Requests are admitted first come, first served: each tick admits the
        longest prefix of the waiting requests whose expected chunks fit the
        free-chunk count (less the chunks live requests will still take) and
        for which a server slot is free. All per-tick work on the host is
        vector operations over the slot table and the waiting range. With
        pipelined (batched ticks only), run_pipelined serves instead."""
        if pipelined and batched:
            return self.run_pipelined(arrivals, lengths, seeds, realtime=realtime, max_seconds=max_seconds)
        n = len(arrivals)
        arrivals = np.asarray(arrivals)
        lengths = np.asarray(lengths, dtype=np.int64)
        seeds = np.asarray(seeds, dtype=np.int64)
        need = -(-lengths // ELEMS_PER_CHUNK)
        admit_t = np.full(n, np.nan)
        done_t = np.full(n, np.nan)
        checksum = np.zeros(n, dtype=np.uint64)
        w_lo = 0  # requests w_lo .. nxt-1 have arrived and wait, in arrival order
        nxt = 0
        free_slots = list(range(self.nslots - 1, -1, -1))
        released = []  # slots whose release is in this tick's queue: reusable from the next tick on
        slot_req = np.full(self.nslots, -1, dtype=np.int64)
        ticks = 0
        done = 0
        q = self._q
        state, nchunks, slot_checksum = self._state, self._nchunks, self._checksum
        # first tick: learn the free-slot count
        self.queue_len[0] = 0
        self.tick(batched)
        t0 = time.perf_counter()
        while done < n:
            now = time.perf_counter() - t0
            if now > max_seconds:
                break
            nxt = n if not realtime else int(np.searchsorted(arrivals, now, side="right"))
            free_slots.extend(released)
            # completions of the last tick
            fin = np.flatnonzero((state == L.MMC_SERVE_DONE) & (slot_req >= 0))
            cmds = len(fin)
            if cmds:
                r = slot_req[fin]
                done_t[r] = now
                checksum[r] = slot_checksum[fin]
                done += cmds
                slot_req[fin] = -1
                q["kind"][:cmds] = 2
                q["slot"][:cmds] = fin
                q["id"][:cmds] = 0
                q["final_len"][:cmds] = 0
                q["seed"][:cmds] = 0
            released = fin.tolist()
            live = slot_req >= 0
            promised = int((need[slot_req[live]] - nchunks[live]).sum()) if live.any() else 0
            available = int(self.free_chunks[0]) - promised
            k = min(nxt - w_lo, len(free_slots), self.queue_cap - cmds)
            if k > 0:
                k = int(np.searchsorted(np.cumsum(need[w_lo:w_lo + k]), available, side="right"))
            if k > 0:
                reqs = np.arange(w_lo, w_lo + k)
                taken = np.asarray(free_slots[len(free_slots) - k:][::-1], dtype=np.int64)
                del free_slots[len(free_slots) - k:]
                slot_req[taken] = reqs
                sl = slice(cmds, cmds + k)
                q["kind"][sl] = 1
                q["slot"][sl] = taken
                q["id"][sl] = reqs
                q["final_len"][sl] = lengths[reqs]
                q["seed"][sl] = seeds[reqs].astype(np.uint64)
                admit_t[reqs] = now
                cmds += k
                w_lo += k
            self.queue_len[0] = cmds
            self.tick(batched)
            ticks += 1
            if not realtime and w_lo >= n and not (slot_req >= 0).any():
                break
        seconds = time.perf_counter() - t0
        self._drain(slot_req)
        return {"admit": admit_t, "done": done_t, "checksum": checksum, "ticks": ticks, "seconds": seconds,
                "completed": done}

    def _drain(self, slot_req, max_seconds: float = 120.0):
        """After a run that stopped with requests still growing: tick (one graph
        launch each) without admissions until every live request has completed
        and its slot is released, so the next run starts on an empty slot table
        and a heap holding no chunks of this one. Nothing here is timed or
        counted as served."""
        q = self._q
        t0 = time.perf_counter()
        pending = slot_req >= 0
        while time.perf_counter() - t0 < max_seconds:
            fin = np.flatnonzero((self._state == L.MMC_SERVE_DONE) & pending)
            k = len(fin)
            q["kind"][:k] = 2
            q["slot"][:k] = fin
            pending[fin] = False
            self.queue_len[0] = k
            self.tick(True)
            if not pending.any():
                return
        raise RuntimeError("serving loop did not drain its live requests")


def main(argv=None):
    """Serve one rate in one form on a fresh heap (pagesize 64 KiB; 4096 server
    slots of up to 128 chunks, 64 elements per tick) and print one JSON line:
    p50 / p99 admit-to-completion latency, throughput, ticks and the count of
    wrong checksums; exit status 1 if any checksum is wrong or a request did
    not complete."""
    import argparse
    import json

    from .policies import AlignmentPolicies, CreationPolicies, DistributionPolicies

    ap = argparse.ArgumentParser(prog="python -m mallocmc_gb300.serve")
    ap.add_argument("--rate", type=float, default=100000.0, help="Poisson arrivals per second")
    ap.add_argument("--seconds", type=float, default=0.5, help="arrival window (at most 50 000 requests)")
    ap.add_argument("--heap-gib", type=int, default=64)
    ap.add_argument("--mode", default="pipelined", choices=["pipelined", "sync", "per-request"])
    ap.add_argument("--seed", type=int, default=None, help="request seed (default: the rate, as the bench)")
    a = ap.parse_args(argv)

    heap_bytes = a.heap_gib << 30
    creation = CreationPolicies.Scatter(pagesize=65536, accessblocksize=min(16 << 30, heap_bytes // 2),
                                        regionsize=16)
    alloc = Allocator(creation, DistributionPolicies.XMallocSIMD(65536), None, None, AlignmentPolicies.Shrink(16),
                      size=heap_bytes)
    srv = Server(alloc, slots=4096, max_chunks=128, step=64, queue_cap=8192)
    n = int(min(a.rate * a.seconds, 50000))
    arrivals, lengths, seeds = make_requests(n, a.rate, seed=int(a.seed if a.seed is not None else a.rate))
    want = np.array([expected_checksum(int(s), int(l)) for s, l in zip(seeds, lengths)], dtype=np.uint64)
    try:
        res = srv.run(arrivals, lengths, seeds, batched=(a.mode != "per-request"), realtime=True,
                      max_seconds=max(5.0, 4 * a.seconds), pipelined=(a.mode == "pipelined"))
    finally:
        srv.close()
        alloc.close()
    ok = ~np.isnan(res["done"])
    lat = (res["done"] - res["admit"])[ok] * 1e3
    bad = int((res["checksum"][ok] != want[ok]).sum())
    out = {"rate_per_s": a.rate, "mode": a.mode, "requests": n, "completed": int(ok.sum()), "checksum_errors": bad,
           "p50_ms": float(np.percentile(lat, 50)) if ok.any() else None,
           "p99_ms": float(np.percentile(lat, 99)) if ok.any() else None, "ticks": int(res.get("ticks", 0))}
    print(json.dumps(out))
    return 0 if bad == 0 and int(ok.sum()) == n else 1


if __name__ == "__main__":
    raise SystemExit(main())
