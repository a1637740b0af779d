"""The serving loop's host logic (mallocmc_gb300.serve.Server.run) on CPU,
against a numpy model of one device tick: apply the queued admissions and
releases, grow every live request by `step` elements taking one 16 KiB chunk
per 256 elements from a pool, complete a request at its length (checksum, chunks
back to the pool) and publish the pool's free count. The model is test
infrastructure standing in for the GPU; it checks what the host decides:
first-come-first-served admission, never more chunks promised than the pool
holds (so no live request ever fails to grow), slot reuse only after release,
and the drain of a run cut short."""
import numpy as np
import pytest

from mallocmc_gb300 import _lib as L
from mallocmc_gb300.serve import (CMD_DTYPE, DONE_DTYPE, ELEMS_PER_CHUNK, SLOT_DTYPE, Server, expected_checksum,
                                  make_requests)


class ModelServer(Server):
    def __init__(self, pool_chunks, slots=16, step=64, queue_cap=64):
        self.nslots, self.step, self.queue_cap, self.max_chunks = slots, step, queue_cap, 128
        self.queue = np.zeros(queue_cap, dtype=CMD_DTYPE)
        self.queue_len = np.zeros(1, dtype=np.uint32)
        self.slots = np.zeros(slots, dtype=SLOT_DTYPE)
        self.free_chunks = np.zeros(1, dtype=np.uint32)
        self._state, self._nchunks, self._checksum = (self.slots[f] for f in ("state", "nchunks", "checksum"))
        self._q = {f: self.queue[f] for f in ("kind", "slot", "id", "final_len", "seed")}
        self.pool = pool_chunks
        self.grow_failures = 0
        self.ticks_seen = 0
        self.max_live = 0
        self._pipe = []
        for _ in (0, 1):
            queue = np.zeros(queue_cap, dtype=CMD_DTYPE)
            done = np.zeros(slots, dtype=DONE_DTYPE)
            self._pipe.append({"queue": queue, "q": {f: queue[f] for f in CMD_DTYPE.names},
                               "qlen": np.zeros(1, np.uint32), "done": done, "done_slot": done["slot"],
                               "done_checksum": done["checksum"], "done_len": np.zeros(1, np.uint32),
                               "remaining": np.zeros(1, np.uint64), "free": np.zeros(1, np.uint32)})

    def launch(self, b):
        """The pipelined tick, run at once: the host only reads its results two
        ticks later, as it would while the tick ran on the device."""
        p = self._pipe[b]
        completed = self._tick(p["queue"], int(p["qlen"][0]))
        p["done_len"][0] = len(completed)
        for j, w in enumerate(completed):
            p["done"][j] = (w, 0, self.slots[w]["checksum"])
        live = self.slots["state"] == L.MMC_SERVE_LIVE
        p["remaining"][0] = int((-(-self.slots["final_len"][live].astype(np.int64) // ELEMS_PER_CHUNK)
                                 - self.slots["nchunks"][live]).sum())
        p["free"][0] = self.pool

    def wait(self):
        pass

    def wait_buffer(self, b):
        pass

    def tick(self, batched=True):
        self._tick(self.queue, int(self.queue_len[0]))
        self.free_chunks[0] = self.pool

    def _tick(self, queue, qlen):
        self.ticks_seen += 1
        completed = []
        for c in queue[:qlen]:
            s = self.slots[c["slot"]]
            if c["kind"] == 1:
                assert s["state"] == L.MMC_SERVE_FREE, "admitted into a slot that was not released"
                s["id"], s["final_len"], s["seed"] = c["id"], c["final_len"], c["seed"]
                s["len"] = s["nchunks"] = s["failed"] = 0
                s["checksum"] = 0
                s["state"] = L.MMC_SERVE_LIVE
            elif c["kind"] == 2:
                assert s["state"] == L.MMC_SERVE_DONE
                s["state"] = L.MMC_SERVE_FREE
            self.slots[c["slot"]] = s
        live = np.flatnonzero(self.slots["state"] == L.MMC_SERVE_LIVE)
        self.max_live = max(self.max_live, len(live))
        for w in live:
            s = self.slots[w]
            end = min(int(s["len"]) + self.step, int(s["final_len"]))
            chunks = -(-end // ELEMS_PER_CHUNK)
            need = chunks - int(s["nchunks"])
            if need > self.pool:
                s["failed"] += 1
                self.grow_failures += 1
            else:
                self.pool -= need
                s["len"], s["nchunks"] = end, chunks
                if end == s["final_len"]:
                    s["checksum"] = expected_checksum(int(s["seed"]), end)
                    s["state"] = L.MMC_SERVE_DONE
                    self.pool += chunks
                    completed.append(int(w))
            self.slots[w] = s
        return completed

    def close(self):
        pass


@pytest.mark.parametrize("pipelined", [False, True])
@pytest.mark.parametrize("pool,slots", [(10_000, 16), (40, 16), (16, 64)])
def test_admission_never_overcommits_and_every_request_completes(pool, slots, pipelined):
    arrivals, lengths, seeds = make_requests(60, rate=1e9, seed=3, median=1024, sigma=1.0, cap=4096)
    srv = ModelServer(pool, slots=slots)
    res = srv.run(arrivals, lengths, seeds, batched=True, realtime=False, pipelined=pipelined)
    assert res["completed"] == len(arrivals)
    want = np.array([expected_checksum(int(s), int(n)) for s, n in zip(seeds, lengths)], dtype=np.uint64)
    assert np.array_equal(res["checksum"], want)
    assert srv.grow_failures == 0  # admission kept every promised chunk available
    assert srv.pool == pool  # every chunk came back
    admit = res["admit"]
    assert np.all(np.diff(admit) >= 0)  # first come, first served
    assert srv.max_live <= slots


@pytest.mark.parametrize("pipelined", [False, True])
def test_small_pool_holds_requests_back(pipelined):
    arrivals, lengths, seeds = make_requests(30, rate=1e9, seed=4, median=2048, sigma=0.2, cap=4096)
    need = -(-lengths // ELEMS_PER_CHUNK)
    srv = ModelServer(int(need.max()), slots=16)
    res = srv.run(arrivals, lengths, seeds, batched=True, realtime=False, pipelined=pipelined)
    assert res["completed"] == len(arrivals)
    # the pool holds one largest request: never more live than the smallest needs fit
    assert srv.max_live <= int(need.max()) // int(need.min())
    assert len(np.unique(res["admit"])) > 1  # later requests waited for chunks to come back
    assert srv.grow_failures == 0


@pytest.mark.parametrize("pipelined", [False, True])
def test_cut_short_run_drains(pipelined):
    arrivals, lengths, seeds = make_requests(40, rate=1e9, seed=5, median=4096, sigma=0.1, cap=8192)
    srv = ModelServer(10_000, slots=32, step=16)
    first = srv.run(arrivals, lengths, seeds, batched=True, realtime=False, max_seconds=0.0, pipelined=pipelined)
    assert first["completed"] < len(arrivals)
    assert not (srv.slots["state"] != L.MMC_SERVE_FREE).any()
    assert srv.pool == 10_000
    again = srv.run(arrivals, lengths, seeds, batched=True, realtime=False)
    assert again["completed"] == len(arrivals)


def test_pipelined_ticks_need_room_to_release_every_slot():
    """A pipelined tick may release every slot at once: a queue shorter than the
    slot table is refused up front instead of overflowing."""
    arrivals, lengths, seeds = make_requests(4, rate=1e9, seed=6)
    srv = ModelServer(1000, slots=64, queue_cap=32)
    with pytest.raises(ValueError):
        srv.run(arrivals, lengths, seeds, batched=True, realtime=False, pipelined=True)


def test_queue_check_refuses_out_of_range_commands():
    """mmc_serve_check_queue, the host-side check every tick launch runs first:
    a queue length beyond the queue's capacity, a slot beyond the table or an
    unknown command kind is MMC_ERR_ARG; a valid queue is MMC_OK. No GPU."""
    import ctypes

    from mallocmc_gb300 import _lib as L
    from mallocmc_gb300.serve import CMD_DTYPE

    lib = L.lib()
    q = np.zeros(4, dtype=CMD_DTYPE)
    q["kind"] = [1, 2, 1, 1]
    q["slot"] = [0, 7, 3, 5]
    ptr = q.ctypes.data_as(ctypes.c_void_p)
    assert lib.mmc_serve_check_queue(ptr, 4, 4, 8) == L.MMC_OK
    assert lib.mmc_serve_check_queue(ptr, 0, 4, 8) == L.MMC_OK
    assert lib.mmc_serve_check_queue(ptr, 5, 4, 8) == L.MMC_ERR_ARG
    assert b"exceeds the queue's capacity" in lib.mmc_last_error()
    q["slot"][1] = 8
    assert lib.mmc_serve_check_queue(ptr, 4, 4, 8) == L.MMC_ERR_ARG
    assert b"names slot 8" in lib.mmc_last_error()
    q["slot"][1] = 7
    q["kind"][2] = 3
    assert lib.mmc_serve_check_queue(ptr, 4, 4, 8) == L.MMC_ERR_ARG
    assert b"unknown kind" in lib.mmc_last_error()
    assert lib.mmc_serve_check_queue(None, 1, 4, 8) == L.MMC_ERR_ARG
