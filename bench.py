"""Benchmark: device malloc+free throughput of the GB300 ScatterAlloc heap.

Headline workload (the full-GPU uniform stress): an 8 GiB heap (pagesize 4096,
4 GiB access blocks by default, regionsize 16, wastefactor 2, XMallocSIMD,
ReturnNull, Shrink<16>); grid = SMs x 8 blocks x 256 threads; every thread
runs 100 rounds of {malloc(size), write a u64 pattern, verify it, free}; sizes
uniform in {16, 32, ..., 1024}, drawn from a seeded SplitMix64 table
(synthetic). One step = one launch over the whole grid.

  value            pairs/s with the size table resident in HBM (kernel time, CUDA events)
  e2e              pairs/s through the C ABI with host buffers: H2D of each step's size
                   table from pinned memory (pipelined on a copy stream) + kernel + D2H
                   of the result counters, over the whole span
  roofline         L2 atomic roofline of the stress kernel: the reference algorithm's
                   minimum atomics per pair x pairs / kernel time, against the atomicOr
                   rate measured in the same run (and against the non-returning `red` rate)
  hbm_roofline     the kernel's DRAM traffic (ncu) / kernel time against measured HBM
  l2_bytes         the workload's SM<->L2 bytes (payload written and read back + metadata)
  oldmalloc        the same stress on CUDA's device heap (CreationPolicies::OldMalloc)
  batched          uneven jobs in one graph-captured persistent launch vs one launch per job,
                   with its own atomic roofline (the reference algorithm's atomics for
                   the jobs' draws against the same measured peak)
  serving          the continuous-batching request loop: p50/p99 latency and throughput
                   (and each row's atomic fraction)
  fragmentation    fill at out-of-memory against the oracle's serial run (and the run's
                   atomic fraction)
  cpu_baseline     the reference's own CPU backends on the host cores: the unmodified
                   reference headers on alpaka AccCpuOmp2Blocks (every host core) and
                   AccCpuSerial (one core), the faster reported (oracle/ref_stress.cpp),
                   beside the oracle port (oracle/scatter_oracle.c)

`--impl reference` times the same reference CPU backends (the oracle port where
the reference headers are not installed under baseline/_ref) on the host cores.
Multi-GPU: replicas only (each rank owns an independent heap); `--gpus N`
without a launcher starts N ranks under torch.distributed.run itself.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "malloc+free ops/s on 1 GB300 (batched vs plain launch); p99 serve latency"
UNIT = "malloc+free pairs/s"
SEED = 20261203


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--heap-gib", type=float, default=8.0)
    ap.add_argument("--accessblock-mib", type=int, default=4096,
                    help="access block size; 4096 (two blocks on 8 GiB) is the autotuned choice for this workload, "
                         "the reference default is 2048")
    ap.add_argument("--rounds", type=int, default=100)
    ap.add_argument("--blocks-per-sm", type=int, default=8)
    ap.add_argument("--threads", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-peak", action="store_true")
    ap.add_argument("--no-oldmalloc", action="store_true")
    ap.add_argument("--pattern", default="warp", choices=["warp", "thread"],
                    help="how each block is written and verified: by its warp, 512 B per instruction, or by its thread")
    ap.add_argument("--oldmalloc-rounds", type=int, default=10, help="rounds of the CUDA device-malloc comparison")
    ap.add_argument("--cpu-seconds", type=float, default=4.0,
                    help="target length of each CPU baseline step (reference backends and oracle port)")
    ap.add_argument("--ref-step-seconds", type=float, default=1.5,
                    help="target length of each step of the reference arm (--impl reference)")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-frag", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=1.0, help="arrival window per rate of the serving loop")
    ap.add_argument("--autotune", action="store_true", help="re-run the batched workload's autotuner first")
    return ap.parse_args()


def size_table(rounds: int, nthreads: int, seed: int = SEED) -> np.ndarray:
    """u16 [rounds, nthreads]: 16 * (1 + (mix64(seed, t, r) >> 32) % 64), the
    draw the stress kernel and the CPU port make when given no table."""
    from mallocmc_gb300.seeds import mix64

    t = np.arange(nthreads, dtype=np.uint64)
    out = np.empty((rounds, nthreads), dtype=np.uint16)
    for r in range(rounds):
        out[r] = (16 * (1 + ((mix64(seed, t, r) >> np.uint64(32)) % np.uint64(64)))).astype(np.uint16)
    return out


def warp_atomics(w: np.ndarray, act: np.ndarray, pagesize: int) -> int:
    """Minimum global atomics of malloc+free under the reference algorithm for
    warp-synchronous rounds: w[..., 32] padded sizes, act[..., 32] the lanes
    that take part in that round.

    Lanes with size < pagesize/32 coalesce (XMallocSIMD) when there are at least
    two: one chunk of 16 + sum, malloc 3 atomics (CAS chunksize, add count, or
    mask), free k refcount subtractions + 3 (hierarchical chunk) or + 2; every
    other lane: 3 + 3 or 3 + 2. Hierarchical iff chunk <= (P-8)/33."""
    ht = (pagesize - 8) // 33
    w = w.astype(np.int64)
    co = act & (w < pagesize // 32)
    k = co.sum(axis=-1)
    csum = np.where(co, w, 0).sum(axis=-1)
    grp = k >= 2
    atom_g = np.where(grp, 3 + np.where(16 + csum <= ht, 3, 2) + k, 0)
    single = act & ~(co & grp[..., None])
    atom_s = np.where(single, 3 + np.where(np.maximum(w, 16) <= ht, 3, 2), 0)
    return int(atom_g.sum() + atom_s.sum())


def algorithmic_work(sizes: np.ndarray, pagesize: int = 4096):
    """Minimum global atomics and bytes per launch of the stress under the
    reference algorithm (warp_atomics over every (warp, round)).
    Bytes: payload written and read back (2 x size) + 4 B per atomic + 16 B of
    metadata reads per pair (chunksize on free, region counter, first-free-block,
    segment mask)."""
    s = sizes.astype(np.int64)
    R, T = s.shape
    w = s[:, : (T // 32) * 32].reshape(R, -1, 32)
    atomics = warp_atomics(w, np.ones(w.shape, dtype=bool), pagesize)
    pairs = int(s.size)
    payload = int(2 * s.sum())
    meta = 4 * atomics + 16 * pairs
    return {"pairs": pairs, "atomics": atomics, "atomics_per_pair": atomics / pairs, "payload_bytes": payload,
            "metadata_bytes": meta, "bytes": payload + meta}


def batched_algorithmic_atomics(jobs, pagesize: int) -> dict:
    """warp_atomics of the uneven-job workload: each job's threads form warps of
    32 consecutive job threads; in cycle c the lanes whose cycle count exceeds c
    take part with the size the kernels draw (geometric, float32 inverse CDF,
    capped, padded to 16; csrc/batch.cu draw_size)."""
    from mallocmc_gb300.seeds import mix64

    atomics = pairs = payload = 0
    for j in jobs:
        T = (int(j.threads) + 31) // 32 * 32
        t = np.arange(T, dtype=np.uint64)
        span = np.uint64(j.max_cycles - j.min_cycles + 1)
        cyc = j.min_cycles + ((mix64(j.seed, t, 0xC1C1E) >> np.uint64(32)) % span).astype(np.int64)
        cyc[int(j.threads):] = 0
        c = np.arange(j.max_cycles, dtype=np.uint64)[:, None]
        m = mix64(j.seed, t[None, :], c)
        u = ((m >> np.uint64(40)).astype(np.float32) + np.float32(0.5)) * np.float32(1.0 / 16777216.0)
        q = np.float32(1.0) - np.float32(1.0) / np.float32(j.mean_size)
        x = np.float32(1.0) + np.floor(np.log(u) / np.log(q))
        x = np.minimum(x, np.float32(j.max_size))
        sz = (x.astype(np.int64) + 15) & ~15
        act = np.arange(j.max_cycles)[:, None] < cyc[None, :]
        atomics += warp_atomics(sz.reshape(j.max_cycles, -1, 32), act.reshape(j.max_cycles, -1, 32), pagesize)
        pairs += int(act.sum())
        payload += int(np.where(act, sz, 0).sum())
    return {"pairs": pairs, "atomics": atomics, "atomics_per_pair": atomics / pairs, "payload_bytes": payload}


# DRAM bytes (read + written) per malloc+free pair of the stress kernel, from one
# ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) of the same kernel on
# a 2 GiB heap with 20 rounds (profiles/mmc_stress_kernel_uniform_2GiB_20rounds.md):
# the partial lines at the blocks' ends (their whole lines are discarded from L2
# before the free) and the metadata, so it scales with pairs.
STRESS_DRAM_BYTES_PER_PAIR = 145.0
# L2 atomic requests per pair counted by ncu (lts__t_requests_srcunit_tex_op_atom*
# + op_red) in the same capture: below the reference algorithm's 4.72 because a
# formatted page's chunk size is loaded instead of CAS'd and same-size lanes
# share one reservation.
STRESS_NCU_ATOMICS_PER_PAIR = 3.93
# L2 atomic requests per pair of the batched workload's persistent kernel, from
# an ncu capture on the tuned geometry (profiles/mmc_batch_kernel_512jobs_4GiB.md).
BATCH_NCU_ATOMICS_PER_PAIR = 0.212
STRESS_TRAFFIC_NOTE = ("dram__bytes_read.sum + dram__bytes_write.sum per pair from an ncu capture of the same "
                       "kernel on a 2 GiB heap / 20 rounds, times the pairs of one launch")


class ClockSampler:
    """nvidia-smi samples during the timed region (clocks and throttle reasons)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once nvidia-smi is sampling (its first line is out)
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0:
                time.sleep(0.01)
            self.lines.clear()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def atomic_peak(torch, sms):
    """Measured relaxed device-scope atomicOr throughput (ops/s)."""
    from mallocmc_gb300.workloads import atomic_peak as launch

    res = {}
    sink = torch.zeros(1, dtype=torch.int64, device="cuda")
    blocks, tpb, iters = sms * 8, 256, 512
    for name, words, returning, contended in (("atom_l2_32MiB", 8 << 20, True, False),
                                              ("red_l2_32MiB", 8 << 20, False, False),
                                              ("atom_hbm_4GiB", 1 << 30, True, False),
                                              ("atom_warp_same_word", 8 << 20, True, True)):
        buf = torch.zeros(words, dtype=torch.int32, device="cuda")
        s = torch.cuda.current_stream()
        for _ in range(2):
            launch(buf.data_ptr(), words, blocks, tpb, iters, returning, contended, sink.data_ptr())
        torch.cuda.synchronize()
        best = 0.0
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            launch(buf.data_ptr(), words, blocks, tpb, iters, returning, contended, sink.data_ptr())
            e1.record(s)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = max(best, blocks * tpb * iters / (ms * 1e-3))
        res[name] = best
        del buf
    torch.cuda.empty_cache()
    return res


def oldmalloc_column(torch, stream, heap_bytes, blocks, tpb, rounds, d_sizes, flush, pattern):
    """The same stress on CUDA's built-in device malloc (the OldMalloc policy with
    CudaSetLimits sizing its heap to the Scatter heap's size), over the first
    `rounds` rows of the size table: the comparison column for the GB300 heap."""
    from mallocmc_gb300 import _lib
    from mallocmc_gb300.workloads import stress_params

    L = _lib.lib()
    _lib.check(L.mmc_oldmalloc_set_heap(heap_bytes, torch.cuda.current_device()), "oldmalloc heap")
    stats = torch.zeros(4, dtype=torch.int64, device="cuda")
    p = stress_params(blocks, tpb, rounds, 16, 1024, 16, SEED, pattern)
    import ctypes

    for _ in range(2):
        _lib.check(L.mmc_run_stress_oldmalloc(ctypes.byref(p), d_sizes.data_ptr(), stats.data_ptr(),
                                              stream.cuda_stream), "oldmalloc stress")
    torch.cuda.synchronize()
    stats.zero_()
    ms = []
    for _ in range(3):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _lib.check(L.mmc_run_stress_oldmalloc(ctypes.byref(p), d_sizes.data_ptr(), stats.data_ptr(),
                                              stream.cuda_stream), "oldmalloc stress")
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    st = stats.cpu().numpy().view(np.uint64)
    pairs = blocks * tpb * rounds
    return {"value": pairs / (statistics.median(ms) * 1e-3), "unit": UNIT, "policy": "OldMalloc+CudaSetLimits",
            "rounds": rounds, "ms_per_launch": statistics.median(ms), "nulls": int(st[1]), "pattern_errors": int(st[2])}


def batched_column(torch, args, sms, atom_peak=None, red_peak=None):
    """512 uneven jobs on one 16 GiB heap: one persistent graph-captured launch
    against one plain launch per job (same allocations, checked job by job).
    With atom_peak (measured L2 atomics/s), each form's algorithmic atomics per
    second (batched_algorithmic_atomics) against it."""
    from mallocmc_gb300 import AlignmentPolicies, Allocator, CreationPolicies, DistributionPolicies
    from mallocmc_gb300.autotune import GB300_TUNED, TuneConfig, _accessblock, autotune
    from mallocmc_gb300.batch import Batch, expected_pairs, make_jobs

    heap_bytes = 16 << 30
    jobs = make_jobs(512, seed=3)
    want = expected_pairs(jobs)
    tune_trace = None
    cfg = GB300_TUNED
    if args.autotune:
        cfg, _, tune_trace = autotune(jobs, heap_bytes, expected=want)

    def run(cfg, label):
        creation = CreationPolicies.Scatter(pagesize=cfg.pagesize, regionsize=cfg.regionsize,
                                            accessblocksize=_accessblock(heap_bytes, cfg.pagesize,
                                                                         cfg.accessblock_fraction),
                                            hashingK=cfg.hashingK, hashingDistMP=cfg.hashingDistMP)
        alloc = Allocator(creation, DistributionPolicies.XMallocSIMD(cfg.pagesize), None, None,
                          AlignmentPolicies.Shrink(16), size=heap_bytes)
        b = Batch(alloc, jobs, persistent_blocks=sms * cfg.blocks_per_sm, use_graph=True)
        stream = torch.cuda.current_stream()
        out = {}
        for form, fn in (("plain", b.run_plain), ("graph", b.run)):
            for _ in range(max(3, args.warmup)):
                fn()
            torch.cuda.synchronize()
            b.stats(clear=True)
            ms = []
            for _ in range(args.steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
            st = b.stats(clear=True)
            ok = (np.array_equal(st[:, 0].astype(np.int64), args.steps * want) and int(st[:, 1].sum()) == 0
                  and int(st[:, 2].sum()) == 0)
            if not ok:
                raise RuntimeError(f"batched workload ({form}, {label}) failed its per-job check")
            out[form] = statistics.median(ms)
        b.close()
        alloc.close()
        return out

    tuned = run(cfg, "tuned")
    ref_cfg = TuneConfig()
    ref = run(ref_cfg, "reference defaults")
    pairs = int(want.sum())

    def atomic_roofline(c, ms):
        if atom_peak is None:
            return None
        w = batched_algorithmic_atomics(jobs, c.pagesize)
        ach = w["atomics"] / (ms * 1e-3)
        out = {"bound": "l2_atomic", "achieved": ach / 1e9, "peak": atom_peak / 1e9, "unit": "Gatomic/s",
               "frac": ach / atom_peak, "atomics_per_pair": w["atomics_per_pair"], "form": "graph"}
        if red_peak:
            out["frac_vs_red_peak"] = ach / red_peak
        if c == GB300_TUNED:
            out["ncu_atomics_per_pair"] = BATCH_NCU_ATOMICS_PER_PAIR
            out["ncu_frac"] = pairs / (ms * 1e-3) * BATCH_NCU_ATOMICS_PER_PAIR / atom_peak
        return out

    res = {"workload": "512 jobs on a 16 GiB heap, threads log-uniform in [32, 65536], sizes geometric "
                       "(mean 64 B, cap 4 KiB, padded to 16), 1-16 cycles per thread",
           "pairs_per_step": pairs, "threads": int(sum(j.threads for j in jobs)),
           "graph_value": pairs / (tuned["graph"] * 1e-3), "plain_value": pairs / (tuned["plain"] * 1e-3),
           "speedup_graph_vs_plain": tuned["plain"] / tuned["graph"], "unit": UNIT,
           "ms": tuned, "tuned_config": dict(cfg.__dict__),
           "atomic_roofline": atomic_roofline(cfg, tuned["graph"]),
           "reference_defaults": {"ms": ref, "speedup_graph_vs_plain": ref["plain"] / ref["graph"],
                                  "graph_value": pairs / (ref["graph"] * 1e-3),
                                  "atomic_roofline": atomic_roofline(ref_cfg, ref["graph"])}}
    if tune_trace is not None:
        res["autotune_trace"] = tune_trace
    return res


def serving_column(torch, args, atom_peak=None):
    """Continuous batching on a 64 GiB device-resident heap (pagesize 64 KiB, so a
    16 KiB chunk is a plain chunk): Poisson arrivals at each rate, lognormal
    lengths (median 1024, sigma 1, cap 32768 elements of 2 B), one 16 KiB chunk per
    256 elements, admission by the free-chunk count. Three forms: pipelined graph
    ticks (the host prepares tick i + 1 while tick i runs), synchronous graph
    ticks, and one launch per live request per tick. Latency = admit to
    completion."""
    from mallocmc_gb300 import AlignmentPolicies, Allocator, CreationPolicies, DistributionPolicies
    from mallocmc_gb300.serve import Server, expected_checksum, make_requests

    heap_bytes = 64 << 30
    creation = CreationPolicies.Scatter(pagesize=65536, accessblocksize=16 << 30, regionsize=16)
    alloc = Allocator(creation, DistributionPolicies.XMallocSIMD(65536), None, None, AlignmentPolicies.Shrink(16),
                      size=heap_bytes)
    srv = Server(alloc, slots=4096, max_chunks=128, step=64, queue_cap=8192)
    rows = []
    for rate in (1000, 10000, 100000):
        n = int(min(rate * args.serve_seconds, 50000))
        arrivals, lengths, seeds = make_requests(n, rate, seed=rate)
        want = np.array([expected_checksum(int(s), int(l)) for s, l in zip(seeds, lengths)], dtype=np.uint64)
        for mode in ("graph_pipelined", "graph_per_tick", "launch_per_request"):
            res = srv.run(arrivals, lengths, seeds, batched=(mode != "launch_per_request"), realtime=True,
                          max_seconds=max(5.0, 4 * args.serve_seconds), pipelined=(mode == "graph_pipelined"))
            ok = ~np.isnan(res["done"])
            lat = (res["done"] - res["admit"])[ok] * 1e3
            qlat = (res["done"] - arrivals)[ok] * 1e3
            span = float(np.nanmax(res["done"]) - arrivals[0]) if ok.any() else float("nan")
            rows.append({"rate_per_s": rate, "mode": mode, "requests": n, "completed": int(ok.sum()),
                         "checksum_errors": int((res["checksum"][ok] != want[ok]).sum()),
                         "p50_ms": float(np.percentile(lat, 50)) if ok.any() else None,
                         "p99_ms": float(np.percentile(lat, 99)) if ok.any() else None,
                         "p99_arrival_to_done_ms": float(np.percentile(qlat, 99)) if ok.any() else None,
                         "throughput_req_per_s": ok.sum() / span if ok.any() else 0.0,
                         "chunks_per_s": float((-(-lengths[ok] // 256)).sum() / span) if ok.any() else 0.0,
                         "ticks": res["ticks"]})
            if "wait_seconds" in res:
                # the share of the run the host spent blocked on the device: near 1
                # when the device's tick is the longer side, near 0 when the host's is
                rows[-1]["host_blocked_share"] = res["wait_seconds"] / max(res["seconds"], 1e-9)
            if atom_peak:
                # a 16 KiB chunk on a 64 KiB page: malloc 3 atomics, free 2 (reference algorithm)
                rows[-1]["atomic_frac"] = rows[-1]["chunks_per_s"] * 5 / atom_peak
    srv.close()
    alloc.close()
    return {"workload": "64 GiB heap, pagesize 64 KiB; Poisson arrivals; lognormal lengths (median 1024, sigma 1, "
                        "cap 32768) of 2-byte elements; a 16 KiB chunk per 256 elements; 64 elements per tick",
            "latency": "admit to completion (host clock at the admitting and completing ticks)", "rows": rows}


FRAG_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "frag_fill.json")


def fragmentation_column(torch, args, sms, atom_peak=None):
    """Fill until the first NULL, free a seeded half, refill until the next NULL
    on a 32 GiB heap (pagesize 4096, 256 MiB access blocks): 90 % of requests
    uniform in [16, 2048] B, 10 % log-uniform in [8 KiB, 1 MiB]. Requests go out
    in waves of SMs x 2 x 256 (one per thread). The reference's fill is the
    oracle's serial run on the same seed and geometry, recorded in
    tests/golden/frag_fill.json (ten minutes of CPU at this size). Run with the
    hash distances tuned for fill (hashingDistMP, WP and WPRel 0) and with the
    reference's defaults."""
    from mallocmc_gb300.autotune import GB300_FRAG_TUNED, FragConfig, autotune_fragmentation, frag_allocator
    from mallocmc_gb300.fragmentation import run_fragmentation

    heap_bytes, ab, seed = 32 << 30, 256 << 20, 42

    def golden(hb):
        if not os.path.exists(FRAG_GOLDEN):
            return None
        with open(FRAG_GOLDEN) as f:
            doc = json.load(f)
        for g in doc["geometries"]:
            if g["heap_bytes"] == hb and g["accessblocksize"] == ab and doc["seed"] == seed:
                return {"phase1_fill": g["phase1_fill"], "final_fill": g["final_fill"],
                        "phase1_allocs": g["phase1_allocs"], "phase2_allocs": g["phase2_allocs"],
                        "source": "oracle (serial reference algorithm), tests/golden/frag_fill.json"}
        return None

    ref = golden(heap_bytes)
    tuned, trace = GB300_FRAG_TUNED, None
    if args.autotune and golden(4 << 30) is not None:
        tuned, trace = autotune_fragmentation(4 << 30, ab, golden(4 << 30), seed, sms * 2, 256)
    runs = {}
    for label, cfg in (("tuned_hash", tuned), ("reference_hash", FragConfig())):
        mp, wp, wprel = cfg.hashingDistMP, cfg.hashingDistWP, cfg.hashingDistWPRel
        alloc = frag_allocator(heap_bytes, ab, cfg)
        r = run_fragmentation(alloc, seed, sms * 2, 256, capacity=1 << 23)
        r["error_flags"] = alloc.error_flags()
        alloc.close()
        r["hash"] = {"hashingDistMP": mp, "hashingDistWP": wp, "hashingDistWPRel": wprel}
        if atom_peak:
            r["atomic_roofline"] = {"bound": "l2_atomic", "achieved": r["atomics_per_second"] / 1e9,
                                    "peak": atom_peak / 1e9, "unit": "Gatomic/s",
                                    "frac": r["atomics_per_second"] / atom_peak,
                                    "note": "reference algorithm's minimum atomics of the run's mallocs and frees "
                                            "(fragmentation.run_fragmentation) / run time"}
        if ref is not None:
            r["fill_vs_reference"] = {"phase1": r["phase1_fill"] - ref["phase1_fill"],
                                      "final": r["final_fill"] - ref["final_fill"]}
        runs[label] = r
    out = {"workload": "32 GiB heap, pagesize 4096, access block 256 MiB; 90% uniform [16, 2048] B, 10% "
                       "log-uniform [8 KiB, 1 MiB]; fill to first NULL, free seeded half, refill to next NULL",
           "unit": "ops/s (mallocs incl. the failing ones + frees) and fill = live requested bytes / heap bytes",
           "tuned_hash_source": ("autotune_fragmentation in this run (4 GiB heap)" if trace is not None else
                                 "mallocmc_gb300.autotune.GB300_FRAG_TUNED (autotune_fragmentation's pick on GB300)"),
           "reference": ref, **runs}
    if trace is not None:
        out["autotune_trace"] = trace
    return out


def host_cores() -> int:
    """Host threads this process may run on (the cgroup/affinity set, not the machine's count)."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def cpu_model() -> str:
    """The host CPU's model name (lscpu), for the baseline's description."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform

    return platform.machine()


def cpu_port_run(heap_gib, accessblock_mib, threads_total, rounds, target_s, workers):
    """The oracle port of the reference's CPU backend on `workers` host threads,
    on a bounded sample (virtual threads x rounds) of the same workload and
    heap geometry."""
    from oracle.oracle import HeapConfig, OracleHeap

    cfg = HeapConfig(4096, accessblock_mib << 20, 16, 2, False)
    heap = OracleHeap(cfg, int(heap_gib * (1 << 30)))
    cal = heap.run_stress(4096, 4, SEED, 16, 1024, 16, workers)
    rate = cal["pairs"] / max(cal["seconds"], 1e-6)
    vthreads = int(min(threads_total, max(1024, target_s * rate / rounds)))
    # whole steps repeated (new seeds) until the sample reaches target_s, when one step is shorter
    total = {"pairs": 0, "nulls": 0, "bad": 0, "seconds": 0.0, "steps": 0}
    while total["steps"] == 0 or total["seconds"] < target_s:
        r = heap.run_stress(vthreads, rounds, SEED + 1 + total["steps"], 16, 1024, 16, workers)
        for k in ("pairs", "nulls", "bad", "seconds"):
            total[k] += r[k]
        total["steps"] += 1
    heap.close()
    return total, vthreads


# The reference's own CPU backends (alpaka AccCpuOmp2Blocks on all host cores,
# AccCpuSerial on one) running the stress through the unmodified reference
# headers: oracle/ref_stress.cpp, built by oracle/Makefile from the reference's
# headers installed under baseline/_ref (`make -C oracle install-ref REF=...`).
REF_INSTALL = os.path.join(ROOT, "baseline", "_ref")
REF_STRESS = {"omp": os.path.join(ROOT, "oracle", "_ref", "ref_stress_omp"),
              "serial": os.path.join(ROOT, "oracle", "_ref", "ref_stress_serial")}
REF_STRESS_CONFIGS = {4096: "p4k_ab4g_r16_w2", 2048: "p4k_ab2g_r16_w2", 8: "p4k_ab8m_r16_w2"}


def ensure_ref_stress():
    """Build the reference stress binaries if they are missing. Returns None when
    they are ready, else the reason they cannot be built."""
    if all(os.access(b, os.X_OK) for b in REF_STRESS.values()):
        return None
    src = os.environ.get("MALLOCMC_REFERENCE") or REF_INSTALL
    if not os.path.isdir(os.path.join(src, "src", "include", "mallocMC")):
        return f"reference headers not installed under {os.path.relpath(src, ROOT)}"
    r = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref-stress", f"REF={src}"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        return "reference stress build failed: " + (r.stderr.strip().splitlines() or ["?"])[-1]
    return None


def ref_stress_run(backend, accessblock_mib, heap_bytes, threads_total, rounds, warmup, steps, target_s, workers):
    """Run the reference's stress on one alpaka CPU backend ('omp' on `workers`
    host threads, 'serial' on one): per-step pairs/s over a bounded sample of
    the workload. Returns the per-step results and the summary line."""
    cfg = REF_STRESS_CONFIGS.get(accessblock_mib)
    if cfg is None:
        raise ValueError(f"no reference configuration for a {accessblock_mib} MiB access block")
    env = dict(os.environ)
    if backend == "omp":
        env["OMP_NUM_THREADS"] = str(workers)
        env.setdefault("OMP_PROC_BIND", "false")
    cmd = [REF_STRESS[backend], cfg, str(heap_bytes), str(threads_total), str(rounds), str(SEED), str(warmup),
           str(steps), f"{target_s:g}"]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"reference stress failed ({r.returncode}): {r.stderr.strip()[-400:]}")
    rows = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    summary = next(x for x in rows if x.get("summary"))
    per_step = [x for x in rows if "step" in x]
    if summary["nulls"] or summary["bad"]:
        raise RuntimeError(f"reference stress reported nulls or pattern errors: {summary}")
    return per_step, summary


def reference_cpu_baseline(args, threads_total, warmup, steps, target_s):
    """Both alpaka CPU backends of the reference on this host; the faster one
    is the baseline (on the stress the striped-mutex atomics of the OpenMP
    backend make all cores slower than one). None, reason if unavailable."""
    why = ensure_ref_stress()
    if why is not None:
        return None, why
    workers = host_cores()
    heap_bytes = int(args.heap_gib * (1 << 30))
    runs = {}
    for backend in ("omp", "serial"):
        try:
            per_step, summ = ref_stress_run(backend, args.accessblock_mib, heap_bytes, threads_total, args.rounds,
                                            warmup, steps, target_s, workers)
        except (RuntimeError, ValueError, OSError) as e:
            return None, str(e)
        vals = [x["pairs"] / x["seconds"] for x in per_step]
        runs[backend] = {"value": float(statistics.median(vals)), "per_step": vals, "summary": summ,
                         "cores": summ["workers"]}
    best = max(runs, key=lambda b: runs[b]["value"])
    return {"best": best, "runs": runs, "model": cpu_model()}, None


def max_over_ranks(x: float, dist, device) -> float:
    """The largest of every rank's x (the slowest rank's time); x itself on one rank."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(pairs_per_rank_step: int, world: int, slowest_ms_per_step: float) -> float:
    """Whole-job pairs/s: every rank runs the same workload on its own heap
    (replicas), so the job does world x the pairs in the slowest rank's time."""
    return pairs_per_rank_step * world / (slowest_ms_per_step * 1e-3)


def stress_config(args, sms, world):
    """The headline workload's `config`, shared by both arms of the bench."""
    tpb = args.threads
    return {"workload": f"uniform_stress_{args.heap_gib:g}GiB", "heap_bytes": int(args.heap_gib * (1 << 30)),
            "grid": f"{sms}x{args.blocks_per_sm} blocks x {tpb} threads", "rounds": args.rounds,
            "sizes": "uniform {16,32,...,1024} (u16 table in HBM)",
            "pattern": (f"u64 pattern written and verified per block by its {args.pattern}"
                        + (" (512 B per instruction)" if args.pattern == "warp" else " (16 B per store)")),
            "policies": f"Scatter<4096,{args.accessblock_mib}MiB,16,2,noreset>+XMallocSIMD+ReturnNull+Shrink<16>",
            "pairs_per_step": sms * args.blocks_per_sm * tpb * args.rounds,
            "l2": "flushed between timed steps (512 MiB write)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def sm_count() -> int:
    """SMs of the GPU this rank would use (152 on GB300 when no GPU is visible)."""
    try:
        import torch

        if torch.cuda.is_available():
            return torch.cuda.get_device_properties(int(os.environ.get("LOCAL_RANK", "0"))).multi_processor_count
    except Exception:
        pass
    return 152


def reference_arm(args):
    """The reference's CPU implementation of the path on the host cores: the
    unmodified reference headers on alpaka's CPU backends (the faster of
    AccCpuOmp2Blocks on every host core and AccCpuSerial), or the oracle port
    of its CPU backend when the reference headers are not installed. Rank 0
    alone runs; the other ranks exit without work."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    if rank != 0:
        return
    sms = sm_count()
    threads_total = sms * args.blocks_per_sm * args.threads
    per_step_s = args.ref_step_seconds
    ref, why = reference_cpu_baseline(args, threads_total, args.warmup, args.steps, per_step_s)
    if ref is not None:
        run = ref["runs"][ref["best"]]
        v = run["value"]
        summ = run["summary"]
        other = "serial" if ref["best"] == "omp" else "omp"
        cpu = {"value": v, "unit": UNIT, "cores": run["cores"], "kind": "reference",
               "backend": summ["backend"], "cpu_model": ref["model"],
               "sample": (f"per step {summ['virtual_threads']} virtual threads x {args.rounds} rounds of the workload "
                          f"(the unmodified reference headers, {summ['backend']}, {run['cores']} host threads, "
                          f"heap {args.heap_gib:g} GiB with {args.accessblock_mib} MiB access blocks), about "
                          f"{per_step_s:g} s"),
               "other_backend": {"backend": ref["runs"][other]["summary"]["backend"],
                                 "value": ref["runs"][other]["value"], "cores": ref["runs"][other]["cores"]}}
        ms = 1e3 * summ["seconds"] / max(1, summ["steps"])
        errors = {"nulls": summ["nulls"], "pattern": summ["bad"]}
    else:
        workers = host_cores()
        olib_ok = True
        try:
            from oracle.oracle import lib as olib

            olib()
        except Exception:
            olib_ok = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"],
                                     capture_output=True).returncode == 0
        if not olib_ok:
            print(json.dumps({"impl": "reference", "unavailable": f"{why}; oracle port failed to build"}))
            return
        vals, samples = [], None
        for i in range(args.warmup + args.steps):
            r, vt = cpu_port_run(args.heap_gib, args.accessblock_mib, threads_total, args.rounds, per_step_s, workers)
            if i >= args.warmup:
                vals.append(r["pairs"] / r["seconds"])
                samples = (vt, r)
        v = float(statistics.median(vals))
        vt, r = samples
        cpu = {"value": v, "unit": UNIT, "cores": workers, "kind": "port", "cpu_model": cpu_model(),
               "reference_unavailable": why,
               "sample": f"per step {r['steps']} x ({vt} virtual threads x {args.rounds} rounds) of the workload "
                         f"(oracle port, alpaka CPU-backend semantics: warp size 1, smid = warpid = 0; same heap "
                         f"geometry) on {workers} host threads, about {per_step_s:g} s"}
        ms = 1e3 * r["seconds"]
        errors = {"nulls": r["nulls"], "pattern": r["bad"]}
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded SplitMix64 size draws)",
        "config": stress_config(args, sms, world),
        "cpu_baseline": cpu,
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "errors": errors,
    }
    print(json.dumps(line))


def relaunch_as_ranks(args) -> int:
    """`--gpus N` (N > 1) without a launcher: start N ranks of this script under
    torch.distributed.run on this node (one rank per GPU, replicas) and return
    their exit status."""
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr=127.0.0.1", f"--master-port={port}", os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.run(cmd).returncode


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_as_ranks(args))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world != args.gpus:
        raise SystemExit(f"--gpus {args.gpus} but {world} ranks were launched")
    if args.impl == "reference":
        reference_arm(args)
        return
    import torch

    from mallocmc_gb300 import AlignmentPolicies, Allocator, CreationPolicies, DistributionPolicies, _lib
    from mallocmc_gb300.workloads import launch_stress, stress_params

    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if not os.path.exists(_lib.LIB_PATH):
        import __graft_entry__

        __graft_entry__.build()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    props = torch.cuda.get_device_properties(local)
    sms = props.multi_processor_count
    blocks = sms * args.blocks_per_sm
    tpb = args.threads
    nthreads = blocks * tpb
    rounds = args.rounds
    heap_bytes = int(args.heap_gib * (1 << 30))

    sizes_np = size_table(rounds, nthreads)
    work = algorithmic_work(sizes_np)
    creation = CreationPolicies.Scatter(pagesize=4096, accessblocksize=args.accessblock_mib << 20, regionsize=16,
                                        wastefactor=2)
    alloc = Allocator(creation, DistributionPolicies.XMallocSIMD(4096), None, None, AlignmentPolicies.Shrink(16),
                      size=heap_bytes, device=local)
    stream = torch.cuda.current_stream()
    h_sizes = torch.from_numpy(sizes_np.view(np.int16)).pin_memory()
    d_sizes = h_sizes.to("cuda", non_blocking=False)
    stats = torch.zeros(4, dtype=torch.int64, device="cuda")
    h_stats = torch.zeros(4, dtype=torch.int64).pin_memory()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    from mallocmc_gb300.workloads import PATTERN_THREAD, PATTERN_WARP

    pattern = PATTERN_WARP if args.pattern == "warp" else PATTERN_THREAD
    params = stress_params(blocks, tpb, rounds, 16, 1024, 16, SEED, pattern)

    def step(sizes_ptr):
        launch_stress(alloc, params, sizes_ptr, stats.data_ptr(), stream)

    for _ in range(max(3, args.warmup)):
        stats.zero_()
        step(d_sizes.data_ptr())
    torch.cuda.synchronize()
    if int(stats[1].item()) or int(stats[2].item()):
        raise RuntimeError(f"warm-up step reported nulls/pattern errors: {stats.tolist()}")

    # ---- value: size table resident in HBM, kernel time only ----
    stats.zero_()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for e0, e1 in evs:
            flush.zero_()  # L2 flush (512 MiB write) between timed steps, outside the events
            e0.record(stream)
            step(d_sizes.data_ptr())
            e1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    st = stats.cpu().numpy().view(np.uint64)
    if int(st[0]) != work["pairs"] * args.steps or int(st[1]) or int(st[2]):
        raise RuntimeError(f"timed steps failed verification: {st.tolist()}")
    total_ms = max_over_ranks(float(sum(ms)), dist, "cuda")
    per_step_ms = total_ms / args.steps
    value = job_throughput(work["pairs"], world, per_step_ms)

    # ---- e2e: through the C ABI with host buffers ----
    e2e = None
    if not args.no_e2e:
        # Each step's size table comes from pinned host memory and its counters go
        # back to the host. The copy of step i+1's table runs on a copy stream
        # while step i computes (two device buffers), as a pipelined caller would;
        # the time is the whole span, from the first copy's start to the last
        # step's counters on the host, L2 flushes between the steps included.
        bufs = [d_sizes, torch.empty_like(d_sizes)]
        copy_stream = torch.cuda.Stream()
        ready = [torch.cuda.Event(), torch.cuda.Event()]
        free = [torch.cuda.Event(), torch.cuda.Event()]
        t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t_start.record(stream)
        copy_stream.wait_event(t_start)
        with torch.cuda.stream(copy_stream):
            bufs[0].copy_(h_sizes, non_blocking=True)
            ready[0].record(copy_stream)
        for i in range(args.steps):
            b = i % 2
            if i + 1 < args.steps:
                nb = (i + 1) % 2
                if i >= 1:
                    copy_stream.wait_event(free[nb])  # step i-1 is done with that buffer
                with torch.cuda.stream(copy_stream):
                    bufs[nb].copy_(h_sizes, non_blocking=True)
                    ready[nb].record(copy_stream)
            flush.zero_()
            stats.zero_()
            stream.wait_event(ready[b])
            step(bufs[b].data_ptr())
            free[b].record(stream)
            h_stats.copy_(stats, non_blocking=True)
        t_end.record(stream)
        torch.cuda.synchronize()
        e2e_ms = max_over_ranks(t_start.elapsed_time(t_end) / args.steps, dist, "cuda")
        e2e = {"value": job_throughput(work["pairs"], world, e2e_ms), "unit": UNIT,
               "h2d_bytes_per_step": int(sizes_np.nbytes), "d2h_bytes_per_step": int(h_stats.numel() * 8),
               "ms_per_step": e2e_ms,
               "pipelining": "next step's H2D on a copy stream during the current step; L2 flushes inside the span"}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    peaks, peak_kind = measured_peaks()
    kernel_s = per_step_ms * 1e-3
    traffic = STRESS_DRAM_BYTES_PER_PAIR * work["pairs"]
    # DRAM bytes against HBM: the payload stays in L2 (written, read back and
    # discarded there), so what crosses HBM is the partial end lines and metadata
    hbm = {"bound": "hbm", "achieved": traffic / kernel_s / 1e9, "peak": peaks["hbm_gbs"], "unit": "GB/s",
           "frac": traffic / kernel_s / 1e9 / peaks["hbm_gbs"], "traffic": traffic, "traffic_note": STRESS_TRAFFIC_NOTE,
           "peak_kind": peak_kind, "kernel": "mmc_stress_kernel"}
    # the workload's algorithmic bytes (payload written and read back + metadata),
    # which move between the SMs and L2, not DRAM
    l2_bytes = {"achieved_gbs": work["bytes"] / kernel_s / 1e9, "algorithmic_bytes_per_launch": work["bytes"],
                "payload_bytes_per_launch": work["payload_bytes"], "metadata_bytes_per_launch": work["metadata_bytes"],
                "unit": "GB/s", "note": "SM<->L2 bytes of the workload (not DRAM): 2 x payload + metadata"}
    roofline = dict(hbm)
    pk = None
    if not args.no_peak:
        # The contract's roofline is the L2 atomic one (the unit this path
        # exercises): the reference algorithm's minimum atomics per pair x
        # pairs / kernel time, against the atomicOr rate measured in this run.
        pk = atomic_peak(torch, sms)
        ach = work["atomics"] / kernel_s
        roofline = {"bound": "l2_atomic", "achieved": ach / 1e9, "peak": pk["atom_l2_32MiB"] / 1e9,
                    "unit": "Gatomic/s", "frac": ach / pk["atom_l2_32MiB"],
                    "frac_vs_red_peak": ach / pk["red_l2_32MiB"],
                    "traffic": traffic, "traffic_note": STRESS_TRAFFIC_NOTE,
                    "peak_kind": "measured in this run: mmc_atomic_peak, returning relaxed atomicOr on random words "
                                 "of a 32 MiB L2-resident buffer (MEASURED_PEAKS.json has no atomic rate)",
                    "atomics_per_pair": work["atomics_per_pair"], "atomics_per_launch": work["atomics"],
                    "ncu_atomics_per_pair": STRESS_NCU_ATOMICS_PER_PAIR,
                    "ncu_frac": work["pairs"] / kernel_s * STRESS_NCU_ATOMICS_PER_PAIR / pk["atom_l2_32MiB"],
                    "peaks_measured_gops": {k: v / 1e9 for k, v in pk.items()}, "kernel": "mmc_stress_kernel"}
    batched = None
    if not args.no_batched:
        batched = batched_column(torch, args, sms, pk["atom_l2_32MiB"] if pk else None,
                                 pk["red_l2_32MiB"] if pk else None)
    serving = None
    if not args.no_serve:
        serving = serving_column(torch, args, pk["atom_l2_32MiB"] if pk else None)
    frag = None
    if not args.no_frag:
        frag = fragmentation_column(torch, args, sms, pk["atom_l2_32MiB"] if pk else None)
    oldm = None
    if not args.no_oldmalloc:
        oldm = oldmalloc_column(torch, stream, heap_bytes, blocks, tpb, args.oldmalloc_rounds, d_sizes, flush, pattern)
    cpu = None
    if not args.no_cpu_baseline:
        workers = host_cores()
        r, vt = cpu_port_run(args.heap_gib, args.accessblock_mib, nthreads, rounds, args.cpu_seconds, workers)
        port = {"value": r["pairs"] / r["seconds"], "unit": UNIT, "cores": workers, "kind": "port",
                "sample": f"{r['steps']} x ({vt} virtual threads x {rounds} rounds) (oracle port, alpaka CPU-backend "
                          f"semantics) on {workers} host threads, {r['seconds']:.1f} s"}
        ref, why = reference_cpu_baseline(args, nthreads, 1, 3, args.cpu_seconds)
        if ref is None:
            cpu = dict(port, reference_unavailable=why, cpu_model=cpu_model())
        else:
            run = ref["runs"][ref["best"]]
            summ = run["summary"]
            cpu = {"value": run["value"], "unit": UNIT, "cores": run["cores"], "kind": "reference",
                   "backend": summ["backend"], "cpu_model": ref["model"],
                   "sample": (f"3 steps of {summ['virtual_threads']} virtual threads x {rounds} rounds (the unmodified "
                              f"reference headers on {summ['backend']}, {run['cores']} host threads), "
                              f"{summ['seconds']:.1f} s"),
                   "backends": {b: {"value": x["value"], "cores": x["cores"], "backend": x["summary"]["backend"]}
                                for b, x in ref["runs"].items()},
                   "port": port}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": per_step_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded SplitMix64 size draws)",
        "config": stress_config(args, sms, world),
        "roofline": roofline, "hbm_roofline": hbm, "l2_bytes": l2_bytes, "cpu_baseline": cpu, "e2e": e2e,
        "oldmalloc": oldm, "batched": batched, "serving": serving, "fragmentation": frag,
        "gpu_launches": args.steps, "clocks": clk.summary(), "wall_s_timed": wall,
        "per_step_ms": ms,
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
