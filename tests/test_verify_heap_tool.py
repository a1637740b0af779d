"""The verify_heap tool (mallocmc_gb300/csrc/verify_heap.cu), the counterpart
of the reference's tests/verify_heap.cpp: command line, CSV output and the
fill / verify / damage / free cycle on the device."""
import os
import subprocess

import pytest

from oracle.oracle import HeapConfig, OracleHeap

HEADER = ("PagesizeByte,Accessblocks,Regionsize,Wastefactor,ResetFreedPage,Gridsize,Blocksize,ELEMS_PER_SLOT,"
          "allocElemByte,heapsizeByte,maxSpaceByte,maxSlots,usedSlots,allocFraction,wastedBytes,correct")


def tool():
    from mallocmc_gb300 import build

    exe = os.path.join(build.PKG, "verify_heap")
    if not os.path.exists(exe):
        build.build()
    return exe


def test_help_lists_the_reference_options():
    r = subprocess.run([tool(), "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0
    for opt in ("--threads=N", "--blocks=N", "--heapsize=N", "--machine_readable", "--verbose"):
        assert opt in r.stdout


def test_rejects_empty_grid():
    r = subprocess.run([tool(), "--threads=0"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2


def _run_csv(*args):
    r = subprocess.run([tool(), "-m", *args], capture_output=True, text=True, timeout=600)
    lines = r.stdout.strip().splitlines()
    assert len(lines) == 2, r.stdout + r.stderr
    assert lines[0] == HEADER
    return r.returncode, dict(zip(lines[0].split(","), lines[1].split(",")))


@pytest.mark.gpu
@pytest.mark.parametrize("heap_mb,blocks,threads", [(1024, 64, 128), (2048, 152, 256), (4096, 304, 256),
                                                    (64, 8, 32)])
def test_fill_verify_damage_free(heap_mb, blocks, threads):
    rc, v = _run_csv(f"--heapsize={heap_mb}", f"--blocks={blocks}", f"--threads={threads}")
    assert rc == 0 and v["correct"] == "1", v
    heap = heap_mb << 20
    area = heap // (16 * (12 + 4096) + 4) * 16 * 4096
    ab = (2 << 30) if area >= (2 << 30) else (256 << 20) if area >= (256 << 20) else (8 << 20)
    assert int(v["Accessblocks"]) == ab and int(v["heapsizeByte"]) == heap
    slot = 750 * 8
    assert int(v["maxSlots"]) == heap // slot
    used = int(v["usedSlots"])
    assert int(v["wastedBytes"]) == heap - used * slot == int(v["Wastefactor"])
    # 6000-byte slots take two 4 KiB pages each: the heap holds numpages // 2 of them
    pages = OracleHeap(HeapConfig(4096, ab, 16, 2, False), heap).numpages
    assert pages // 2 * 0.99 <= used <= pages // 2


def _reference_runs():
    import json

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "verify_heap_ref.json")
    return json.load(open(path))["runs"]


def test_reference_fixture_is_well_formed():
    for run in _reference_runs():
        assert run["csv_header"] == HEADER and run["exit_status"] == 0
        assert run["csv_values"].endswith(",1")  # the reference tool verified its own run


@pytest.mark.gpu
@pytest.mark.parametrize("heap_mb", [4096, 8192])
def test_matches_the_reference_tool(heap_mb):
    """The reference's tests/verify_heap.cpp (recorded by gen_verify_heap_golden.py
    on alpaka's CPU-serial backend) and this tool, same heap: the configuration
    columns are equal; the fill of 6000-byte slots is within 1 % of the
    reference's (concurrent multi-page claims may leave a few pages unused)."""
    ref = next(r for r in _reference_runs() if r["heapsize_mb"] == heap_mb)
    want = dict(zip(HEADER.split(","), ref["csv_values"].split(",")))
    rc, got = _run_csv(f"--heapsize={heap_mb}", "--blocks=304", "--threads=256")
    assert rc == 0 and got["correct"] == "1"
    for col in ("PagesizeByte", "Accessblocks", "Regionsize", "ResetFreedPage", "ELEMS_PER_SLOT", "allocElemByte",
                "heapsizeByte", "maxSpaceByte", "maxSlots", "correct"):
        assert got[col] == want[col], col
    assert int(want["usedSlots"]) * 0.99 <= int(got["usedSlots"]) <= int(want["usedSlots"])
