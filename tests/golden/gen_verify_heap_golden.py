"""Generate tests/golden/verify_heap_ref.json: the CSV line of the reference's
own heap verification tool (tests/verify_heap.cpp, unmodified, built by
oracle/Makefile into oracle/_ref/verify_heap on alpaka's CPU-serial backend)
for the heap sizes the GPU tool's tests compare against.

The reference tool divides by zero below one 2 GiB access block of page area
(Scatter.hpp:991-993), so only heaps of 4096 MB and more are recorded. Its
main() passes --threads as the grid size and --blocks as the block size
(verify_heap.cpp:95 against :619), and the CPU-serial backend runs one thread
per block, so its Gridsize/Blocksize columns are those of that run.

Usage: python tests/golden/gen_verify_heap_golden.py
"""
import json
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
TOOL = os.path.join(ROOT, "oracle", "_ref", "verify_heap")
ARGS = ["-m", "--blocks=64", "--threads=128"]


def main():
    rows = []
    for mb in (4096, 8192):
        r = subprocess.run([TOOL, f"--heapsize={mb}"] + ARGS, capture_output=True, text=True, check=True)
        header, values = r.stdout.strip().splitlines()[-2:]
        rows.append({"heapsize_mb": mb, "args": ARGS, "csv_header": header, "csv_values": values,
                     "exit_status": r.returncode})
    doc = {"tool": "reference tests/verify_heap.cpp on alpaka AccCpuSerial (oracle/_ref/verify_heap)",
           "runs": rows}
    with open(os.path.join(HERE, "verify_heap_ref.json"), "w") as f:
        json.dump(doc, f, indent=1)
    print(json.dumps(doc, indent=1))


if __name__ == "__main__":
    main()
