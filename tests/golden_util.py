"""Helpers shared by the tests that replay tests/golden fixtures."""
import glob
import hashlib
import json
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


# fixtures that are not op programs: fill fractions (gen_frag_golden.py) and the
# reference verify_heap tool's CSV lines (gen_verify_heap_golden.py)
NOT_PROGRAMS = {"frag_fill.json", "verify_heap_ref.json"}


def fixture_paths():
    """The op-program fixtures (gen_golden.py)."""
    return sorted(p for p in glob.glob(os.path.join(GOLDEN_DIR, "*.json")) if os.path.basename(p) not in NOT_PROGRAMS)


def load(path):
    with open(path) as f:
        return json.load(f)


def digest(arr) -> str:
    return hashlib.sha256(np.ascontiguousarray(arr, dtype="<u4").tobytes()).hexdigest()


def encode_ops(ops):
    """(kinds bytes, args u64) of a fixture program; 'S' (snapshot) rows are
    kept as no-ops so result indices line up."""
    kinds = bytes(ord(k) for k, _ in ops)
    args = np.array([a for _, a in ops], dtype=np.uint64)
    return kinds, args


def expected_results(case):
    """Per-op expected values: pool offset for malloc, slot count for s/d, None otherwise."""
    return case["results"]
