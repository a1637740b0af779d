"""The reference CPU baseline tool (oracle/ref_stress.cpp: the unmodified
reference headers on alpaka's CPU backends, built into oracle/_ref where the
reference's headers are installed). Every virtual thread's rounds complete
with no NULL and no pattern error, on both backends. Skipped where the tool
is not built."""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("backend", ["serial", "omp"])
def test_reference_stress_runs_clean(backend):
    import bench

    exe = bench.REF_STRESS[backend]
    if not os.access(exe, os.X_OK):
        pytest.skip("reference stress tool not built (reference headers not installed)")
    per_step, summ = bench.ref_stress_run(backend, 8, 64 << 20, 4096, 10, 1, 2, 0.05, 2)
    assert len(per_step) == 2
    n = summ["virtual_threads"]
    assert all(s["pairs"] == n * 10 for s in per_step)
    assert summ["nulls"] == 0 and summ["bad"] == 0
    assert summ["backend"] == ("alpaka AccCpuOmp2Blocks" if backend == "omp" else "alpaka AccCpuSerial")
    assert summ["workers"] == (2 if backend == "omp" else 1)


def test_reference_stress_refuses_unknown_config():
    import bench

    exe = bench.REF_STRESS["serial"]
    if not os.access(exe, os.X_OK):
        pytest.skip("reference stress tool not built (reference headers not installed)")
    r = subprocess.run([exe, "nope", "1", "1", "1", "1", "0", "1", "0.1"], capture_output=True, text=True)
    assert r.returncode == 2 and "unknown config" in r.stderr
    assert not [x for x in r.stdout.splitlines() if x.startswith("{") and json.loads(x)]
