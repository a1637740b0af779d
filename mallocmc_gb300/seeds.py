"""Host twin of the workload kernels' counter-based draws (the device `mix64`
of csrc/workloads.cu, batch.cu and serve.cu): SplitMix64's finaliser applied to
seed + a * 0x9E3779B97F4A7C15 + b * 0xD1B54A32D192ED03, on numpy arrays. Used
to predict what a workload kernel draws (cycle counts, element values) without
running it."""
from __future__ import annotations

import numpy as np


def mix64(seed: int, a, b):
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) + np.asarray(a, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
             + np.asarray(b, dtype=np.uint64) * np.uint64(0xD1B54A32D192ED03))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))
