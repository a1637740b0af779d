"""The C++ drop-in API (include/mallocMC/mallocMC.hpp) used the way the
reference's examples use mallocMC (examples/mallocMC_example01.cpp,
examples/mallocMC_example03.cpp), via libmallocmc_examples.so."""
import ctypes
import os

import numpy as np
import pytest

from oracle.oracle import HeapConfig, OracleHeap


@pytest.fixture(scope="module")
def ex():
    from mallocmc_gb300 import build

    if not os.path.exists(build.EXAMPLES_PATH):
        build.build()
    L = ctypes.CDLL(build.EXAMPLES_PATH)
    L.mmcx_example01.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_ulonglong),
                                 ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_uint),
                                 ctypes.POINTER(ctypes.c_int)]
    L.mmcx_example03.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint)]
    L.mmcx_bad_config.argtypes = [ctypes.c_int]
    L.mmcx_oldmalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_ulonglong),
                                 ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_uint),
                                 ctypes.POINTER(ctypes.c_int)]
    L.mmcx_small_requests.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint)]
    L.mmcx_info.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.mmcx_policy_matrix_info.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.mmcx_policy_matrix_kernel.argtypes = [ctypes.c_int]
    L.mmcx_policy_matrix_kernel.restype = ctypes.c_void_p
    return L


def test_info_strings(ex):
    buf = ctypes.create_string_buffer(4096)
    assert ex.mmcx_info(buf, len(buf)) == 0
    s = buf.value.decode()
    assert "CreationPolicy:      Scatter[pagesize=4096,accessblocksize=268435456,regionsize=16" in s
    assert "HierarchyThreshold=123" in s and "minChunkSize=3" in s
    assert "DistributionPolicy:  XMallocSIMD[4096]" in s and "DistributionPolicy:  Noop" in s
    assert "AlignmentPolicy:     Shrink[16]" in s and "OOMPolicy:           ReturnNull" in s


def test_policy_matrix_compiles(ex):
    """The reference's policy matrix (tests/policies.cpp:83-187): every
    combination of Scatter/OldMalloc, XMallocSIMD/Noop distribution and
    Shrink/Noop alignment names its policies and has its device code built."""
    buf = ctypes.create_string_buffer(16384)
    assert ex.mmcx_policy_matrix_info(buf, len(buf)) == 0
    blocks = buf.value.decode().split("--\n")
    assert len(blocks) == 8
    want = [(c, d, r, a) for c, r in (("Scatter[", "AlpakaBuf"), ("OldMalloc", "CudaSetLimits"))
            for d in ("XMallocSIMD[", "Noop") for a in ("Shrink[", "Noop")]
    for b, (c, d, r, a) in zip(blocks, want):
        lines = dict(line.split(":", 1) for line in b.strip().splitlines())
        assert lines["CreationPolicy"].strip().startswith(c)
        assert lines["DistributionPolicy"].strip().startswith(d)
        assert lines["ReservePoolPolicy"].strip() == r
        assert lines["AlignmentPolicy"].strip().startswith(a)
        assert lines["OOMPolicy"].strip() == "ReturnNull"
    kernels = [ex.mmcx_policy_matrix_kernel(i) for i in range(8)]
    assert all(kernels) and len(set(kernels)) == 8
    assert ex.mmcx_policy_matrix_kernel(8) is None


def test_reference_example_config_is_rejected(ex):
    """1 GB heap, 2 GiB access block: the reference divides by zero
    (Scatter.hpp:991-993); the C++ API throws std::invalid_argument first."""
    assert ex.mmcx_bad_config(0) == 1


@pytest.mark.gpu
def test_example01_arrays_of_arrays(ex):
    s, g, slots, fails = ctypes.c_ulonglong(), ctypes.c_ulonglong(), ctypes.c_uint(), ctypes.c_int()
    assert ex.mmcx_example01(0, 100, ctypes.byref(s), ctypes.byref(g), ctypes.byref(slots), ctypes.byref(fails)) == 0
    assert fails.value == 0
    assert s.value == g.value  # the gaussian sum n(n-1), n = threads x length
    assert slots.value > 0


@pytest.mark.gpu
def test_example03_device_side_slots(ex):
    slots = np.zeros(32, dtype=np.uint32)
    values = np.full(32, -1, dtype=np.int32)
    host = ctypes.c_uint()
    assert ex.mmcx_example03(0, slots.ctypes.data, values.ctypes.data, ctypes.byref(host)) == 0
    assert np.array_equal(values, np.arange(32))
    # one page is formatted for 128-byte chunks, which 16-byte slots may not use
    fresh = OracleHeap(HeapConfig(4096, 256 << 20, 16, 2, False), 1 << 30).available_slots(1)
    assert np.all(slots == fresh - 254)
    assert host.value == fresh - 254


@pytest.mark.gpu
def test_oldmalloc_policy_on_cuda_device_heap(ex):
    """CreationPolicies::OldMalloc + ReservePoolPolicies::CudaSetLimits: the same
    handle API on CUDA's own device heap; no slot count (OldMalloc.hpp:51)."""
    s, g, slots, fails = ctypes.c_ulonglong(), ctypes.c_ulonglong(), ctypes.c_uint(), ctypes.c_int()
    assert ex.mmcx_oldmalloc(0, 50, ctypes.byref(s), ctypes.byref(g), ctypes.byref(slots), ctypes.byref(fails)) == 0
    assert fails.value == 0
    assert s.value == g.value
    assert slots.value == 0


@pytest.mark.gpu
def test_small_requests_kernel_has_no_multi_page_path(ex):
    """A user kernel built with mmc::dev::SmallRequests (no multi-page search):
    its small request is served, its request above a page fails with
    MMC_DEVERR_PAGEBASED, and the handle's own malloc serves the same large
    request."""
    from mallocmc_gb300 import _lib as L

    out = np.zeros(3, dtype=np.int32)
    flags = ctypes.c_uint()
    assert ex.mmcx_small_requests(0, out.ctypes.data, ctypes.byref(flags)) == 0
    assert list(out) == [1, 1, 1]
    assert flags.value == L.MMC_DEVERR_PAGEBASED
