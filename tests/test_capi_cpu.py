"""CPU-only checks of the C-ABI library and the host-side logic (no GPU calls).

- the library loads and exports every function include/mallocmc_gb300.h declares;
- configuration errors are reported before any device work, with the
  reference's error cases (heap smaller than an access block, bad alignment);
- the Python policy layer enforces the reference's constraints.
"""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mallocmc_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mmc_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from mallocmc_gb300 import _lib

    if not os.path.exists(_lib.LIB_PATH):
        from mallocmc_gb300 import build

        build.build()
    return _lib.lib()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_the_header():
    from mallocmc_gb300 import _lib

    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_config_default_matches_reference_defaults(lib):
    from mallocmc_gb300 import _lib as L

    c = L.MmcConfig()
    lib.mmc_config_default(ctypes.byref(c))
    # DefaultScatterConfig / DefaultScatterHashingParams (Scatter.hpp:56-85), Shrink<16>
    assert (c.pagesize, c.accessblocksize, c.regionsize, c.wastefactor, c.resetfreedpages) == (4096, 2 << 30, 16, 2, 0)
    assert (c.hashingK, c.hashingDistMP, c.hashingDistWP, c.hashingDistWPRel) == (38183, 17497, 1, 1)
    assert (c.dataAlignment, c.distribution, c.oom_policy, c.reference_quirks) == (16, L.MMC_DIST_XMALLOCSIMD, 0, 1)


def _create(lib, cfg, size):
    h = ctypes.c_void_p()
    st = lib.mmc_heap_create(ctypes.byref(cfg), size, 0, None, ctypes.byref(h))
    return st, lib.mmc_last_error().decode()


def test_heap_smaller_than_access_block_is_a_config_error(lib):
    from mallocmc_gb300 import _lib as L

    c = L.MmcConfig()
    lib.mmc_config_default(ctypes.byref(c))
    st, msg = _create(lib, c, 1 << 20)  # 1 MiB heap, 2 GiB access block: the reference divides by zero
    assert st == L.MMC_ERR_CONFIG
    assert "access block" in msg


@pytest.mark.parametrize("field,value", [("pagesize", 100), ("pagesize", 4100), ("regionsize", 0),
                                         ("wastefactor", 0), ("accessblocksize", 0), ("dataAlignment", 24),
                                         ("distribution", 7), ("oom_policy", 9)])
def test_invalid_config_rejected_without_device(lib, field, value):
    from mallocmc_gb300 import _lib as L

    c = L.MmcConfig()
    lib.mmc_config_default(ctypes.byref(c))
    setattr(c, field, value)
    st, _ = _create(lib, c, 64 << 20)
    assert st == L.MMC_ERR_CONFIG


def test_null_arguments(lib):
    from mallocmc_gb300 import _lib as L

    assert lib.mmc_heap_create(None, 1 << 20, 0, None, None) == L.MMC_ERR_ARG
    assert lib.mmc_heap_destroy(None) == L.MMC_OK
    out = ctypes.c_uint()
    assert lib.mmc_available_slots(None, 16, None, ctypes.byref(out)) == L.MMC_ERR_ARG


def test_policy_constraints():
    from mallocmc_gb300.policies import AlignmentPolicies, CreationPolicies, DistributionPolicies, OOMPolicies
    from mallocmc_gb300.policies import make_config

    with pytest.raises(ValueError, match="Pagesize must be the same"):
        make_config(CreationPolicies.Scatter(pagesize=4096), DistributionPolicies.XMallocSIMD(pagesize=16384),
                    OOMPolicies.ReturnNull(), AlignmentPolicies.Shrink())
    with pytest.raises(ValueError):
        AlignmentPolicies.Shrink(dataAlignment=12)
    assert AlignmentPolicies.Shrink(16).applyPadding(17) == 32
    assert AlignmentPolicies.Shrink(16).applyPadding((1 << 32) + 1) == 16  # size_t -> uint32 narrowing
    assert AlignmentPolicies.Noop.applyPadding(17) == 17
    c = make_config(CreationPolicies.Scatter(pagesize=16384, regionsize=8), DistributionPolicies.Noop(),
                    OOMPolicies.BadAllocException(), AlignmentPolicies.Noop())
    assert (c.pagesize, c.regionsize, c.distribution, c.oom_policy, c.dataAlignment) == (16384, 8, 0, 1, 1)


def test_package_never_imports_the_oracle():
    """The oracle is test infrastructure: no module of the product package names it."""
    import glob
    import os

    pkg = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "mallocmc_gb300")
    for path in glob.glob(os.path.join(pkg, "*.py")):
        src = open(path).read()
        assert "import oracle" not in src and "from oracle" not in src, path


def test_seed_twin_matches_the_oracle_draws():
    import numpy as np

    from mallocmc_gb300.seeds import mix64
    from oracle.oracle import lib, mix64 as oracle_mix64

    a = np.arange(1000, dtype=np.uint64)
    for seed, b in ((0, 0), (42, 0x5E7), (2**63 + 5, 0xC1C1E)):
        assert np.array_equal(mix64(seed, a, b), oracle_mix64(seed, a, b))
        assert int(mix64(seed, 7, b)) == lib().oc_mix64(seed, 7, b)
