"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares (no compute calls here)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(dqmc_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_header_declares_the_api():
    names = declared_functions()
    for must in ("dqmc_create", "dqmc_sweep", "dqmc_calculate_greens", "dqmc_get_greens",
                 "dqmc_initialize_run", "dqmc_set_hopping", "dqmc_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(pkg):
    from montecarlo_gb300 import build, _lib

    try:
        build.build()
    except RuntimeError as e:  # pragma: no cover - toolkit missing
        pytest.skip(f"CUDA toolkit unavailable: {e}")
    lib = C.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    lib.dqmc_abi_version.restype = C.c_int
    assert lib.dqmc_abi_version() == 6


def test_create_without_gpu_fails_loudly(pkg):
    """No CPU fallback: without a device dqmc_create reports a CUDA error."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from montecarlo_gb300 import build, _lib

    build.build()
    cfg = _lib.ChainConfig(16, 1, 10, 5, 0, 1, 0.5, 1)
    with pytest.raises(_lib.DQMCError) as ei:
        _lib.Handle([cfg])
    assert ei.value.code == 2


def test_invalid_config_rejected(pkg):
    from montecarlo_gb300 import build, _lib

    build.build()
    L = _lib.load()
    cfg = _lib.ChainConfig(16, 2, 10, 5, 0, 1, 0.5, 1)  # density field with two flavours
    h = C.c_void_p()
    code = L.dqmc_create(0, C.byref(cfg), 1, 0, C.byref(h))
    assert code == 1
    assert b"n_flavors" in L.dqmc_last_error()
