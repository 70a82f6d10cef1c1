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
    assert lib.dqmc_abi_version() == 10


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
    # size limits and non-finite constants (checked before any device call)
    for bad, what in (((513, 2, 10, 5, 1, 1, 0.5, 1, 0.0), b"n_sites"),
                      ((0, 1, 10, 5, 0, 1, 0.5, 1, 0.0), b"n_sites"),
                      ((16, 1, 0, 5, 0, 1, 0.5, 1, 0.0), b"slices"),
                      ((16, 1, 10, 0, 0, 1, 0.5, 1, 0.0), b"safe_mult"),
                      ((16, 1, 10, 5, 4, 1, 0.5, 1, 0.0), b"field"),
                      ((16, 1, 3000, 5, 0, 1, 0.5, 1, 0.0), b"chunks"),
                      ((129, 1, 10, 5, 0, 1, 0.0, 1, 0.6), b"complex"),
                      ((16, 1, 10, 5, 0, 1, float("nan"), 1, 0.0), b"alpha"),
                      ((16, 1, 10, 5, 0, 1, 0.5, 1, float("inf")), b"alpha")):
        cfg = _lib.ChainConfig(*bad)
        assert L.dqmc_create(0, C.byref(cfg), 1, 0, C.byref(h)) == 1, bad
        assert what in L.dqmc_last_error(), (bad, L.dqmc_last_error())
    # a complex chain at the largest size is valid, but not in mixed precision
    cfg = _lib.ChainConfig(128, 1, 10, 5, 0, 1, 0.0, 1, 0.6)
    assert L.dqmc_create(0, C.byref(cfg), 1, 1, C.byref(h)) == 1
    assert b"FP64" in L.dqmc_last_error()


def test_ctypes_structs_match_the_header(pkg, tmp_path):
    """The ctypes mirrors of the ABI structs have the header's sizes and offsets."""
    import shutil
    import subprocess
    from montecarlo_gb300 import _lib
    if shutil.which("gcc") is None:  # pragma: no cover
        pytest.skip("gcc unavailable")
    structs = {"dqmc_chain_config": _lib.ChainConfig, "dqmc_stats": _lib.Stats,
               "dqmc_measure_config": _lib.MeasureConfig, "dqmc_observables": _lib.Observables}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "dqmc_gb300.h"', "int main(void){"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "sizes.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True,
                                                  text=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(got[cname]) == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(py, fname).offset, (cname, fname)


def test_complex_matrix_buffers_round_trip(pkg):
    """The ctypes side's interleaved-complex buffers (Julia's ComplexF64
    layout, column-major per block) round-trip the (nf, n, n) blocks."""
    import numpy as np
    from montecarlo_gb300 import _lib
    rng = np.random.default_rng(0)
    G = rng.standard_normal((2, 5, 5)) + 1j * rng.standard_normal((2, 5, 5))
    buf = _lib.complex_blocks_to_buf(G)
    assert buf.dtype == np.float64 and buf.size == 2 * 2 * 25
    # entry (b, i, j) sits at 2 * (b n^2 + j n + i) (+1 for the imaginary part)
    assert buf[2 * (25 + 3 * 5 + 1)] == G[1, 1, 3].real
    assert buf[2 * (25 + 3 * 5 + 1) + 1] == G[1, 1, 3].imag
    back = _lib.buf_to_blocks(buf.view(np.complex128), 2, 5)
    assert np.array_equal(back, G)
    cfg = _lib.ChainConfig(16, 1, 10, 5, 0, 1, 0.0, 1, 0.6)
    assert _lib.is_complex(cfg) and not _lib.is_complex(_lib.ChainConfig(16, 1, 10, 5, 0, 1, 0.5, 1))


def test_julia_shim_buffer_sizes_match_the_header(pkg):
    """The Julia shim of the integration guide allocates the dqmc_stats
    buffer and names the struct sizes it mirrors: they must be the header's
    (a smaller buffer would be overrun by dqmc_sweep)."""
    import re
    from montecarlo_gb300 import _lib
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    m = re.search(r"Vector\{UInt8\}\(undef, (\d+)\)\s+# dqmc_stats \(ABI (\d+), (\d+) bytes\)", text)
    assert m, "the shim's dqmc_stats buffer line is missing"
    assert int(m.group(1)) == int(m.group(3)) == C.sizeof(_lib.Stats)
    assert int(m.group(2)) == _header_abi()
    m = re.search(r"# dqmc_chain_config \(ABI (\d+), (\d+) bytes\)", text)
    assert m, "the shim's dqmc_chain_config line is missing"
    assert int(m.group(1)) == _header_abi() and int(m.group(2)) == C.sizeof(_lib.ChainConfig)


def _header_abi():
    import re
    hdr = open(os.path.join(ROOT, "include", "dqmc_gb300.h")).read()
    return int(re.search(r"#define DQMC_GB300_ABI_VERSION (\d+)", hdr).group(1))


def test_python_binding_covers_the_header(pkg):
    """The ctypes layer binds exactly the entry points the header declares."""
    from montecarlo_gb300 import _lib
    assert sorted(_lib.EXPORTS) == declared_functions()


def _build_c_host(tmp_path):
    import shutil
    import subprocess
    from montecarlo_gb300 import build, _lib

    if shutil.which("gcc") is None:  # pragma: no cover
        pytest.skip("gcc unavailable")
    build.build()
    exe = tmp_path / "c_host_example"
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c_host_example.c"), "-L", libdir,
                    "-ldqmc_gb300", "-lm", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return exe


def test_c_host_links_and_fails_loudly_without_gpu(pkg, tmp_path):
    """A pure C host (tests/c_host_example.c: the pool calls of the serving
    loop) compiles against the header and links against the library; without
    a device its first call reports the CUDA error (no CPU fallback)."""
    import subprocess
    import torch

    exe = _build_c_host(tmp_path)
    if torch.cuda.is_available():
        pytest.skip("a GPU is present (the GPU test runs the example)")
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 3, (r.returncode, r.stdout, r.stderr)
    assert "dqmc_pool_create" in r.stdout


@pytest.mark.gpu
def test_c_host_runs_a_pool(pkg, tmp_path):
    """The pure C host on the GPU: admits a 4x4 chain, runs 50 ms time slices
    until its 5 sweeps are done, and reads a sane acceptance and propagation
    error."""
    import subprocess

    exe = _build_c_host(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    parts = r.stdout.split()
    assert parts[0] == "sweeps" and int(parts[1]) == 5
    assert 0.0 < float(parts[3]) < 1.0 and float(parts[5]) < 1e-6
