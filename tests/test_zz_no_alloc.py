"""The allocation-free Green's function entry point (dqmc_calculate_greens_noalloc).

It exists for callers that cannot allocate device memory when they need G --
a host whose device memory is owned by its own pool allocator, or a
latency-critical loop where cudaMalloc / cudaFree would synchronise the device.
It computes calculate_greens(mc, slice) from device inputs into a device
output using only the library's fixed device array.  This file is collected
last on purpose (its name sorts after the other test files).
"""
import ctypes as C

import numpy as np
import pytest

from _util import FIELD_U, chain_config, make_setup, maxdiff

pytestmark = pytest.mark.gpu

TOL_G = 1e-10


def _noalloc(lib, cfg, d_hop, d_conf, slice_, d_out, stream):
    L = lib.load()
    fn = L.dqmc_calculate_greens_noalloc
    fn.argtypes = [C.POINTER(lib.ChainConfig), C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                   C.c_void_p, C.c_void_p]
    return fn(C.byref(cfg), C.c_void_p(d_hop), C.c_void_p(d_conf), int(slice_), 0,
              C.c_void_p(d_out), C.c_void_p(stream or None))


# n = 64 / 36 factor in shared memory; n = 81 (one block, 6561 <= 8192
# elements) takes the global-memory QR with the scratch's last matrix as its
# pivot workspace
@pytest.mark.parametrize("field,L", [("MagneticHirschField", 8), ("DensityGHQField", 6),
                                     ("DensityHirschField", 9)])
def test_noalloc_matches_handle_path_twice(pkg, lib, field, L):
    import torch

    model, param, fld, exps = make_setup(pkg, L=L, U=FIELD_U[field], beta=2.0, safe_mult=5,
                                         field=getattr(pkg, field))
    n, nf, M = len(model.l), fld.unique_flavors, param.slices
    cfgs = [chain_config(lib, model, param, fld, seed) for seed in (3, 4)]
    h = lib.Handle(cfgs)
    h.set_hopping(-1, exps)
    h.init_random_field(-1)
    hop = torch.tensor(np.stack([np.asarray(e).T for e in exps]), dtype=torch.float64,
                       device="cuda").contiguous()  # column-major blocks
    out = torch.empty(nf * n * n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row, on different configurations and slices: the second
    # must not see anything left over from the first
    for chain, slice_ in ((0, 7), (1, 13)):
        conf = torch.tensor(np.asfortranarray(h.get_field(chain)).ravel(order="F"),
                            dtype=torch.int8, device="cuda")
        out.fill_(float("nan"))
        code = _noalloc(lib, cfgs[chain], hop.data_ptr(), conf.data_ptr(), slice_,
                        out.data_ptr(), stream)
        assert code == 0, lib.load().dqmc_last_error()
        torch.cuda.synchronize()
        got = lib.buf_to_blocks(out.cpu().numpy(), nf, n)
        want = h.calculate_greens(chain, slice_)
        assert maxdiff(got, want) < TOL_G


def test_noalloc_rejects_oversize(pkg, lib):
    model, param, fld, exps = make_setup(pkg, L=12, U=-4.0, beta=1.0, safe_mult=5)
    cfg = chain_config(lib, model, param, fld, 1)  # 2 * 144^2 elements > 8192
    code = _noalloc(lib, cfg, 1, 1, 1, 1, 0)  # rejected before any pointer is used
    assert code == lib.DQMC_OK + 1
    assert b"exceeds the fixed scratch" in lib.load().dqmc_last_error()
