"""The allocation-free normFactor entry point, cf_norm_factor_noalloc.

It serves callers that must not allocate device memory (an application whose
own memory pool owns the GPU, or a latency-critical loop that cannot afford a
cudaMalloc/cudaFree).  Here it is called through the C ABI on device arrays,
twice in a row with different inputs (its scratch array keeps the previous
call's contents), and each result is compared with the allocating entry
point cf_norm_factor: identical bits in the reference summation order, and
within 1e-13 relative in the fast order (the tolerance the other
normFactor tests use is 1e-14 to 1e-12).  Once the first call on the device
has looked up the scratch array, further calls must leave the device's free
memory (cudaMemGetInfo) unchanged.
"""
import ctypes as C

import numpy as np
import pytest

import cufoam_gb300 as cf
from cufoam_gb300 import _capi
from cufoam_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_noalloc_norm_factor_matches_allocating_entry_point():
    import torch
    lib = _capi.load()
    ctx = cf.Context(0)
    L = W.grid_lognormal(24, 20, 18, 4)
    M = cf.LduMatrix.from_ldu(L, ctx)
    ro, cols, vals = M.to_csr()
    dev = torch.device("cuda:0")
    d_ro = torch.from_numpy(ro).to(dev)
    d_cols = torch.from_numpy(cols).to(dev)
    d_vals = torch.from_numpy(vals).to(dev)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    orders = {"reference": _capi.CF_REDUCE_REFERENCE, "fast": _capi.CF_REDUCE_FAST}
    inputs = []
    for seed_b, seed_x in ((1, 2), (3, 4)):  # two calls in a row, different inputs
        b = W.uniform(seed_b, L.n)
        x = W.uniform(seed_x, L.n, 0.0, 2.0)
        want = {name: M.norm_factor(b, x, reduction=name) for name in orders}
        inputs.append((torch.from_numpy(b).to(dev), torch.from_numpy(x).to(dev), want))

    def call(d_b, d_x, code):
        return lib.cf_norm_factor_noalloc(L.n, d_ro.data_ptr(), d_cols.data_ptr(),
                                          d_vals.data_ptr(), d_b.data_ptr(), d_x.data_ptr(),
                                          code, out.data_ptr(), C.c_void_p(stream.cuda_stream))

    # first call on this device: looks up the scratch array's device address
    assert call(inputs[0][0], inputs[0][1], orders["fast"]) == _capi.CF_OK
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(dev)[0]
    for d_b, d_x, want in inputs:
        for name, code in orders.items():
            out.fill_(-1.0)
            assert call(d_b, d_x, code) == _capi.CF_OK
            torch.cuda.synchronize()
            got = float(out.item())
            if name == "reference":
                assert got == want[name]
            else:
                assert abs(got - want[name]) <= 1e-13 * want[name]
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(dev)[0] == free_before, "the no-alloc calls allocated device memory"


def test_noalloc_norm_factor_rejects_bad_arguments():
    import torch
    lib = _capi.load()
    dev = torch.device("cuda:0")
    t = torch.zeros(4, dtype=torch.float64, device=dev)
    i = torch.zeros(4, dtype=torch.int32, device=dev)
    p = t.data_ptr()
    assert lib.cf_norm_factor_noalloc(0, i.data_ptr(), i.data_ptr(), p, p, p, 0, p, None) == \
        _capi.CF_BAD_INPUT
    assert lib.cf_norm_factor_noalloc(3, None, i.data_ptr(), p, p, p, 0, p, None) == \
        _capi.CF_BAD_INPUT
    assert lib.cf_norm_factor_noalloc(3, i.data_ptr(), i.data_ptr(), p, p, p, 7, p, None) == \
        _capi.CF_BAD_INPUT
