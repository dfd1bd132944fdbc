"""The allocation-free apply (vs_op_apply_device_noalloc) against the ordinary
device apply, through the C ABI.

This entry point exists for callers that cannot allocate device memory when
they need a matvec (stream capture, fixed-memory services); its pipeline
intermediates live in a static 64 MiB device array.  The file is named to be
collected last, so a run that stops at the first failure has already run every
other test."""
import ctypes

import numpy as np
import pytest

import oracle as O
from voxscatter_gb300 import workloads as W

pytestmark = pytest.mark.gpu

C64_TOL = 5e-6
C128_TOL = 1e-11


def test_noalloc_apply_matches_device_apply():
    import torch
    from voxscatter_gb300 import build
    build.build()
    from voxscatter_gb300 import api, _lib
    p = W.small_hex(m=1.31 + 0.05j, diameter=3.0, nper=4)
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx = p["idx"]
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    Toep = O.green_toeplitz(p["r"], p["ko"])
    alpha = O.alpha_ldr(p["refInd"], p["ko"], p["d"], p["kvec"], p["Eo"])
    dV = p["d"] ** 3
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    lib = op.ctx._lib
    rng = np.random.default_rng(21)
    for dtype, prec, tol in ((torch.complex64, _lib.VS_C64, C64_TOL), (torch.complex128, _lib.VS_C128, C128_TOL)):
        for call in range(2):  # two calls in a row share (and reuse) the static scratch
            x = torch.tensor(rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size), dtype=dtype,
                             device="cuda")
            y_ref = torch.empty_like(x)
            y_new = torch.full_like(x, float("nan"))
            torch.cuda.synchronize()
            _lib.check(lib.vs_op_apply_device(op.h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y_ref.data_ptr()),
                                              1, _lib.VS_NOTRANSP, prec), op.ctx.h)
            _lib.check(lib.vs_op_apply_device_noalloc(op.h, ctypes.c_void_p(x.data_ptr()),
                                                      ctypes.c_void_p(y_new.data_ptr()), 1, _lib.VS_NOTRANSP, prec),
                       op.ctx.h)
            op.ctx.synchronize()
            a, b = y_new.cpu().numpy(), y_ref.cpu().numpy()
            assert np.all(np.isfinite(a))
            assert np.linalg.norm(a - b) / np.linalg.norm(b) < tol, (dtype, call)
    # a request beyond the static limit is rejected with a clear error
    # 96 x 96 x 32 grid: c128 intermediates of ~85 MB exceed the 64 MiB array
    big = api.Operator(96, 96, 32, np.arange(3 * 96 * 96 * 32), 1.0, 1e-3, 2.0,
                       toep=np.zeros((96, 96, 32, 6), complex))
    xb = torch.zeros(big.n3, dtype=torch.complex128, device="cuda")
    yb = torch.empty_like(xb)
    st = lib.vs_op_apply_device_noalloc(big.h, ctypes.c_void_p(xb.data_ptr()), ctypes.c_void_p(yb.data_ptr()), 1,
                                        _lib.VS_NOTRANSP, _lib.VS_C128)
    assert st == _lib.VS_ERR_UNSUPPORTED
    assert b"static limit" in lib.vs_last_error(big.ctx.h)
