"""The allocation-free apply (vs_op_apply_device_noalloc) against the ordinary
device apply and against the oracle's MVP, through the C ABI.

This entry point exists for callers that cannot allocate device memory when
they need a matvec: services that reserve their device memory at start-up and
forbid allocation afterwards, and hosts that run the solver inside a memory
budget owned by another allocator.  Its pipeline intermediates live in a
static 64 MiB device array that every call shares.  The file is named to be
collected last, so a run that stops at the first failure has already run every
other test; it builds everything it needs itself, so it also passes alone in a
fresh process."""
import ctypes

import numpy as np
import pytest

import oracle as O
from oracle.mvp import MVP_plain_transpose
from voxscatter_gb300 import workloads as W

pytestmark = pytest.mark.gpu

C64_TOL = 5e-6
C128_TOL = 1e-11


def _rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


@pytest.fixture(scope="module")
def setup():
    from voxscatter_gb300 import build
    build.build()
    from voxscatter_gb300 import api, _lib
    p = W.small_hex(m=1.31 + 0.05j, diameter=3.0, nper=4)
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx = p["idx"]
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    fN, Toep, alpha = O.getOPERATOR_DDA(p["r"], p["ko"], p["refInd"], p["kvec"], p["Eo"])
    dV = p["d"] ** 3
    chi = np.zeros(nD); chi[idx] = 1
    Mc = dV * chi.reshape((L, M, N), order="F")
    rng = np.random.default_rng(3)
    # a complex per-voxel Mr makes the three modes differ in their diagonal term
    Mr = 1 + 0.1 * (rng.random((L, M, N)) + 1j * rng.random((L, M, N)))
    op = api.Operator(L, M, N, idx3, Mr, Mc, 1 / alpha, toep=Toep)
    oracle_modes = {
        _lib.VS_NOTRANSP: lambda v: O.MVP(v, fN, Mr, Mc, 1 / alpha, "notransp", idx3),
        _lib.VS_CONJTRANSP: lambda v: O.MVP(v, fN, Mr, Mc, 1 / alpha, "transp", idx3),
        _lib.VS_TRANSP: lambda v: MVP_plain_transpose(v, fN, Mr, Mc, 1 / alpha, idx3),
    }
    return api, _lib, op, idx3, oracle_modes


@pytest.mark.parametrize("nrhs", [1, 3])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_noalloc_apply_matches_device_apply_and_oracle(setup, mode, nrhs):
    import torch
    api, _lib, op, idx3, oracle_modes = setup
    lib = op.ctx._lib
    rng = np.random.default_rng(21 + 7 * mode + nrhs)
    n = idx3.size
    for dtype, prec, tol in ((torch.complex64, _lib.VS_C64, C64_TOL), (torch.complex128, _lib.VS_C128, C128_TOL)):
        for call in range(2):  # two calls in a row share (and reuse) the static scratch
            xh = rng.normal(size=(nrhs, n)) + 1j * rng.normal(size=(nrhs, n))
            x = torch.tensor(xh, dtype=dtype, device="cuda")
            y_ref = torch.empty_like(x)
            y_new = torch.full_like(x, float("nan"))
            torch.cuda.synchronize()
            _lib.check(lib.vs_op_apply_device(op.h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y_ref.data_ptr()),
                                              nrhs, mode, prec), op.ctx.h)
            _lib.check(lib.vs_op_apply_device_noalloc(op.h, ctypes.c_void_p(x.data_ptr()),
                                                      ctypes.c_void_p(y_new.data_ptr()), nrhs, mode, prec),
                       op.ctx.h)
            op.ctx.synchronize()
            a, b = y_new.cpu().numpy(), y_ref.cpu().numpy()
            assert np.all(np.isfinite(a))
            assert _rel(a, b) < tol, (dtype, mode, nrhs, call)
            xr = x.cpu().numpy().astype(np.complex128)  # the rounded input the GPU saw
            for r in range(nrhs):
                assert _rel(a[r], oracle_modes[mode](xr[r])) < tol, (dtype, mode, nrhs, call, r)


def test_noalloc_rejects_sizes_beyond_the_static_array(setup):
    import torch
    api, _lib, op, idx3, _ = setup
    lib = op.ctx._lib
    # 96 x 96 x 32 grid: c128 intermediates of ~85 MB exceed the 64 MiB array
    big = api.Operator(96, 96, 32, np.arange(3 * 96 * 96 * 32), 1.0, 1e-3, 2.0,
                       toep=np.zeros((96, 96, 32, 6), complex))
    xb = torch.zeros(big.n3, dtype=torch.complex128, device="cuda")
    yb = torch.empty_like(xb)
    torch.cuda.synchronize()
    st = lib.vs_op_apply_device_noalloc(big.h, ctypes.c_void_p(xb.data_ptr()), ctypes.c_void_p(yb.data_ptr()), 1,
                                        _lib.VS_NOTRANSP, _lib.VS_C128)
    assert st == _lib.VS_ERR_UNSUPPORTED
    assert b"static limit" in lib.vs_last_error(big.ctx.h)
    # the thread's last error carries the same message
    assert b"static limit" in lib.vs_last_error(None)
