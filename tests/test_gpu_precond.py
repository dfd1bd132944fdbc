"""GPU parity of the 2-level circulant preconditioner (build and apply) against
the FP64 oracle, through the C ABI.  Tolerances: FP64 device paths <= 1e-10
relative; the FP32 inversion + c64 apply <= 1e-4 relative (blocks inverted in
single precision)."""
import numpy as np
import pytest

import oracle as O
from voxscatter_gb300._lib import VoxScatterError
from voxscatter_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from voxscatter_gb300 import build
    build.build()
    from voxscatter_gb300 import api as A
    return A


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def _setup(p):
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx = p["idx"]
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    Toep = O.green_toeplitz(p["r"], p["ko"])
    alpha = O.alpha_ldr(p["refInd"], p["ko"], p["d"], p["kvec"], p["Eo"])
    return L, M, N, idx3, Toep, alpha, p["d"] ** 3


SHAPES = [dict(diameter=2.0, nper=3), dict(diameter=2.0, nper=5), dict(diameter=3.3, nper=4),
          dict(diameter=1.0, nper=2, aspect_ratio=0.2)]


@pytest.mark.parametrize("shape", SHAPES)
def test_circ_levels_match_oracle(api, shape):
    p = W.small_hex(m=1.31 + 0.05j, **shape)
    L, M, N, idx3, Toep, alpha, dV = _setup(p)
    _, c1_o = O.circ_1_level(Toep, L, M, N, 0, "off")
    c2_o, blk_o = O.circ_2_level(c1_o, L, M, N)
    _, c1 = api.circ_1_level(Toep, L, M, N, 0, "off")
    assert rel(c1, c1_o) < 1e-12
    c2, blk = api.circ_2_level(c1, L, M, N, opToeplitz=Toep)
    assert rel(c2, c2_o) < 1e-12
    assert rel(blk, blk_o) < 1e-12


@pytest.mark.parametrize("shape", SHAPES)
def test_prec_build_and_apply(api, shape):
    p = W.small_hex(m=1.31 + 0.05j, **shape)
    L, M, N, idx3, Toep, alpha, dV = _setup(p)
    _, c1_o = O.circ_1_level(Toep, L, M, N, 0, "off")
    _, blk_o = O.circ_2_level(c1_o, L, M, N)
    inv_o = O.invert_blocks(blk_o, 1 / alpha, dV)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    assert rel(pr.blocks(L, M, N, "c128"), inv_o) < 1e-10
    assert rel(pr.blocks(L, M, N, "c64"), inv_o) < 1e-4
    rng = np.random.default_rng(1)
    x = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
    y_o = O.mvp_circ_2_level(inv_o, x, L, M, N, idx3)
    assert rel(pr.apply(x, "c128"), y_o) < 1e-10
    assert rel(pr.apply(x, "c64"), y_o) < 1e-4
    # both GEMV kernels (register-direct; streamed in whole blocks or in
    # column chunks), one and five right-hand sides (5: 4 per CTA + 1)
    X = rng.normal(size=(5, idx3.size)) + 1j * rng.normal(size=(5, idx3.size))
    Y_o = np.array([O.mvp_circ_2_level(inv_o, X[k], L, M, N, idx3) for k in range(5)])
    for prec, tol in (("c128", 1e-10), ("c64", 1e-4)):
        # mode 2: packed symmetric blocks, chunk = ring depth
        for mode, chunk, ctas in ((0, 0, 2), (1, 0, 1), (1, 0, 2), (1, 2, 2), (1, 5, 1), (1, 0, 3), (1, 3, 4),
                                  (1, 0, 4), (2, 2, 1), (2, 3, 2), (2, 4, 4)):
            pr.set_shape(prec, gemv_mode=mode, gemv_chunk=min(chunk, 3 * N), gemv_blocks=ctas, gemv_threads=0)
            assert rel(pr.apply(x, prec), y_o) < tol, (prec, mode, chunk)
            Y = pr.apply(X.ravel(), prec).reshape(5, -1)
            assert rel(Y, Y_o) < tol, (prec, mode, chunk, "batched")
    # both FFTs of each plane in one CTA (c64; c128 planes of this size fit too)
    for prec, tol in (("c128", 1e-10), ("c64", 1e-4)):
        pr.set_shape(prec, gemv_mode=1, gemv_chunk=0, gemv_blocks=2, gemv_threads=0, fuse_xy=1)
        assert rel(pr.apply(x, prec), y_o) < tol, (prec, "fused")
        Y = pr.apply(X.ravel(), prec).reshape(5, -1)
        assert rel(Y, Y_o) < tol, (prec, "fused batched")
        pr.set_shape(prec, fuse_xy=0)
    # the MATLAB-style call with caller-supplied inverse blocks
    assert rel(api.mvp_circ_2_level(inv_o, x, L, M, N, idx3), y_o) < 1e-10


def test_prec_jvie_face_vector_and_batch(api):
    p = W.small_hex(m=1.5 + 0.1j, diameter=2.5, nper=3)
    L, M, N, idx3, Toep, alpha, dV = _setup(p)
    _, c1_o = O.circ_1_level(Toep, L, M, N, 0, "off")
    _, blk_o = O.circ_2_level(c1_o, L, M, N)
    rng = np.random.default_rng(2)
    # the face vector of scatteringHumanHead.m:157-177 from an inhomogeneous
    # permittivity grid (the library's averaging against the oracle's)
    eps_r = 1.8 + 0.4 * rng.normal(size=(L, M, N)) + 0.05j * rng.normal(size=(L, M, N))
    face3 = api.eps_layer_average(eps_r)
    assert rel(face3, O.eps_layer_average(eps_r)) < 1e-14
    gram = 0.8
    inv_o = O.invert_blocks(blk_o, gram, face3)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=gram, d=face3)
    with pytest.raises(VoxScatterError, match="packed"):  # a face vector breaks the block symmetry
        pr.set_shape("c128", gemv_mode=2, gemv_chunk=2)
    X = rng.normal(size=(3, idx3.size)) + 1j * rng.normal(size=(3, idx3.size))
    Y = pr.apply(X.ravel(), "c128").reshape(3, -1)
    for k in range(3):
        assert rel(Y[k], O.mvp_circ_2_level(inv_o, X[k], L, M, N, idx3)) < 1e-10


def test_prec_config1_size(api):
    """Hex plate 27x23x7 (23 is prime: generic radix-23 DFT along y)."""
    p = W.config1()
    L, M, N, idx3, Toep, alpha, dV = _setup(p)
    _, c1_o = O.circ_1_level(Toep, L, M, N, 0, "off")
    _, blk_o = O.circ_2_level(c1_o, L, M, N)
    inv_o = O.invert_blocks(blk_o, 1 / alpha, dV)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    x = np.random.default_rng(4).normal(size=idx3.size) + 0j
    y_o = O.mvp_circ_2_level(inv_o, x, L, M, N, idx3)
    assert rel(pr.apply(x, "c128"), y_o) < 1e-10
    assert rel(pr.apply(x, "c64"), y_o) < 1e-4
    for fuse in (0, 1):  # fused x/y planes with the generic radix-23 stage
        pr.set_shape("c64", fuse_xy=fuse)
        assert rel(pr.apply(x, "c64"), y_o) < 1e-4, fuse


def test_prec_full_storage_when_parity_is_not_exact(api):
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N, idx3, Toep, alpha, dV = _setup(p)
    Toep = Toep.copy()
    rng = np.random.default_rng(10)
    Toep[0, :, :, 2] += 1e-3 * rng.normal(size=(M, N))
    _, c1_o = O.circ_1_level(Toep, L, M, N, 0, "off")
    _, blk_o = O.circ_2_level(c1_o, L, M, N)
    inv_o = O.invert_blocks(blk_o, 1 / alpha, dV)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    assert rel(pr.blocks(L, M, N, "c128"), inv_o) < 1e-10
    x = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
    assert rel(pr.apply(x, "c128"), O.mvp_circ_2_level(inv_o, x, L, M, N, idx3)) < 1e-10
    with pytest.raises(VoxScatterError, match="packed"):  # no quadrant storage, no packed blocks
        pr.set_shape("c64", gemv_mode=2, gemv_chunk=2)


@pytest.mark.parametrize("N,L,M", [(48, 5, 6), (64, 6, 5)])
def test_prec_large_blocks(api, N, L, M):
    """3N x 3N blocks beyond the shared-memory inversion: n = 144 inverts in
    FP32 in shared memory and in FP64 with the blocked global-memory kernel;
    n = 192 (the 256x256x64 snowflake's block size) uses the blocked kernel in
    both precisions.  Largest block condition number here is about 115."""
    p = W.config5(level=2, L=L, M=M, N=N, layers=N - 8)
    L, M, N, idx3, Toep, alpha, dV = _setup(p)
    _, c1_o = O.circ_1_level(Toep, L, M, N, 0, "off")
    _, blk_o = O.circ_2_level(c1_o, L, M, N)
    inv_o = O.invert_blocks(blk_o, 1 / alpha, dV)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    assert rel(pr.blocks(L, M, N, "c128"), inv_o) < 1e-10
    assert rel(pr.blocks(L, M, N, "c64"), inv_o) < 1e-4
    _, blk = api.circ_2_level(api.circ_1_level(Toep, L, M, N, 0, "off")[1], L, M, N, opToeplitz=Toep)
    assert rel(blk, blk_o) < 1e-12
    rng = np.random.default_rng(5)
    x = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
    y_o = O.mvp_circ_2_level(inv_o, x, L, M, N, idx3)
    for prec, tol in (("c128", 1e-10), ("c64", 1e-4)):
        for mode, chunk in ((0, 0), (1, 0), (1, 16), (1, 7)):
            pr.set_shape(prec, gemv_mode=mode, gemv_chunk=chunk, gemv_blocks=1, gemv_threads=0)
            assert rel(pr.apply(x, prec), y_o) < tol, (prec, mode, chunk)
        # packed symmetric blocks where a two-block ring fits in shared memory
        # (n = 144 in c64); otherwise the mode is refused
        if prec == "c64" and 3 * N == 144:
            pr.set_shape(prec, gemv_mode=2, gemv_chunk=2, gemv_blocks=1, gemv_threads=0)
            assert rel(pr.apply(x, prec), y_o) < tol, (prec, "packed")
        else:
            with pytest.raises(VoxScatterError, match="packed"):
                pr.set_shape(prec, gemv_mode=2, gemv_chunk=2, gemv_blocks=1, gemv_threads=0)


@pytest.mark.parametrize("N,L,M", [(3, 5, 4), (12, 8, 6), (26, 6, 5), (40, 4, 4), (64, 3, 3), (80, 3, 2)])
def test_prec_tensor_core_inversion(api, N, L, M):
    """FP32 blocks inverted on the tensor cores (batched blocked Gauss-Jordan,
    tcgen05 3xTF32 trailing updates; forced for every 3N <= 256) against the
    oracle's FP64 inverses (inv of main_DDA.m:107-111) at the FP32 tolerance
    and against the CUDA-core FP32 inverses.  3N = 9 is one partial panel,
    3N = 36 two panels, 3N = 78 the 105x91x26 plate's block (a partial last
    panel and row tile), 3N = 120, 192 (the snowflake's block) and 240 several
    panels and row tiles."""
    p = W.config5(level=2, L=L, M=M, N=N, layers=max(N - 8, 1))
    L, M, N, idx3, Toep, alpha, dV = _setup(p)
    _, c1_o = O.circ_1_level(Toep, L, M, N, 0, "off")
    _, blk_o = O.circ_2_level(c1_o, L, M, N)
    inv_o = O.invert_blocks(blk_o, 1 / alpha, dV)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr_tc = api.Preconditioner(op, shift=1 / alpha, d=dV, precisions=("c64",), lu="tc")
    pr_cu = api.Preconditioner(op, shift=1 / alpha, d=dV, precisions=("c64",), lu="cuda")
    b_tc, b_cu = pr_tc.blocks(L, M, N, "c64"), pr_cu.blocks(L, M, N, "c64")
    assert np.all(np.isfinite(b_tc))
    assert rel(b_tc, inv_o) < 1e-4
    assert rel(b_tc, b_cu) < 1e-4
    # every block individually (a wrong panel or tile shows in one block)
    for i in range(L):
        for j in range(M):
            assert rel(b_tc[i, j], inv_o[i, j]) < 1e-4, (i, j)
    rng = np.random.default_rng(9)
    x = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
    assert rel(pr_tc.apply(x, "c64"), O.mvp_circ_2_level(inv_o, x, L, M, N, idx3)) < 1e-4


@pytest.mark.parametrize("n", [17, 78, 192, 256, 300])
def test_invert_blocks_device(api, n):
    """vs_invert_blocks_device on a batch of complex FP32 matrices, tensor
    cores (n <= 256) and CUDA cores, against FP64 inverses; a singular matrix
    in the batch is reported."""
    import torch
    rng = np.random.default_rng(n)
    nmat = 5
    A = (rng.normal(size=(nmat, n, n)) + 1j * rng.normal(size=(nmat, n, n))) * (0.5 / np.sqrt(n)) + \
        np.eye(n) * (1.0 + 0.3j)
    inv = np.linalg.inv(A)
    for method in (("tc", "cuda", "auto") if n <= 256 else ("auto", "cuda")):
        W = torch.tensor(A, dtype=torch.complex64, device="cuda")
        torch.cuda.synchronize()
        api.invert_blocks_device(W.data_ptr(), n, nmat, method)
        Wh = W.cpu().numpy()
        for k in range(nmat):
            assert rel(Wh[k], inv[k]) < 1e-5, (method, k)
    S = A.copy()
    S[2] = 0
    W = torch.tensor(S, dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    with pytest.raises(VoxScatterError, match="singular"):
        api.invert_blocks_device(W.data_ptr(), n, nmat, "auto")


def test_streamed_gemv_wait_that_runs_out_is_reported_and_recovered(api):
    """The streamed GEMV's waits on other warp roles are bounded; with the
    bound set to none every such wait gives up at once: the CTAs stop (the
    producer still lets its own copies land), the apply reports
    VS_ERR_TIMEOUT, and with the default bound restored the next apply is
    correct."""
    from voxscatter_gb300 import _lib
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N, idx3, Toep, alpha, dV = _setup(p)
    _, c1_o = O.circ_1_level(Toep, L, M, N, 0, "off")
    _, blk_o = O.circ_2_level(c1_o, L, M, N)
    inv_o = O.invert_blocks(blk_o, 1 / alpha, dV)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    x = np.random.default_rng(4).normal(size=idx3.size) + 0j
    y_o = O.mvp_circ_2_level(inv_o, x, L, M, N, idx3)
    for prec, tol in (("c64", 1e-4), ("c128", 1e-10)):
        pr.set_shape(prec, gemv_mode=1, gemv_chunk=0, gemv_blocks=1, gemv_threads=0, fuse_xy=0, wait_polls=-1)
        with pytest.raises(VoxScatterError) as e:
            pr.apply(x, prec)
        assert e.value.status == _lib.VS_ERR_TIMEOUT
        pr.set_shape(prec, wait_polls=0)
        assert pr.shape(prec)["wait_polls"] == 0
        assert rel(pr.apply(x, prec), y_o) < tol
        assert rel(pr.apply(x, prec), y_o) < tol


def test_prec_build_options_rejected(api):
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.0, nper=3)
    L, M, N, idx3, Toep, alpha, dV = _setup(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    from voxscatter_gb300 import _lib
    import ctypes
    h = ctypes.c_void_p()
    sh = np.array([1 / alpha], dtype=np.complex128)
    dd = np.array([dV], dtype=np.complex128)
    both = _lib.VS_BUILD_C64 | _lib.VS_BUILD_LU_TC | _lib.VS_BUILD_LU_CUDA
    st = op.ctx._lib.vs_prec_create(op.h, _lib.dptr(sh), _lib.dptr(dd), 1, both, ctypes.byref(h))
    assert st == _lib.VS_ERR_ARG
    st = op.ctx._lib.vs_prec_create(op.h, _lib.dptr(sh), _lib.dptr(dd), 1, _lib.VS_BUILD_LU_TC, ctypes.byref(h))
    assert st == _lib.VS_ERR_ARG


def test_context_outlives_its_objects(api):
    """vs_ctx_destroy before the operator and preconditioner made on the
    context: both keep working (they hold the context) and are released
    afterwards in any order."""
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.0, nper=3)
    L, M, N, idx3, Toep, alpha, dV = _setup(p)
    ctx = api.Context(0)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep, ctx=ctx)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    x = np.random.default_rng(3).normal(size=idx3.size) + 0j
    y0, z0 = op.apply(x, "notransp", "c128"), pr.apply(x, "c128")
    raw = ctx.h
    ctx.h = None  # the Python wrapper forgets it; the library keeps it for op and pr
    ctx._lib.vs_ctx_destroy(raw)
    assert rel(op.apply(x, "notransp", "c128"), y0) < 1e-14
    assert rel(pr.apply(x, "c128"), z0) < 1e-14
    op.close()
    assert rel(pr.apply(x, "c128"), z0) < 1e-14
    pr.close()


def test_prec_fused_planes_hexplate_105x91x26(api):
    """The fused x/y plane kernel (105 x 91 planes, 78 of them) against the
    separate two-level passes at the bench size, c64, 1 and 4 right-hand sides
    (<= 2e-6 relative: the two paths round differently)."""
    p = W.config2()
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx3 = np.concatenate([p["idx"], nD + p["idx"], 2 * nD + p["idx"]])
    Toep = api.green_dda(p["r"], p["ko"])
    alpha = api.alpha_ldr(p["refInd"], p["ko"], p["d"], p["kvec"], p["Eo"])
    dV = p["d"] ** 3
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV, precisions=("c64",))
    rng = np.random.default_rng(8)
    X = rng.normal(size=(4, idx3.size)) + 1j * rng.normal(size=(4, idx3.size))
    pr.set_shape("c64", x_reg=1, y_reg=1, fuse_xy=0)
    y_sep = pr.apply(X[0], "c64")
    Y_sep = pr.apply(X.ravel(), "c64").reshape(4, -1)
    pr.set_shape("c64", fuse_xy=1)
    assert rel(pr.apply(X[0], "c64"), y_sep) < 2e-6
    assert rel(pr.apply(X.ravel(), "c64").reshape(4, -1), Y_sep) < 2e-6
