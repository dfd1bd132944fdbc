"""GPU parity of operator assembly and the fused FFT matvec against the FP64
oracle (through the C ABI).  Tolerances: FP64 device paths <= 1e-12 relative
(setup) / 1e-11 (c128 matvec); the c64 pipeline <= 5e-6 relative in the 2-norm."""
import numpy as np
import pytest

import oracle as O
from oracle.mvp import MVP_plain_transpose
from voxscatter_gb300 import workloads as W
from voxscatter_gb300._lib import VoxScatterError

pytestmark = pytest.mark.gpu

C128_TOL = 1e-11
C64_TOL = 5e-6


@pytest.fixture(scope="module")
def api():
    from voxscatter_gb300 import build
    build.build()
    from voxscatter_gb300 import api as A
    return A


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def _problem(p):
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx = p["idx"]
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    chi = np.zeros(nD); chi[idx] = 1
    chi = chi.reshape((L, M, N), order="F")
    return L, M, N, idx3, chi


@pytest.mark.parametrize("nearby", ["off", "on"])
def test_green_and_circulant_fft(api, nearby):
    p = W.small_hex(m=1.31 + 0.05j)
    Toep_o = O.green_toeplitz(p["r"], p["ko"], nearby)
    Toep_g = api.green_dda(p["r"], p["ko"], nearby)
    assert rel(Toep_g, Toep_o) < 1e-12
    fN_o = O.fft_operator(O.circulant_nop_const(Toep_o))
    fN_g = api.circulant_fft(Toep_o)
    assert rel(fN_g, fN_o) < 1e-12
    a_o = O.alpha_ldr(p["refInd"], p["ko"], p["d"], p["kvec"], p["Eo"])
    a_g = api.alpha_ldr(p["refInd"], p["ko"], p["d"], p["kvec"], p["Eo"])
    assert abs(a_g - a_o) <= 1e-14 * abs(a_o)


SHAPES = [
    dict(diameter=2.0, nper=3),      # 8x7x2
    dict(diameter=2.0, nper=5),      # odd sizes
    dict(diameter=3.3, nper=4),
    dict(diameter=1.0, nper=2, aspect_ratio=0.2),
]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("flag", ["notransp", "transp"])
def test_mvp_matches_oracle(api, shape, flag):
    p = W.small_hex(m=1.31 + 0.05j, **shape)
    L, M, N, idx3, chi = _problem(p)
    fN, Toep, alpha = O.getOPERATOR_DDA(p["r"], p["ko"], p["refInd"], p["kvec"], p["Eo"])
    dV = p["d"] ** 3
    rng = np.random.default_rng(7)
    x = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
    Mr = np.ones((L, M, N))
    y_o = O.MVP(x, fN, Mr, dV * chi, 1 / alpha, flag, idx3)
    # reference-style call: the reference's own fN (P=2L)
    y_ref = api.MVP(x, fN, Mr, dV * chi, 1 / alpha, flag, idx3, precision="c128")
    assert rel(y_ref, y_o) < C128_TOL
    # handle built from the Toeplitz tensor at 7-smooth sizes
    op = api.Operator(L, M, N, idx3, Mr, dV * chi, 1 / alpha, toep=Toep)
    assert op.PQR[0] >= 2 * L - 1
    assert rel(op.apply(x, flag, "c128"), y_o) < C128_TOL
    assert rel(op.apply(x, flag, "c64"), y_o) < C64_TOL


def test_plain_transpose_and_varying_diagonals(api):
    p = W.small_hex(m=1.4 + 0.1j, diameter=2.5, nper=3)
    L, M, N, idx3, chi = _problem(p)
    Toep = O.green_toeplitz(p["r"], p["ko"])
    fN = O.fft_operator(O.circulant_nop_const(Toep))
    rng = np.random.default_rng(3)
    Mc = (1 + 0.3 * rng.normal(size=(L, M, N))) + 0.1j * rng.normal(size=(L, M, N))
    Mr = 1 + 0.2j * rng.normal(size=(L, M, N))
    Gram = 0.7 + 0.05 * rng.normal(size=(L, M, N))
    x = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
    op = api.Operator(L, M, N, idx3, Mr, Mc, Gram, toep=Toep)
    for flag in ("notransp", "transp"):
        y_o = O.MVP(x, fN, Mr, Mc, Gram, flag, idx3)
        assert rel(op.apply(x, flag, "c128"), y_o) < C128_TOL
        assert rel(op.apply(x, flag, "c64"), y_o) < C64_TOL
    y_o = MVP_plain_transpose(x, fN, Mr, Mc, Gram * Mr / Mr, idx3)
    assert rel(op.apply(x, "plain_transp", "c128"), y_o) < C128_TOL


def test_batched_rhs_and_all_voxels(api):
    p = W.small_hex(m=1.31, diameter=2.0, nper=4)
    L, M, N, _, _ = _problem(p)
    idx3 = np.arange(3 * L * M * N)
    Toep = O.green_toeplitz(p["r"], p["ko"])
    fN = O.fft_operator(O.circulant_nop_const(Toep))
    op = api.Operator(L, M, N, idx3, 1.0, 0.01, 3.0, toep=Toep)
    rng = np.random.default_rng(5)
    X = rng.normal(size=(4, idx3.size)) + 1j * rng.normal(size=(4, idx3.size))
    Y = op.apply(X.ravel(), "notransp", "c64").reshape(4, -1)
    for k in range(4):
        y_o = O.MVP(X[k], fN, np.ones((L, M, N)), 0.01, 3.0, "notransp", idx3)
        assert rel(Y[k], y_o) < C64_TOL


def test_single_layer_and_line_grids(api):
    from voxscatter_gb300.geometry import grid3d
    for (L, M, N) in [(1, 5, 3), (6, 1, 1), (3, 4, 1), (1, 1, 1), (17, 3, 2)]:
        r = grid3d(np.arange(L) * 0.1, np.arange(M) * 0.1, np.arange(N) * 0.1)
        ko = 2 * np.pi
        Toep = O.green_toeplitz(r, ko)
        fN = O.fft_operator(O.circulant_nop_const(Toep))
        idx3 = np.arange(3 * L * M * N)
        op = api.Operator(L, M, N, idx3, 1.0, 1e-3, 2.0, toep=Toep)
        x = np.random.default_rng(L).normal(size=idx3.size) + 0j
        y_o = O.MVP(x, fN, np.ones((L, M, N)), 1e-3, 2.0, "notransp", idx3)
        assert rel(op.apply(x, "notransp", "c128"), y_o) < C128_TOL


def test_config2_full_size_c64(api):
    """Hex plate 105x91x26 (186,238 voxels): c64 pipeline vs the FP64 oracle and
    linearity at full size."""
    p = W.config2()
    L, M, N, idx3, chi = _problem(p)
    Toep = api.green_dda(p["r"], p["ko"])
    alpha = api.alpha_ldr(p["refInd"], p["ko"], p["d"], p["kvec"], p["Eo"])
    dV = p["d"] ** 3
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    rng = np.random.default_rng(11)
    x = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
    fN = O.fft_operator(O.circulant_nop_const(Toep))
    y_o = O.MVP(x, fN, np.ones((L, M, N)), dV * chi, 1 / alpha, "notransp", idx3)
    y64 = op.apply(x, "notransp", "c64")
    assert rel(y64, y_o) < C64_TOL
    y2 = op.apply(np.concatenate([x, 2 * x - 1j * x]), "notransp", "c64").reshape(2, -1)
    assert rel(y2[1], (2 - 1j) * y64) < C64_TOL


def test_full_storage_when_parity_is_not_exact(api):
    """Odd components made non-zero on their zero-offset planes: the library
    must fall back to full spectrum storage and still match the oracle."""
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N, idx3, chi = _problem(p)
    Toep = O.green_toeplitz(p["r"], p["ko"]).copy()
    rng = np.random.default_rng(9)
    Toep[0, :, :, 1] += 1e-3 * rng.normal(size=(M, N))
    Toep[:, :, 0, 4] += 1e-3 * rng.normal(size=(L, M))
    fN = O.fft_operator(O.circulant_nop_const(Toep))
    alpha = O.alpha_ldr(p["refInd"], p["ko"], p["d"], p["kvec"], p["Eo"])
    dV = p["d"] ** 3
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    x = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
    y_o = O.MVP(x, fN, np.ones((L, M, N)), dV * chi, 1 / alpha, "notransp", idx3)
    assert rel(op.apply(x, "notransp", "c128"), y_o) < C128_TOL
    assert rel(op.apply(x, "notransp", "c64"), y_o) < C64_TOL


@pytest.mark.parametrize("nper,diameter,aspect", [(4, 2.5, 0.5), (10, 2.0, 0.5), (6, 3.0, 0.35), (3, 2.0, 0.9)])
def test_every_launch_shape_matches_oracle(api, nper, diameter, aspect):
    """Both z-pass kernels (two-level registers and shared-memory Stockham)
    and several x/y/z tiles give the same c64 matvec as the oracle."""
    p = W.small_hex(m=1.31 + 0.05j, diameter=diameter, nper=nper, aspect_ratio=aspect)
    L, M, N, idx3, chi = _problem(p)
    Toep = O.green_toeplitz(p["r"], p["ko"])
    fN = O.fft_operator(O.circulant_nop_const(Toep))
    alpha = O.alpha_ldr(p["refInd"], p["ko"], p["d"], p["kvec"], p["Eo"])
    dV = p["d"] ** 3
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    rng = np.random.default_rng(N)
    x = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
    y_o = O.MVP(x, fN, np.ones((L, M, N)), dV * chi, 1 / alpha, "notransp", idx3)
    for z_reg in (0, 1, 2):
        for lg in (1, 3):
            op.set_shape("c64", z_reg=z_reg, lg_tile_z=lg, lg_tile_y=lg + 1, lg_lines_x=lg)
            assert rel(op.apply(x, "notransp", "c64"), y_o) < C64_TOL, (z_reg, lg, op.PQR)


Z_LENGTHS = [4, 6, 8, 9, 10, 12, 15, 16, 18, 20, 24, 27, 30, 32, 36, 40, 45, 48, 54, 60, 64, 72, 80, 90, 96, 108,
             120, 128, 144, 160, 180, 192, 216, 240, 256]


@pytest.mark.parametrize("R", Z_LENGTHS)
def test_z_lengths_both_z_kernels(api, R):
    """Every z length with a two-level register kernel (R = R1*R2), forced on a
    3 x 2 x ceil(R/2) block of voxels: the two-level and the shared-memory
    Stockham z passes (two-level with and without its register cap) in c64
    and c128, with the first-octant spectrum and,
    after breaking the Toeplitz parity, with the full spectrum."""
    from voxscatter_gb300.geometry import grid3d
    L, M, N = 3, 2, (R + 1) // 2
    d = 0.07
    r = grid3d(np.arange(L) * d, np.arange(M) * d, np.arange(N) * d)
    ko = 2 * np.pi
    rng = np.random.default_rng(R)
    for exact_parity in (True, False):
        Toep = O.green_toeplitz(r, ko)
        if not exact_parity:
            Toep = Toep.copy()
            Toep[0, :, :, 2] += 1e-2 * np.abs(Toep).max() * rng.normal(size=(M, N))
        fN = O.fft_operator(O.circulant_nop_const(Toep))
        idx3 = np.arange(3 * L * M * N)
        op = api.Operator(L, M, N, idx3, 1.0, d ** 3, 3.0, toep=Toep, PQR=(0, 0, R))
        assert op.PQR[2] == R
        x = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
        y_o = O.MVP(x, fN, np.ones((L, M, N)), d ** 3, 3.0, "notransp", idx3)
        for prec, tol in (("c64", C64_TOL), ("c128", C128_TOL)):
            for z_reg in (0, 1, 2):
                op.set_shape(prec, z_reg=z_reg, z_df=0)
                assert rel(op.apply(x, "notransp", prec), y_o) < tol, (prec, z_reg, exact_parity, op.PQR)
        # c128 with double-float arithmetic in the z pass (lengths up to 64; the
        # others keep the FP64 kernel): the same FP64 tolerance, all modes
        op.set_shape("c128", z_reg=2, z_df=1)
        assert rel(op.apply(x, "notransp", "c128"), y_o) < C128_TOL, ("df", exact_parity, op.PQR)
        for mode in ("transp", "plain_transp"):
            op.set_shape("c128", z_df=0)
            ref = op.apply(x, mode, "c128")
            op.set_shape("c128", z_df=1)
            assert rel(op.apply(x, mode, "c128"), ref) < C128_TOL, ("df", mode, exact_parity)


Y_LENGTHS = [8, 9, 10, 12, 15, 16, 18, 20, 24, 25, 27, 30, 32, 36, 40, 45, 48, 50, 54, 60, 64, 72, 75, 80, 81, 90,
             91, 96, 100, 108, 120, 125, 128, 135, 144, 150, 160, 162, 180, 192, 200, 216, 225, 240, 243, 250, 256,
             288, 320, 384, 432, 480, 512]


@pytest.mark.parametrize("n", Y_LENGTHS)
def test_y_lengths_both_y_kernels(api, n):
    """Every strided length with a two-level register kernel: the matvec's
    y passes with Q = n forced (M = ceil(n/2)) and the preconditioner's y
    passes with M = n, in c64 and c128, two-level and shared-memory Stockham
    (c128 also two-level in double-float arithmetic, where the length has that
    kernel), against the oracle on a 3 x M x 2 block of voxels (tolerances in
    the body)."""
    from voxscatter_gb300.geometry import grid3d
    rng = np.random.default_rng(n)
    d, ko = 0.07, 2 * np.pi
    for M, PQR, check_prec in (((n + 1) // 2, (0, n, 0), False), (n, (0, 0, 0), True)):
        L, N = 3, 2
        r = grid3d(np.arange(L) * d, np.arange(M) * d, np.arange(N) * d)
        Toep = O.green_toeplitz(r, ko)
        fN = O.fft_operator(O.circulant_nop_const(Toep))
        idx3 = np.arange(3 * L * M * N)
        op = api.Operator(L, M, N, idx3, 1.0, d ** 3, 3.0, toep=Toep, PQR=PQR)
        if not check_prec:
            assert op.PQR[1] == n
        x = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
        y_o = O.MVP(x, fN, np.ones((L, M, N)), d ** 3, 3.0, "notransp", idx3)
        for prec, tol in (("c64", C64_TOL), ("c128", C128_TOL)):
            for y_reg in ((0, 1) if prec == "c64" else (0, 1, 2)):
                op.set_shape(prec, y_reg=y_reg)
                assert rel(op.apply(x, "notransp", prec), y_o) < tol, (prec, y_reg, op.PQR)
        if check_prec:
            _, c1 = O.circ_1_level(Toep, L, M, N, 0, "off")
            _, blk = O.circ_2_level(c1, L, M, N)
            inv = O.invert_blocks(blk, 3.0, d ** 3)
            pr = api.Preconditioner(op, shift=3.0, d=d ** 3)
            z_o = O.mvp_circ_2_level(inv, x, L, M, N, idx3)
            for y_reg in (0, 1):
                pr.set_shape("c128", y_reg=y_reg)
                assert rel(pr.apply(x, "c128"), z_o) < 1e-10, ("c128", y_reg, M)
            # c64: the two kernels on the same FP32-inverted blocks agree to FFT
            # rounding; against the FP64 oracle the FP32 inversion of these
            # blocks (shift 3, d = 0.07) bounds the error
            pr.set_shape("c64", y_reg=0)
            z0 = pr.apply(x, "c64")
            pr.set_shape("c64", y_reg=1)
            z1 = pr.apply(x, "c64")
            assert rel(z1, z0) < 2e-6, M
            assert rel(z1, z_o) < 1e-3, M


X_LENGTHS = Y_LENGTHS + [105]


@pytest.mark.parametrize("n", X_LENGTHS)
def test_x_lengths_both_x_kernels(api, n):
    """Every x length with a two-level register kernel: the matvec's x passes
    with P = n forced (L = ceil(n/2), a quarter of the voxels absent, varying
    diagonals, all three modes) and the preconditioner's x passes with L = n,
    c64 and c128, two-level and shared-memory Stockham (the matvec's c128 also
    two-level in double-float arithmetic, where the length has that kernel),
    against the oracle (tolerances in the body)."""
    from voxscatter_gb300.geometry import grid3d
    rng = np.random.default_rng(1000 + n)
    d, ko = 0.07, 2 * np.pi
    for L, PQR, check_prec in (((n + 1) // 2, (n, 0, 0), False), (n, (0, 0, 0), True)):
        M, N = 2, 2
        r = grid3d(np.arange(L) * d, np.arange(M) * d, np.arange(N) * d)
        Toep = O.green_toeplitz(r, ko)
        fN = O.fft_operator(O.circulant_nop_const(Toep))
        nD = L * M * N
        vox = np.sort(rng.choice(nD, size=max(1, (3 * nD) // 4), replace=False))
        idx3 = np.concatenate([vox, nD + vox, 2 * nD + vox])
        Mc = d ** 3 * ((1 + 0.3 * rng.normal(size=(L, M, N))) + 0.1j * rng.normal(size=(L, M, N)))
        Mr = 1 + 0.2j * rng.normal(size=(L, M, N))
        Gram = 3.0 + 0.05 * rng.normal(size=(L, M, N))
        op = api.Operator(L, M, N, idx3, Mr, Mc, Gram, toep=Toep, PQR=PQR)
        if not check_prec:
            assert op.PQR[0] == n
        x = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
        for flag in ("notransp", "transp"):
            y_o = O.MVP(x, fN, Mr, Mc, Gram, flag, idx3)
            for prec, tol in (("c64", C64_TOL), ("c128", C128_TOL)):
                for x_reg in ((0, 1) if prec == "c64" else (0, 1, 2)):
                    op.set_shape(prec, x_reg=x_reg)
                    assert rel(op.apply(x, flag, prec), y_o) < tol, (flag, prec, x_reg, op.PQR)
        with pytest.raises(VoxScatterError, match="VS_C128 only"):
            op.set_shape("c64", x_reg=2)
        y_t = MVP_plain_transpose(x, fN, Mr, Mc, Gram, idx3)
        for x_reg in (0, 1, 2):
            op.set_shape("c128", x_reg=x_reg)
            assert rel(op.apply(x, "plain_transp", "c128"), y_t) < C128_TOL, (x_reg, op.PQR)
        if check_prec:
            pr = api.Preconditioner(op, shift=3.0, d=d ** 3)
            z = {}
            for prec in ("c64", "c128"):
                for x_reg in (0, 1):
                    pr.set_shape(prec, x_reg=x_reg)
                    z[prec, x_reg] = pr.apply(x, prec)
            assert rel(z["c128", 1], z["c128", 0]) < 1e-12, L
            assert rel(z["c64", 1], z["c64", 0]) < 2e-6, L


@pytest.mark.parametrize("flag", ["notransp", "transp", "plain_transp"])
@pytest.mark.parametrize("per_voxel", [False, True])
def test_apply_with_gram_per_rhs(api, flag, per_voxel):
    """MVP.m called with a different Gram for each right-hand side (the DDA
    drivers' Gram = 1/alpha_LDR of each incident direction and polarisation):
    vs_op_apply_gram on three right-hand sides against three oracle MVP calls,
    with a complex per-voxel Mr so that Gram_r .* Mr (and Gram_r .* conj(Mr) in
    'transp') is exercised, scalar or per-voxel Gram_r."""
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N, idx3, chi = _problem(p)
    fN, Toep, alpha = O.getOPERATOR_DDA(p["r"], p["ko"], p["refInd"], p["kvec"], p["Eo"])
    dV = p["d"] ** 3
    rng = np.random.default_rng(31)
    Mr = 1 + 0.2 * (rng.random((L, M, N)) + 1j * rng.random((L, M, N)))
    op = api.Operator(L, M, N, idx3, Mr, dV * chi, 1 / alpha, toep=Toep)
    nrhs = 3
    X = rng.normal(size=(nrhs, idx3.size)) + 1j * rng.normal(size=(nrhs, idx3.size))
    if per_voxel:
        grams = (1 / alpha) * (1 + 0.1 * (rng.normal(size=(nrhs, L, M, N)) + 1j * rng.normal(size=(nrhs, L, M, N))))
    else:
        grams = (1 / alpha) * np.array([1.0, 1.013 - 0.004j, 0.987 + 0.02j])
    for r in range(nrhs):
        if flag == "plain_transp":
            y_o = MVP_plain_transpose(X[r], fN, Mr, dV * chi, grams[r], idx3)
        else:
            y_o = O.MVP(X[r], fN, Mr, dV * chi, grams[r], flag, idx3)
        Y128 = op.apply(X.ravel(), flag, "c128", gram=grams).reshape(nrhs, -1)
        Y64 = op.apply(X.ravel(), flag, "c64", gram=grams).reshape(nrhs, -1)
        assert rel(Y128[r], y_o) < C128_TOL, r
        assert rel(Y64[r], y_o) < C64_TOL, r
    # the operator's own Gram is untouched by a call with per-rhs Grams
    y0 = O.MVP(X[0], fN, Mr, dV * chi, 1 / alpha, "notransp", idx3)
    assert rel(op.apply(X[0], "notransp", "c128"), y0) < C128_TOL
