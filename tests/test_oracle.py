"""The FP64 oracle against independent mathematics (CPU only)."""
import math
import os

import numpy as np
import pytest

import oracle as O
from oracle.mvp import MVP_plain_transpose
from voxscatter_gb300 import workloads as W
from voxscatter_gb300.geometry import geometry


def _grid_from_vox(L, M, N, idx, vals):
    g = np.zeros(L * M * N, dtype=complex)
    g[idx] = vals
    return g.reshape((L, M, N), order="F")


def _setup(p, nearby="off"):
    fN, Toep, alpha = O.getOPERATOR_DDA(p["r"], p["ko"], p["refInd"], p["kvec"], p["Eo"], nearby)
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx = p["idx"]
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    chi = _grid_from_vox(L, M, N, idx, 1.0)
    dV = p["d"] ** 3
    return fN, Toep, alpha, idx3, chi, dV


@pytest.mark.parametrize("m", [1.31, 1.31 + 0.05j])
def test_mvp_matches_dense_direct_sum(m):
    p = W.small_hex(m=m)
    fN, Toep, alpha, idx3, chi, dV = _setup(p)
    L, M, N = p["L"], p["M"], p["N"]
    A = O.dense_dda_matrix(p["r"], p["idx"], p["ko"], 1 / alpha, dV)
    A2 = O.dense_from_toeplitz(Toep, p["idx"], 1 / alpha, dV)
    assert np.abs(A - A2).max() <= 1e-12 * np.abs(A).max()
    rng = np.random.default_rng(1)
    x = rng.normal(size=len(idx3)) + 1j * rng.normal(size=len(idx3))
    y = O.MVP(x, fN, np.ones((L, M, N)), dV * chi, 1 / alpha, "notransp", idx3)
    yd = A @ x
    assert np.linalg.norm(y - yd) <= 1e-12 * np.linalg.norm(yd)
    # reference 'transp' branch is the conjugate transpose for real Gram
    yt = O.MVP(x, fN, np.ones((L, M, N)), dV * chi, 2.5, "transp", idx3)
    A_real_gram = O.dense_dda_matrix(p["r"], p["idx"], p["ko"], 2.5, dV)
    assert np.linalg.norm(yt - A_real_gram.conj().T @ x) <= 1e-12 * np.linalg.norm(yt)
    # plain transpose of a general (varying-Mc) operator
    mc = dV * (1 + 0.3 * rng.normal(size=(L, M, N)))
    ytt = MVP_plain_transpose(x, fN, np.ones((L, M, N)), mc, 1 / alpha, idx3)
    Amc = O.dense_dda_matrix(p["r"], p["idx"], p["ko"], 1 / alpha, mc)
    assert np.linalg.norm(ytt - Amc.T @ x) <= 1e-12 * np.linalg.norm(ytt)


def test_dda_tensor_symmetry_and_zero_planes():
    p = W.small_hex()
    _, Toep, _, _, _, _ = _setup(p)
    # odd components vanish exactly on their zero-offset planes (used by the
    # sign bookkeeping of the circulant levels)
    assert np.all(Toep[0, :, :, 1] == 0) and np.all(Toep[0, :, :, 2] == 0)
    assert np.all(Toep[:, 0, :, 1] == 0) and np.all(Toep[:, 0, :, 4] == 0)
    assert np.all(Toep[:, :, 0, 2] == 0) and np.all(Toep[:, :, 0, 4] == 0)
    assert np.all(Toep[0, 0, 0] == 0)


def test_alpha_ldr_limits():
    # kd -> 0 gives Clausius-Mossotti
    a = O.alpha_ldr(1.5, 1e-6, 1e-3, [0, 0, 1], [1, 0, 0])
    assert abs(a - 3 / (4 * math.pi) * (2.25 - 1) / (2.25 + 2)) < 1e-12
    eps = 2.0 + 0.1j
    h = 1e-6
    f = lambda e: 1 / O.alpha_ldr(e, 2.0, 0.1, [0, 0, 1], [1, 0, 0], is_eps=True)
    fd = (f(eps + h) - f(eps - h)) / (2 * h)
    assert abs(fd - O.dalpha_inv_deps(eps, 2.0, 0.1, [0, 0, 1], [1, 0, 0])) < 1e-6


def _wrapped_average(T, n, axis_block):
    """Frobenius-optimal circulant of each n x n Toeplitz sub-block."""
    out = np.zeros_like(T)
    i = np.arange(n)
    for k in range(n):
        mask = ((i[:, None] - i[None, :]) % n) == k
        avg = T[..., mask].mean(axis=-1)
        out[..., mask] = avg[..., None]
    return out


def test_circ_levels_match_dense_chan_approximation():
    p = W.small_hex(m=1.4, nper=3, diameter=1.5)
    fN, Toep, alpha, idx3, chi, dV = _setup(p)
    L, M, N = p["L"], p["M"], p["N"]
    allvox = np.arange(L * M * N)
    A = O.dense_from_toeplitz(Toep, allvox, 0.0, -1.0)  # = +G on the full grid
    n3 = 3 * L * M * N
    # index (x, y, z, c) with x fastest
    T = A.reshape(3, N, M, L, 3, N, M, L)  # [c,z,y,x, c',z',y',x']
    T = T.transpose(1, 2, 0, 5, 6, 4, 3, 7)  # [z,y,c,z',y',c',x,x']
    T1 = _wrapped_average(T, L, None)
    F = np.fft.fft(np.eye(L))
    # block for x-frequency i: F T1 F^-1 is diagonal in (x,x')
    D1 = np.einsum("ia,...ab,bj->...ij", F, T1, np.linalg.inv(F))
    lev1 = np.diagonal(D1, axis1=-2, axis2=-1)  # [z,y,c,z',y',c',i]
    lev1 = lev1.transpose(6, 0, 2, 3, 5, 1, 4)  # [i,z,c,z',c',y,y']
    T2 = _wrapped_average(lev1, M, None)
    Fm = np.fft.fft(np.eye(M))
    D2 = np.einsum("ja,...ab,bk->...jk", Fm, T2, np.linalg.inv(Fm))
    lev2 = np.diagonal(D2, axis1=-2, axis2=-1)  # [i,z,c,z',c',j]
    blocks_math = lev2.transpose(0, 5, 2, 1, 4, 3).reshape(L, M, 3 * N, 3 * N)  # (c,z) z fastest
    _, circL = O.circ_1_level(Toep, L, M, N, 0, "off")
    _, blocks = O.circ_2_level(circL, L, M, N)
    assert np.abs(blocks - blocks_math).max() <= 1e-10 * np.abs(blocks_math).max()


def test_prec_inverts_its_circulant():
    p = W.small_hex(m=1.4, nper=3, diameter=1.5)
    fN, Toep, alpha, idx3, chi, dV = _setup(p)
    L, M, N = p["L"], p["M"], p["N"]
    _, circL = O.circ_1_level(Toep, L, M, N, 0, "off")
    _, blocks = O.circ_2_level(circL, L, M, N)
    inv = O.invert_blocks(blocks, 1 / alpha, dV)
    # forward 2-level circulant operator applied through FFTs
    fwd = np.linalg.inv(inv)
    allidx = np.arange(3 * L * M * N)
    rng = np.random.default_rng(2)
    x = rng.normal(size=allidx.size) + 1j * rng.normal(size=allidx.size)
    y = O.mvp_circ_2_level(fwd, x, L, M, N, allidx)
    z = O.mvp_circ_2_level(inv, y, L, M, N, allidx)
    assert np.linalg.norm(z - x) <= 1e-11 * np.linalg.norm(x)


def test_circ_1_level_blocks_and_chan_apply():
    p = W.small_hex(m=1.4, nper=3, diameter=1.5)
    fN, Toep, alpha, idx3, chi, dV = _setup(p)
    L, M, N = p["L"], p["M"], p["N"]
    circ, circL = O.circ_1_level(Toep, L, M, N, 0, "on")
    assert circ.shape == (L, 3 * M * N, 3 * M * N)
    inv = np.linalg.inv((1 / alpha) * np.eye(3 * M * N)[None] - dV * circ)
    allidx = np.arange(3 * L * M * N)
    x = np.random.default_rng(3).normal(size=allidx.size) + 0j
    y = O.chan_mvp_idx(inv, x, L, M, N, allidx)
    z = O.chan_mvp_idx(np.linalg.inv(inv), y, L, M, N, allidx)
    assert np.linalg.norm(z - x) <= 1e-10 * np.linalg.norm(x)


@pytest.mark.parametrize("solver", ["bicgstab", "gmres", "pgmres", "pgmres_dr"])
@pytest.mark.parametrize("prec", [False, True])
def test_krylov_solves(solver, prec):
    p = W.small_hex(m=1.31 + 0.05j)
    fN, Toep, alpha, idx3, chi, dV = _setup(p)
    L, M, N = p["L"], p["M"], p["N"]
    A = lambda v: O.MVP(v, fN, np.ones((L, M, N)), dV * chi, 1 / alpha, "notransp", idx3)
    Einc = O.PlaneWavePointWise(p["Eo"], p["kvec"], p["r"])
    b = Einc.ravel(order="F")[idx3]
    Pm = None
    if prec:
        _, circL = O.circ_1_level(Toep, L, M, N, 0, "off")
        _, blocks = O.circ_2_level(circL, L, M, N)
        inv = O.invert_blocks(blocks, 1 / alpha, dV)
        Pm = lambda v: O.mvp_circ_2_level(inv, v, L, M, N, idx3)
    tol = 1e-8
    if solver == "bicgstab":
        x, flag, relres, it, resvec = O.bicgstab(A, b, tol, 500, Pm)
        assert len(resvec) == int(round(2 * it)) + 1
    elif solver == "gmres":
        x, flag, relres, it, resvec = O.gmres(A, b, 200, tol, 1, Pm)
    elif solver == "pgmres":
        x, flag, relres, it, resvec = O.pgmres(A, b, 200, tol, 2, Pm)
    else:  # restarts short enough that the recycled space is used
        x, flag, relres, it, resvec = O.pgmres_dr(A, b, 6, tol, 100, 3, R1=Pm)
        assert it[1] >= 2
    Ad = O.dense_dda_matrix(p["r"], p["idx"], p["ko"], 1 / alpha, dV)
    xd = np.linalg.solve(Ad, b)
    assert flag == 0
    assert np.linalg.norm(x - xd) <= 1e-6 * np.linalg.norm(xd)


def test_mie_known_answer():
    # Bohren & Huffman BHMIE sample case: radius 0.525, wavelength 0.6328, m=1.55
    x = 2 * math.pi * 0.525 / 0.6328
    assert abs(O.mie_qext(x, 1.55) - 3.10543) < 2e-5


def test_dda_sphere_cext_vs_mie():
    m = 1.31 + 0.01j
    sizeParam = 2.0
    r, idx, res, _, lam_ext, _ = geometry("sphere", m, sizeParam, 14)
    L, M, N, _ = r.shape
    ko = 2 * math.pi / lam_ext
    kvec = np.array([0, 0, ko]); Eo = np.array([1.0, 0, 0])
    fN, Toep, alpha = O.getOPERATOR_DDA(r, ko, m, kvec, Eo, "off")
    nD = L * M * N
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    chi = _grid_from_vox(L, M, N, idx, 1.0)
    dV = res ** 3
    A = lambda v: O.MVP(v, fN, np.ones((L, M, N)), dV * chi, 1 / alpha, "notransp", idx3)
    b = O.PlaneWavePointWise(Eo, kvec, r).ravel(order="F")[idx3]
    P, flag, *_ = O.bicgstab(A, b, 1e-8, 1000)
    assert flag == 0
    cext = O.cext_dda(P, b, ko, dV, Eo)
    a_eff = (3 * len(idx) * dV / (4 * math.pi)) ** (1 / 3)
    q = cext / (math.pi * a_eff ** 2)
    qmie = O.mie_qext(ko * a_eff, m)
    assert abs(q - qmie) / qmie < 0.05


def test_cext_gradient_central_differences():
    p = W.config4(L=5, M=4, N=3)
    L, M, N = p["L"], p["M"], p["N"]
    d, ko = p["d"], p["ko"]
    idx = p["idx"]
    nD = L * M * N
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    Toep = O.green_toeplitz(p["r"], ko)
    fN = O.fft_operator(O.circulant_nop_const(Toep))
    dV = d ** 3
    b = O.PlaneWavePointWise(p["Eo"], p["kvec"], p["r"]).ravel(order="F")[idx3]

    def solve(eps, rhs, transpose=False):
        ainv = 1 / O.alpha_ldr(eps, ko, d, p["kvec"], p["Eo"], is_eps=True)
        G = _grid_from_vox(L, M, N, idx, ainv)
        if transpose:
            A = lambda v: MVP_plain_transpose(v, fN, np.ones((L, M, N)), dV, G, idx3)
        else:
            A = lambda v: O.MVP(v, fN, np.ones((L, M, N)), dV, G, "notransp", idx3)
        x, flag, *_ = O.bicgstab(A, rhs, 1e-13, 2000)
        assert flag == 0
        return x

    eps = p["eps"]
    P = solve(eps, b)
    lam = solve(eps, np.conj(b), transpose=True)
    gre, gim = O.cext_grad_dda(P, lam, eps, ko, d, p["kvec"], p["Eo"])
    h = 1e-6
    rng = np.random.default_rng(0)
    for j in rng.choice(len(idx), 6, replace=False):
        for step, g in ((h, gre), (1j * h, gim)):
            ep = eps.copy(); ep[j] += step
            em = eps.copy(); em[j] -= step
            cp = O.cext_dda(solve(ep, b), b, ko, dV, p["Eo"])
            cm = O.cext_dda(solve(em, b), b, ko, dV, p["Eo"])
            fd = (cp - cm) / (2 * h)
            assert abs(fd - g[j]) <= 1e-5 * max(abs(g).max(), 1e-30)


def test_nop_cubature_matches_reference_source():
    """The face-pair cubature restatement against the reference's own
    cubature_nop_const.cpp compiled here (skipped where it cannot be
    compiled), 4x4, 10x10 and 20x20 rules."""
    from oracle import nop
    ref = nop.reference_cubature()
    if ref is None:
        pytest.skip("reference cubature source not available")
    ko, dx = 2 * np.pi * 0.7, 0.08
    Rf = nop.cube_faces(dx)
    for n in (4, 10, 20):
        W, U, V = nop.gauss_2d(n)
        for m in ([3, 2, 1], [0, 1, 1], [9, 0, 4], [2, 2, 2]):
            a = nop.cubature_nop(W, U, V, np.array(m) * dx, np.zeros(3), Rf, ko, dx)
            b = ref(W, U, V, np.array(m) * dx, np.zeros(3), Rf, ko, dx)
            assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max(), (n, m)


def test_nop_assembly_matches_golden():
    """N-operator Toeplitz tensor (far + medium cells) against the fixtures
    made with the reference's own cubature (tests/golden/make_nop_golden.py)."""
    from oracle import nop
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "nop_assembly.npz"))
    ko, dx = float(g["ko"]), float(g["dx"])
    Rf = nop.cube_faces(dx)
    for n in (4, 10, 20):
        W, U, V = nop.gauss_2d(n)
        for o, Jref in zip(g["J_offsets"], g[f"J_rule{n}"]):
            J = nop.cubature_nop(W, U, V, o * dx, np.zeros(3), Rf, ko, dx)
            assert np.abs(J - Jref).max() <= 1e-13 * np.abs(Jref).max(), (n, o)
    for name, shape in (("G_7x6x5", (7, 6, 5)), ("G_1x1x6", (1, 1, 6))):
        G = nop.assembly_nop(*shape, ko, dx)
        assert np.linalg.norm(G - g[name]) <= 1e-12 * np.linalg.norm(g[name]), name


def test_far_field_optical_theorem_identity():
    """The oracle's far-field amplitude in the incident direction reproduces the
    C_ext sum (Draine & Flatau 1994) for any polarisation: with E_inc = E0
    exp(i k.r) and E0 orthogonal to k, conj(E0).F(k_hat) = k^2 dV sum conj(E_inc).P."""
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.0, nper=3)
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx3 = np.concatenate([p["idx"], nD + p["idx"], 2 * nD + p["idx"]])
    rng = np.random.default_rng(2)
    P = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
    ko, dV = p["ko"], p["d"] ** 3
    E0 = np.asarray(p["Eo"], dtype=complex)
    Einc = O.PlaneWavePointWise(E0, p["kvec"], p["r"]).ravel(order="F")[idx3]
    F = O.far_field(P, idx3, p["r"], ko, dV, np.asarray(p["kvec"]) / ko)
    c_ot = 4 * np.pi / ko * np.imag(np.vdot(E0, F[0])) / np.sum(np.abs(E0) ** 2)
    c = O.cext_dda(P, Einc, ko, dV, E0)
    assert abs(c_ot - c) <= 1e-12 * abs(c)


def test_pgmres_dr_deflation_beats_restarted_gmres():
    """GCRO-DR (pgmresDR.m) on a matrix with a cluster of small eigenvalues:
    the recycled harmonic Ritz space removes them from later cycles, so it
    needs far fewer Arnoldi steps than plain restarted GMRES (pgmres.m) of the
    same restart length; both reach the tolerance."""
    rng = np.random.default_rng(2)
    n = 300
    ev = np.concatenate([np.linspace(0.01, 0.1, 8), 1 + rng.random(n - 8)]) * np.exp(1j * rng.random(n) * 0.3)
    X = np.eye(n) + 0.1 * rng.normal(size=(n, n)) / np.sqrt(n)
    A = X @ np.diag(ev) @ np.linalg.inv(X)
    b = rng.normal(size=n) + 1j * rng.normal(size=n)
    x1, f1, r1, it1, rv1 = O.pgmres_dr(A, b, 20, 1e-10, 100, 10)
    x2, f2, r2, it2, rv2 = O.pgmres(A, b, 20, 1e-10, 100)
    assert f1 == 0 and f2 == 0
    assert np.linalg.norm(A @ x1 - b) <= 1e-10 * np.linalg.norm(b)
    assert len(rv1) < 0.5 * len(rv2)
    # resvec: one entry per Arnoldi step after the initial 1
    assert rv1[0] == 1.0 and len(rv1) == 1 + 20 * (it1[1]) + it1[0]


def test_inverse_blocks_times_component_flips_are_symmetric():
    """Every inverse block B of the 2-level circulant preconditioner of the DDA
    operator satisfies (B D)^T = B D with D = diag(-1 on the x and y
    components, +1 on z): the property that lets the packed GEMV store only
    the lower triangle of B D.  A face vector d (JVIE) breaks it."""
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    fN, Toep, alpha, idx3, chi, dV = _setup(p)
    L, M, N = p["L"], p["M"], p["N"]
    _, c1 = O.circ_1_level(Toep, L, M, N, 0, "off")
    _, blk = O.circ_2_level(c1, L, M, N)
    D = np.r_[-np.ones(2 * N), np.ones(N)]
    inv = O.invert_blocks(blk, 1 / alpha, dV)
    worst = max(np.linalg.norm(S - S.T) / np.linalg.norm(S) for S in (inv[i, j] * D for i in range(L) for j in range(M)))
    assert worst < 1e-13
    face = 1 + 0.3 * np.random.default_rng(0).random(3 * N)
    inv_f = O.invert_blocks(blk, 0.8, face)
    worst_f = max(np.linalg.norm(S - S.T) / np.linalg.norm(S) for S in (inv_f[i, j] * D for i in range(L) for j in range(M)))
    assert worst_f > 1e-3


def test_unpolarised_cext_and_the_polarisation_basis():
    """The two-polarisation average of C_ext used by the orientation averaging:
    with a polarisation-independent polarisability it is the trace of a
    quadratic form, the same for any orthonormal pair perpendicular to k; with
    the LDR polarisability (its S term depends on the polarisation,
    getOPERATOR_DDA.m:14-26) it is not, which is why an orientation average
    samples the angle of the pair about k as well (dense solves)."""
    p = W.small_hex(m=1.31 + 0.05j, diameter=1.5, nper=4)
    L, M, N = p["L"], p["M"], p["N"]
    idx = p["idx"]
    nD = L * M * N
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    ko, d = p["ko"], p["d"]
    k = np.array([0.3, -0.5, 0.81]); k /= np.linalg.norm(k)
    e1, e2 = O.polarisation_basis(k)
    assert abs(e1 @ k) < 1e-12 and abs(e2 @ k) < 1e-12 and abs(e1 @ e2) < 1e-12

    def cext(e, ldr):
        # without LDR dependence: alpha of a fixed S (that of e1)
        ainv = 1 / O.alpha_ldr(p["refInd"], ko, d, ko * k, e if ldr else e1)
        A = O.dense_dda_matrix(p["r"], idx, ko, ainv, d ** 3)
        b = O.PlaneWavePointWise(e, ko * k, p["r"]).ravel(order="F")[idx3]
        return O.cext_dda(np.linalg.solve(A, b), b, ko, d ** 3, e)

    t = 0.7
    f1, f2 = np.cos(t) * e1 + np.sin(t) * e2, -np.sin(t) * e1 + np.cos(t) * e2
    base = 0.5 * (cext(e1, False) + cext(e2, False))
    assert abs(0.5 * (cext(f1, False) + cext(f2, False)) - base) < 1e-9 * abs(base)
    base_ldr = 0.5 * (cext(e1, True) + cext(e2, True))
    assert abs(0.5 * (cext(f1, True) + cext(f2, True)) - base_ldr) > 1e-5 * abs(base_ldr)
    # the oracle's orientation average honours psi
    solve = lambda kv, e: np.linalg.solve(
        O.dense_dda_matrix(p["r"], idx, ko, 1 / O.alpha_ldr(p["refInd"], ko, d, kv, e), d ** 3),
        O.PlaneWavePointWise(e, kv, p["r"]).ravel(order="F")[idx3])
    einc = lambda kv, e: O.PlaneWavePointWise(e, kv, p["r"]).ravel(order="F")[idx3]
    avg, each = O.orientation_average_cext(solve, einc, ko, d ** 3, [k], psi=[t])
    assert abs(avg - 0.5 * (cext(f1, True) + cext(f2, True))) < 1e-12 * abs(avg)
