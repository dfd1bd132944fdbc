"""GPU plane-wave excitation, extinction cross section and its adjoint
gradient (d C_ext / d eps per voxel) against the FP64 oracle and central
differences (h = 1e-6).  Tolerances: plane wave and C_ext <= 1e-12 relative;
FP64-mode gradients <= 1e-7 relative (max norm) against the oracle gradient;
central differences <= 1e-3 relative to max|grad| (the perturbed solves stop
at a 1e-12 residual, and C_ext round-off of that order divided by 2h bounds
what a difference quotient resolves); the mixed-precision gradient <= 1e-3
relative to the FP64 one."""
import numpy as np
import pytest

import oracle as O
from oracle.mvp import MVP_plain_transpose
from voxscatter_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from voxscatter_gb300 import build
    build.build()
    from voxscatter_gb300 import api as A
    return A


def _slab(api, L=6, M=5, N=3, seed=0):
    p = W.config4(seed=seed, L=L, M=M, N=N)
    idx = p["idx"]
    nD = L * M * N
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    d, ko = p["d"], p["ko"]
    Toep = api.green_dda(p["r"], ko)
    ainv = 1 / api.alpha_ldr(p["eps"], ko, d, p["kvec"], p["Eo"], is_eps=True)
    G = np.zeros(nD, complex); G[idx] = ainv
    op = api.Operator(L, M, N, idx3, 1.0, d ** 3, G.reshape((L, M, N), order="F"), toep=Toep)
    pr = api.Preconditioner(op, shift=np.mean(ainv), d=d ** 3)
    return p, idx3, op, pr, Toep


def test_plane_wave_and_cext(api):
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx3 = np.concatenate([p["idx"], nD + p["idx"], 2 * nD + p["idx"]])
    Toep = O.green_toeplitz(p["r"], p["ko"])
    op = api.Operator(L, M, N, idx3, 1.0, p["d"] ** 3, 2.0, toep=Toep)
    E0 = np.array([0.3 + 0.1j, 1.0, -0.2j])
    kvec = p["ko"] * np.array([0.6, 0.0, 0.8])
    b = api.plane_wave(op, p["r"], kvec, E0)
    b_o = O.PlaneWavePointWise(E0, kvec, p["r"]).ravel(order="F")[idx3]
    assert np.abs(b - b_o).max() <= 1e-13
    P = np.random.default_rng(3).normal(size=idx3.size) + 1j * np.random.default_rng(4).normal(size=idx3.size)
    c = api.cext(op, P, b_o, p["ko"], p["d"] ** 3, E0)
    c_o = O.cext_dda(P, b_o, p["ko"], p["d"] ** 3, E0)
    assert abs(c - c_o) <= 1e-12 * abs(c_o)


def test_gradient_matches_oracle_adjoint(api):
    p, idx3, op, pr, Toep = _slab(api)
    L, M, N = p["L"], p["M"], p["N"]
    d, ko = p["d"], p["ko"]
    b = api.plane_wave(op, p["r"], p["kvec"], p["Eo"])
    c, gre, gim, P, i1, i2 = api.cext_grad(op, pr, b, p["eps"], ko, d, p["kvec"], p["Eo"], tol=1e-12,
                                           precision="fp64")
    assert i1["flag"] == 0 and i2["flag"] == 0
    # oracle: FP64 forward and adjoint solves
    fN = O.fft_operator(O.circulant_nop_const(Toep))
    ainv = 1 / O.alpha_ldr(p["eps"], ko, d, p["kvec"], p["Eo"], is_eps=True)
    nD = L * M * N
    G = np.zeros(nD, complex); G[p["idx"]] = ainv
    G = G.reshape((L, M, N), order="F")
    A = lambda v: O.MVP(v, fN, np.ones((L, M, N)), d ** 3, G, "notransp", idx3)
    At = lambda v: MVP_plain_transpose(v, fN, np.ones((L, M, N)), d ** 3, G, idx3)
    Po, f1, *_ = O.bicgstab(A, b, 1e-13, 3000)
    lo, f2, *_ = O.bicgstab(At, np.conj(b), 1e-13, 3000)
    gre_o, gim_o = O.cext_grad_dda(Po, lo, p["eps"], ko, d, p["kvec"], p["Eo"])
    c_o = O.cext_dda(Po, b, ko, d ** 3, p["Eo"])
    assert abs(c - c_o) <= 1e-9 * abs(c_o)
    sc = max(np.abs(gre_o).max(), np.abs(gim_o).max())
    assert np.abs(gre - gre_o).max() <= 1e-7 * sc
    assert np.abs(gim - gim_o).max() <= 1e-7 * sc


def test_slab_64x64x16_gradient_central_differences(api):
    """The 64x64x16 random-permittivity slab: adjoint gradient (FP64 mode) vs
    central differences h = 1e-6 on 16 seeded voxels (real and imaginary
    parts), and the mixed-precision gradient vs the FP64 one."""
    p, idx3, op, pr, Toep = _slab(api, 64, 64, 16)
    d, ko = p["d"], p["ko"]
    b = api.plane_wave(op, p["r"], p["kvec"], p["Eo"])
    c, gre, gim, P, i1, i2 = api.cext_grad(op, pr, b, p["eps"], ko, d, p["kvec"], p["Eo"], tol=1e-12,
                                           precision="fp64")
    cm, grem, gimm, Pm, j1, j2 = api.cext_grad(op, pr, b, p["eps"], ko, d, p["kvec"], p["Eo"], tol=1e-6,
                                               precision="mixed")
    assert i1["flag"] == 0 and i2["flag"] == 0 and j1["flag"] == 0 and j2["flag"] == 0
    sc = max(np.abs(gre).max(), np.abs(gim).max())
    assert np.abs(grem - gre).max() <= 1e-3 * sc
    assert np.abs(gimm - gim).max() <= 1e-3 * sc
    assert abs(cm - c) <= 1e-5 * abs(c)
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N

    def cext_of(eps):
        ainv = 1 / api.alpha_ldr(eps, ko, d, p["kvec"], p["Eo"], is_eps=True)
        G = np.zeros(nD, complex); G[p["idx"]] = ainv
        o2 = api.Operator(L, M, N, idx3, 1.0, d ** 3, G.reshape((L, M, N), order="F"), toep=Toep)
        x, info, _ = api.solve(o2, b, pr, tol=1e-12, precision="fp64", x0=P, want_resvec=False)
        assert info["flag"] == 0, info
        return api.cext(o2, x, b, ko, d ** 3, p["Eo"])

    h = 1e-6
    rng = np.random.default_rng(1234)
    worst = 0.0
    for j in rng.choice(len(p["idx"]), 16, replace=False):
        for step, g in ((h, gre), (1j * h, gim)):
            ep = p["eps"].copy(); ep[j] += step
            em = p["eps"].copy(); em[j] -= step
            fd = (cext_of(ep) - cext_of(em)) / (2 * h)
            worst = max(worst, abs(fd - g[j]) / sc)
            assert abs(fd - g[j]) <= 1e-3 * sc, (j, step, fd, g[j], sc)
    print(f"central differences: worst |fd - adjoint| / max|grad| = {worst:.2e}")


def _hex_op(api, m=1.31 + 0.05j):
    p = W.small_hex(m=m, diameter=2.5, nper=4)
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx3 = np.concatenate([p["idx"], nD + p["idx"], 2 * nD + p["idx"]])
    fN, Toep, alpha = O.getOPERATOR_DDA(p["r"], p["ko"], p["refInd"], p["kvec"], p["Eo"])
    dV = p["d"] ** 3
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    return p, idx3, fN, Toep, alpha, op


def test_whole_domain_field_matches_oracle(api):
    """main_DDA.m:136-148 (total field over the grid) and the mv_L_const.m form
    of the whole-domain apply, c128 <= 1e-12 and c64 <= 2e-6 relative."""
    p, idx3, fN, Toep, alpha, op = _hex_op(api)
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    dV = p["d"] ** 3
    rng = np.random.default_rng(11)
    P = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
    Einc = O.PlaneWavePointWise(p["Eo"], p["kvec"], p["r"]).ravel(order="F")
    chi = (p["refInd"] ** 2 - 1) / (4 * np.pi)
    E_o = O.field_dda(P, idx3, Einc, fN, alpha, dV, chi, L, M, N)
    for prec, tol in (("c128", 1e-12), ("c64", 2e-6)):
        E = api.field_dda(op, P, Einc, alpha, dV, chi, precision=prec)
        assert np.linalg.norm(E - E_o) <= tol * np.linalg.norm(E_o), prec
    # two right-hand sides in one call
    P2 = np.stack([P, 1j * P[::-1]])
    E2 = api.field_dda(op, P2, np.stack([Einc, Einc]), alpha, dV, chi)
    E2_o = O.field_dda(P2[1], idx3, Einc, fN, alpha, dV, chi, L, M, N)
    assert np.linalg.norm(E2[0] - E_o) <= 1e-12 * np.linalg.norm(E_o)
    assert np.linalg.norm(E2[1] - E2_o) <= 1e-12 * np.linalg.norm(E2_o)
    # JOut = crop(fN * J) - Gram J over the whole domain (a = -Gram, b = 1)
    gram = 0.7 - 0.2j
    J = rng.normal(size=3 * nD) + 1j * rng.normal(size=3 * nD)
    Y_o = O.MVP(J, fN, np.ones((L, M, N)), -1.0, -gram, "notransp", np.arange(3 * nD))
    for prec, tol in (("c128", 1e-12), ("c64", 2e-6)):
        Y = api.apply_domain(op, J, -gram, 1.0, precision=prec)
        assert np.linalg.norm(Y - Y_o) <= tol * np.linalg.norm(Y_o), prec


def test_far_field_and_optical_theorem(api):
    """F(n) against the direct sum (<= 1e-12 relative) and the optical theorem:
    4 pi / ko Im(conj(E0).F(k_inc)) / |E0|^2 equals the C_ext sum for any P
    (E0 orthogonal to k_inc), here on the solved polarisation."""
    p, idx3, fN, Toep, alpha, op = _hex_op(api)
    dV = p["d"] ** 3
    ko = p["ko"]
    rng = np.random.default_rng(12)
    dirs = rng.normal(size=(7, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    khat = np.asarray(p["kvec"]) / ko
    dirs = np.vstack([khat, dirs])
    Einc = api.plane_wave(op, p["r"], p["kvec"], p["Eo"])
    P, info, _ = api.solve(op, Einc, tol=1e-10, precision="fp64")
    F = api.far_field(op, P, p["r"], ko, dV, dirs)
    F_o = O.far_field(P, idx3, p["r"], ko, dV, dirs)
    assert np.linalg.norm(F - F_o) <= 1e-12 * np.linalg.norm(F_o)
    E0 = np.asarray(p["Eo"], dtype=complex)
    c_ot = 4 * np.pi / ko * np.imag(np.vdot(E0, F[0])) / np.sum(np.abs(E0) ** 2)
    c_sum = api.cext(op, P, Einc, ko, dV, p["Eo"])
    assert abs(c_ot - c_sum) <= 1e-11 * abs(c_sum)
    # transversality and two right-hand sides
    assert np.abs(np.einsum("dc,dc->d", F, dirs)).max() <= 1e-12 * np.abs(F).max()
    F2 = api.far_field(op, np.stack([P, 2 * P]), p["r"], ko, dV, dirs)
    assert np.linalg.norm(F2[1] - 2 * F) <= 1e-13 * np.linalg.norm(F)


def _orientation_oracle(p, idx3, m_vox, dirs, weights, psi):
    """Dense direct solve per (direction, polarisation), each with its own
    alpha_LDR (per voxel when m varies)."""
    L, M, N = p["L"], p["M"], p["N"]
    ko, d = p["ko"], p["d"]
    idx = p["idx"]

    def solve(kvec, e):
        ainv = 1 / O.alpha_ldr(m_vox, ko, d, kvec, e)
        G = np.ones(L * M * N, complex); G[idx] = ainv
        A = O.dense_dda_matrix(p["r"], idx, ko, G.reshape((L, M, N), order="F"), d ** 3)
        return np.linalg.solve(A, O.PlaneWavePointWise(e, kvec, p["r"]).ravel(order="F")[idx3])

    einc = lambda kvec, e: O.PlaneWavePointWise(e, kvec, p["r"]).ravel(order="F")[idx3]
    return O.orientation_average_cext(solve, einc, ko, d ** 3, dirs, weights, psi)


@pytest.mark.parametrize("precision,tol,ctol", [("mixed", 1e-6, 2e-5), ("fp64", 1e-11, 1e-9)])
@pytest.mark.parametrize("per_voxel", [False, True])
def test_orientation_average_matches_oracle(api, precision, tol, ctol, per_voxel):
    """Random-orientation averaging (README.md:37): 10 weighted orientations
    (incident direction and polarisation-pair angle psi; one direction along
    z, where the basis switches to k x x), two polarisations each, every
    incidence with its own alpha_LDR; the
    per-(direction, polarisation) C_ext and the weighted average against dense
    direct solves of the oracle.  Directions split over two batched solves (8 + 2)."""
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.0, nper=4)
    L, M, N = p["L"], p["M"], p["N"]
    idx = p["idx"]
    nD = L * M * N
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    ko, d = p["ko"], p["d"]
    rng = np.random.default_rng(17)
    m_vox = p["refInd"] * (1 + (0.05 * rng.random(len(idx)) if per_voxel else 0.0))
    a0 = O.alpha_ldr(m_vox, ko, d, p["kvec"], p["Eo"])
    G0 = np.ones(nD, complex); G0[idx] = 1 / a0
    op = api.Operator(L, M, N, idx3, 1.0, d ** 3, G0.reshape((L, M, N), order="F"),
                      toep=O.green_toeplitz(p["r"], ko))
    pr = api.Preconditioner(op, shift=np.mean(1 / a0), d=d ** 3)
    dirs = rng.normal(size=(10, 3))
    dirs[3] = [0, 0, -2.0]
    weights = rng.random(10) + 0.5
    psi = rng.random(10) * np.pi
    avg, each, infos = api.orientation_average(op, pr, m_vox if per_voxel else p["refInd"], p["r"], ko, d, dirs,
                                               weights, psi, tol=tol, precision=precision)
    assert all(i["flag"] == 0 for i in infos)
    avg_o, each_o = _orientation_oracle(p, idx3, m_vox, dirs, weights, psi)
    assert np.max(np.abs(each - each_o) / np.abs(each_o)) < ctol
    assert abs(avg - avg_o) / abs(avg_o) < ctol
    # the two polarisations really differ for an oblique incidence on the plate
    assert np.max(np.abs(each[:, 0] - each[:, 1]) / np.abs(each[:, 0])) > 1e-3
