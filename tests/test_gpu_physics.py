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
