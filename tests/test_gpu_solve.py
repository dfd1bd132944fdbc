"""GPU Krylov solves (BiCGSTAB, mixed c64 + FP64 refinement and plain FP64)
against dense FP64 direct solves of the oracle operator.  Every solution is
also re-checked with the oracle's FP64 MVP: ||b - A x||/||b|| <= tol."""
import numpy as np
import pytest

import oracle as O
from voxscatter_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from voxscatter_gb300 import build
    build.build()
    from voxscatter_gb300 import api as A
    return A


def _system(p):
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx = p["idx"]
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    Toep = O.green_toeplitz(p["r"], p["ko"])
    alpha = O.alpha_ldr(p["refInd"], p["ko"], p["d"], p["kvec"], p["Eo"])
    dV = p["d"] ** 3
    chi = np.zeros(nD); chi[idx] = 1
    chi = chi.reshape((L, M, N), order="F")
    fN = O.fft_operator(O.circulant_nop_const(Toep))
    b = O.PlaneWavePointWise(p["Eo"], p["kvec"], p["r"]).ravel(order="F")[idx3]
    Aor = lambda v: O.MVP(v, fN, np.ones((L, M, N)), dV * chi, 1 / alpha, "notransp", idx3)
    return L, M, N, idx3, Toep, alpha, dV, b, Aor


@pytest.mark.parametrize("precision,tol", [("mixed", 1e-6), ("fp64", 1e-10)])
@pytest.mark.parametrize("use_prec", [False, True])
def test_bicgstab_small(api, precision, tol, use_prec):
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N, idx3, Toep, alpha, dV, b, Aor = _system(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV) if use_prec else None
    x, flag, relres, it, resvec = api.bicgstab(op, b, tol, 500, pr, precision=precision)
    assert flag == 0, (flag, relres, it)
    true_rel = np.linalg.norm(b - Aor(x)) / np.linalg.norm(b)
    assert true_rel <= tol * 1.01
    assert abs(true_rel - relres) <= 0.05 * max(true_rel, relres) + 1e-15
    Ad = O.dense_dda_matrix(p["r"], p["idx"], p["ko"], 1 / alpha, dV)
    xd = np.linalg.solve(Ad, b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 100 * tol
    assert len(resvec) >= 2 and resvec[0] > 0
    if precision == "fp64":
        assert len(resvec) == int(round(2 * it)) + 1


def test_bicgstab_iteration_count_matches_oracle(api):
    """FP64 device BiCGSTAB follows the oracle's recurrences: same iteration count."""
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N, idx3, Toep, alpha, dV, b, Aor = _system(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    _, circL = O.circ_1_level(Toep, L, M, N, 0, "off")
    _, blk = O.circ_2_level(circL, L, M, N)
    inv = O.invert_blocks(blk, 1 / alpha, dV)
    Pm = lambda v: O.mvp_circ_2_level(inv, v, L, M, N, idx3)
    xo, fo, ro, ito, rvo = O.bicgstab(Aor, b, 1e-8, 500, Pm)
    x, flag, relres, it, rv = api.bicgstab(op, b, 1e-8, 500, pr, precision="fp64")
    assert flag == fo == 0
    assert it == ito
    n = min(len(rv), len(rvo))
    assert np.allclose(rv[:n], rvo[:n], rtol=1e-6, atol=1e-12 * rvo[0])


def test_bicgstab_flags(api):
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N, idx3, Toep, alpha, dV, b, Aor = _system(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    x, flag, relres, it, rv = api.bicgstab(op, b, 1e-12, 2, None, precision="fp64")
    assert flag == 1 and it <= 2
    from voxscatter_gb300 import _lib
    bad = b.copy(); bad[3] = np.nan
    with pytest.raises(_lib.VoxScatterError) as e:
        api.bicgstab(op, bad, 1e-6, 10, None)
    assert e.value.status == _lib.VS_ERR_NONFINITE
    x, flag, relres, it, rv = api.bicgstab(op, np.zeros_like(b), 1e-6, 10, None)
    assert flag == 0 and np.all(x == 0)


def test_config1_mixed_and_fp64_agree(api):
    """Hex plate 27x23x7 with the 2-level preconditioner, tol 1e-6 (the
    reference's CPU configuration uses 1e-5): mixed and FP64 solutions agree with
    the dense solve."""
    p = W.config1()
    L, M, N, idx3, Toep, alpha, dV, b, Aor = _system(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    xm, im, rvm = api.solve(op, b, pr, tol=1e-6, precision="mixed")
    xf, iff, rvf = api.solve(op, b, pr, tol=1e-6, precision="fp64")
    assert im["flag"] == 0 and iff["flag"] == 0
    for x in (xm, xf):
        assert np.linalg.norm(b - Aor(x)) / np.linalg.norm(b) <= 1e-6 * 1.01
    assert np.linalg.norm(xm - xf) / np.linalg.norm(xf) < 1e-4


@pytest.mark.parametrize("precision,tol", [("mixed", 1e-6), ("fp64", 1e-10)])
@pytest.mark.parametrize("use_prec", [False, True])
@pytest.mark.parametrize("restart", [5, 60])
def test_gmres_small(api, precision, tol, use_prec, restart):
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N, idx3, Toep, alpha, dV, b, Aor = _system(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV) if use_prec else None
    x, flag, relres, it, resvec = api.gmres(op, b, restart, tol, 400, pr, precision=precision)
    assert flag == 0, (flag, relres, it)
    assert np.linalg.norm(b - Aor(x)) / np.linalg.norm(b) <= tol * 1.01
    Ad = O.dense_dda_matrix(p["r"], p["idx"], p["ko"], 1 / alpha, dV)
    xd = np.linalg.solve(Ad, b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 100 * tol
    assert len(resvec) >= 2


def test_gmres_matches_oracle_gmres_steps(api):
    """FP64 device GMRES(restart large) needs the same number of Arnoldi steps
    as the oracle's left-preconditioned GMRES to reach a preconditioned
    residual below tol (both follow the same Krylov space)."""
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N, idx3, Toep, alpha, dV, b, Aor = _system(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    _, circL = O.circ_1_level(Toep, L, M, N, 0, "off")
    _, blk = O.circ_2_level(circL, L, M, N)
    inv = O.invert_blocks(blk, 1 / alpha, dV)
    Pm = lambda v: O.mvp_circ_2_level(inv, v, L, M, N, idx3)
    xo, fo, ro, ito, rvo = O.gmres(Aor, b, 200, 1e-9, 1, Pm)
    x, info, rv = api.solve(op, b, pr, tol=1e-30, maxit=ito[1], precision="fp64", method="gmres", restart=200,
                            inner_tol=1e-9, max_refine=1)
    assert fo == 0
    assert info["iter"] == ito[1]
    n = min(len(rv), len(rvo))
    assert np.allclose(rv[:n] / rv[0], rvo[:n] / rvo[0], rtol=1e-6, atol=1e-12)


def test_config1_gmres_mixed(api):
    p = W.config1()
    L, M, N, idx3, Toep, alpha, dV, b, Aor = _system(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    x, info, rv = api.solve(op, b, pr, tol=1e-6, precision="mixed", method="gmres", restart=50)
    assert info["flag"] == 0
    assert np.linalg.norm(b - Aor(x)) / np.linalg.norm(b) <= 1e-6 * 1.01


def _directions(p, n, seed):
    """n random incident directions x 2 polarisations (as the batched
    configuration draws them): (kvec, pol) pairs."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        v = rng.normal(size=3); v /= np.linalg.norm(v)
        a = np.cross(v, [0, 0, 1.0]); a /= np.linalg.norm(a)
        for pol in (a, np.cross(v, a)):
            out.append((p["ko"] * v, pol))
    return out


@pytest.mark.parametrize("precision,tol", [("mixed", 1e-6), ("fp64", 1e-10)])
def test_batched_rhs_match_single_solves(api, precision, tol):
    """8 incident directions x 2 polarisations of one plate solved as one batch,
    each right-hand side with its own alpha_LDR (getOPERATOR_DDA.m:14-26 takes
    kvec and Eo, so Gram = 1/alpha differs per direction and polarisation,
    main_DDA.m:61-62,75).  Every solution meets tol against the oracle
    operator built with its own alpha, matches a dense direct solve of that
    operator, and the FP64 batch reproduces the single-rhs solves."""
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N, idx3, Toep, alpha, dV, b0, Aor = _system(p)
    fN = O.fft_operator(O.circulant_nop_const(Toep))
    chi = np.zeros(L * M * N); chi[p["idx"]] = 1
    chi = chi.reshape((L, M, N), order="F")
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)   # built for the +z, x-pol alpha
    pairs = _directions(p, 8, 5)
    B = np.array([O.PlaneWavePointWise(pol, kv, p["r"]).ravel(order="F")[idx3] for kv, pol in pairs])
    alphas = np.array([O.alpha_ldr(p["refInd"], p["ko"], p["d"], kv, pol) for kv, pol in pairs])
    # the oblique directions do change the diagonal
    assert np.max(np.abs(alphas / alpha - 1)) > 1e-3
    X, infos = api.solve_batch(op, B, pr, tol=tol, precision=precision, gram=1 / alphas)
    for k in range(len(B)):
        assert infos[k]["flag"] == 0, infos[k]
        Ak = lambda v: O.MVP(v, fN, np.ones((L, M, N)), dV * chi, 1 / alphas[k], "notransp", idx3)
        assert np.linalg.norm(B[k] - Ak(X[k])) / np.linalg.norm(B[k]) <= tol * 1.01
        # against the system with the +z alpha the residual is far larger
        if abs(alphas[k] / alpha - 1) > 1e-3:
            assert np.linalg.norm(B[k] - Aor(X[k])) / np.linalg.norm(B[k]) > 10 * tol
    for k in (0, 5, 11):
        Ad = O.dense_dda_matrix(p["r"], p["idx"], p["ko"], 1 / alphas[k], dV)
        xd = np.linalg.solve(Ad, B[k])
        assert np.linalg.norm(X[k] - xd) / np.linalg.norm(xd) < 100 * tol
        if precision == "fp64":
            x1, i1, _ = api.solve(op, B[k], pr, tol=tol, precision="fp64", gram=1 / alphas[k])
            assert i1["iter"] == infos[k]["iter"]
            assert np.linalg.norm(x1 - X[k]) <= 1e-12 * np.linalg.norm(x1)


def test_gmres_batch_with_gram_per_rhs(api):
    """GMRES solves a batch one right-hand side after another, each with its own Gram."""
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.0, nper=4)
    L, M, N, idx3, Toep, alpha, dV, b0, Aor = _system(p)
    fN = O.fft_operator(O.circulant_nop_const(Toep))
    chi = np.zeros(L * M * N); chi[p["idx"]] = 1
    chi = chi.reshape((L, M, N), order="F")
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pairs = _directions(p, 2, 9)
    B = np.array([O.PlaneWavePointWise(pol, kv, p["r"]).ravel(order="F")[idx3] for kv, pol in pairs])
    alphas = np.array([O.alpha_ldr(p["refInd"], p["ko"], p["d"], kv, pol) for kv, pol in pairs])
    X, infos = api.solve_batch(op, B, None, tol=1e-8, precision="fp64", method="gmres", restart=30, gram=1 / alphas)
    for k in range(len(B)):
        assert infos[k]["flag"] == 0
        Ak = lambda v: O.MVP(v, fN, np.ones((L, M, N)), dV * chi, 1 / alphas[k], "notransp", idx3)
        assert np.linalg.norm(B[k] - Ak(X[k])) / np.linalg.norm(B[k]) <= 1e-8 * 1.01


def _prec_oracle(p, Toep, alpha, dV, idx3):
    L, M, N = p["L"], p["M"], p["N"]
    _, circL = O.circ_1_level(Toep, L, M, N, 0, "off")
    _, blk = O.circ_2_level(circL, L, M, N)
    inv = O.invert_blocks(blk, 1 / alpha, dV)
    return lambda v: O.mvp_circ_2_level(inv, v, L, M, N, idx3)


@pytest.mark.parametrize("use_prec", [False, True])
def test_gmres_dr_matches_oracle_history(api, use_prec):
    """FP64 device GCRO-DR (restart 5, 2 recycled vectors, right
    preconditioned) follows the oracle's pgmresDR.m restatement over several
    cycles: the same Arnoldi residual estimates step by step, so the same
    harmonic Ritz spaces were recycled."""
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N, idx3, Toep, alpha, dV, b, Aor = _system(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV) if use_prec else None
    Pm = _prec_oracle(p, Toep, alpha, dV, idx3) if use_prec else None
    restart, ritz, cycles = 5, 2, 4
    xo, fo, ro, ito, rvo = O.pgmres_dr(Aor, b, restart, 1e-14, cycles - 1, ritz, R1=Pm)
    assert len(rvo) == 1 + restart * cycles          # ran all cycles
    x, info, rv = api.solve(op, b, pr, tol=1e-30, maxit=restart * cycles, precision="fp64", method="gmres_dr",
                            restart=restart, ritz=ritz, inner_tol=1e-30, max_refine=1)
    assert info["iter"] == restart * cycles
    assert len(rv) == len(rvo)
    assert np.allclose(rv, rvo, rtol=1e-6, atol=1e-13), np.max(np.abs(rv - rvo) / np.abs(rvo))
    # the same iterate after the same cycles
    assert np.linalg.norm(x - xo) <= 1e-8 * np.linalg.norm(xo)


@pytest.mark.parametrize("precision,tol", [("mixed", 1e-6), ("fp64", 1e-10)])
@pytest.mark.parametrize("use_prec", [False, True])
def test_gmres_dr_solves(api, precision, tol, use_prec):
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N, idx3, Toep, alpha, dV, b, Aor = _system(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV) if use_prec else None
    x, flag, relres, it, resvec = api.pgmresDR(op, b, 8, tol, 100, 3, R1=pr, precision=precision)
    assert flag == 0, (flag, relres, it)
    assert relres <= tol
    assert np.linalg.norm(b - Aor(x)) / np.linalg.norm(b) <= tol * 1.01
    Ad = O.dense_dda_matrix(p["r"], p["idx"], p["ko"], 1 / alpha, dV)
    xd = np.linalg.solve(Ad, b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 100 * tol
    assert resvec[0] == pytest.approx(1.0) and len(resvec) >= 2


def test_config1_gmres_dr_mixed(api):
    p = W.config1()
    L, M, N, idx3, Toep, alpha, dV, b, Aor = _system(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    x, info, rv = api.solve(op, b, pr, tol=1e-6, precision="mixed", method="gmres_dr", restart=20, ritz=5)
    assert info["flag"] == 0
    assert np.linalg.norm(b - Aor(x)) / np.linalg.norm(b) <= 1e-6 * 1.01


def test_particles_solved_concurrently_match_batch_solves(api):
    """vs_solve_particles_device: three plates of different sizes, two of them
    on one context and one on another (so two host threads run at once), 4
    rhs each; every particle's FP64 solutions and iteration counts equal those
    of its own vs_solve_batch_device call."""
    import torch
    ctxs = [api.Context(0), api.Context(0)]
    parts = []
    for k, (diam, ctx) in enumerate(((2.5, ctxs[0]), (2.0, ctxs[1]), (3.0, ctxs[0]))):
        p = W.small_hex(m=1.31 + 0.05j, diameter=diam, nper=4)
        L, M, N, idx3, Toep, alpha, dV, b0, Aor = _system(p)
        op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep, ctx=ctx)
        pr = api.Preconditioner(op, shift=1 / alpha, d=dV, precisions=("c64", "c128"))
        rng = np.random.default_rng(k)
        B = np.array([b0 * np.exp(1j * rng.random()) + 0.1 * (rng.normal(size=b0.size) + 0j) for _ in range(4)])
        parts.append((op, pr, torch.from_numpy(B).cuda(), Aor, B))
    ref = []
    for op, pr, Bd, _, B in parts:
        X = torch.zeros_like(Bd)
        torch.cuda.synchronize()
        ref.append((X, api.solve_batch_device(op, Bd.data_ptr(), X.data_ptr(), len(B), pr, tol=1e-10,
                                              precision="fp64")))
    Xs = [torch.zeros_like(Bd) for (_, _, Bd, _, _) in parts]
    torch.cuda.synchronize()
    out = api.solve_particles_device([q[0] for q in parts], [q[1] for q in parts], [q[2].data_ptr() for q in parts],
                                     [X.data_ptr() for X in Xs], [len(q[4]) for q in parts], tol=1e-10,
                                     precision="fp64")
    assert len(out) == 3
    for (op, pr, Bd, Aor, B), X, (Xr, ir), inf in zip(parts, Xs, ref, out):
        Xh = X.cpu().numpy()
        for r in range(len(B)):
            assert inf[r]["flag"] == 0 and inf[r]["iter"] == ir[r]["iter"]
            assert np.linalg.norm(B[r] - Aor(Xh[r])) / np.linalg.norm(B[r]) <= 1e-10 * 1.01
        assert np.linalg.norm(Xh - Xr.cpu().numpy()) <= 1e-12 * np.linalg.norm(Xh)
    # one preconditioner for particles on two contexts is refused before any work
    from voxscatter_gb300._lib import VoxScatterError
    with pytest.raises(VoxScatterError, match="share a preconditioner"):
        api.solve_particles_device([parts[0][0], parts[1][0]], [parts[0][1], parts[0][1]],
                                   [parts[0][2].data_ptr(), parts[1][2].data_ptr()], [Xs[0].data_ptr(), Xs[1].data_ptr()],
                                   [4, 4], tol=1e-10, precision="fp64")


@pytest.mark.parametrize("precision,tol", [("mixed", 1e-6), ("fp64", 1e-10)])
def test_particles_lockstep_per_direction_alpha(api, precision, tol):
    """vs_solve_particles: three plates of different sizes on one context,
    4 incident directions / polarisations each with its own alpha_LDR, solved
    in lockstep (one graph launch per inner iteration of all plates).  Every
    right-hand side meets tol against the oracle operator with its own alpha;
    in FP64 every particle reproduces its own vs_solve_batch_device solve
    (same iteration counts, same solutions)."""
    import torch
    parts = []
    for k, diam in enumerate((2.5, 2.0, 3.0)):
        p = W.small_hex(m=1.31 + 0.05j, diameter=diam, nper=4)
        L, M, N, idx3, Toep, alpha, dV, b0, Aor = _system(p)
        fN = O.fft_operator(O.circulant_nop_const(Toep))
        chi = np.zeros(L * M * N); chi[p["idx"]] = 1
        chi = chi.reshape((L, M, N), order="F")
        op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
        pr = api.Preconditioner(op, shift=1 / alpha, d=dV) if k != 1 else None  # one without
        pairs = _directions(p, 2, 20 + k)
        B = np.array([O.PlaneWavePointWise(pol, kv, p["r"]).ravel(order="F")[idx3] for kv, pol in pairs])
        alphas = np.array([O.alpha_ldr(p["refInd"], p["ko"], p["d"], kv, pol) for kv, pol in pairs])
        parts.append(dict(op=op, pr=pr, B=B, Bd=torch.from_numpy(B).cuda(), alphas=alphas, fN=fN, chi=chi, dV=dV,
                          LMN=(L, M, N), idx3=idx3))
    Xs = [torch.zeros_like(q["Bd"]) for q in parts]
    torch.cuda.synchronize()
    out = api.solve_particles([q["op"] for q in parts], [q["pr"] for q in parts], [q["Bd"].data_ptr() for q in parts],
                              [X.data_ptr() for X in Xs], [len(q["B"]) for q in parts],
                              grams=[1 / q["alphas"] for q in parts], tol=tol, precision=precision)
    assert len(out) == 3
    for q, X, inf in zip(parts, Xs, out):
        Xh = X.cpu().numpy()
        L, M, N = q["LMN"]
        for r in range(len(q["B"])):
            assert inf[r]["flag"] == 0, inf[r]
            Ar = O.MVP(Xh[r], q["fN"], np.ones((L, M, N)), q["dV"] * q["chi"], 1 / q["alphas"][r], "notransp", q["idx3"])
            assert np.linalg.norm(q["B"][r] - Ar) / np.linalg.norm(q["B"][r]) <= tol * 1.01
        if precision == "fp64":
            Xr = torch.zeros_like(q["Bd"])
            torch.cuda.synchronize()
            ir = api.solve_batch_device(q["op"], q["Bd"].data_ptr(), Xr.data_ptr(), len(q["B"]), q["pr"], tol=tol,
                                        precision="fp64", gram=1 / q["alphas"])
            for r in range(len(q["B"])):
                assert ir[r]["iter"] == inf[r]["iter"]
            assert np.linalg.norm(Xh - Xr.cpu().numpy()) <= 1e-12 * np.linalg.norm(Xh)
    # a second call reuses the captured graph and gives the same result
    Xs2 = [torch.zeros_like(q["Bd"]) for q in parts]
    torch.cuda.synchronize()
    out2 = api.solve_particles([q["op"] for q in parts], [q["pr"] for q in parts],
                               [q["Bd"].data_ptr() for q in parts], [X.data_ptr() for X in Xs2],
                               [len(q["B"]) for q in parts], grams=[1 / q["alphas"] for q in parts], tol=tol,
                               precision=precision)
    for X, X2, i1, i2 in zip(Xs, Xs2, out, out2):
        assert [a["iter"] for a in i1] == [a["iter"] for a in i2]
        assert torch.equal(X, X2)


def test_particles_rejects_shared_objects(api):
    import torch
    from voxscatter_gb300._lib import VoxScatterError
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.0, nper=3)
    L, M, N, idx3, Toep, alpha, dV, b0, Aor = _system(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    op2 = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    Bd = torch.from_numpy(np.array([b0])).cuda()
    X = torch.zeros_like(Bd)
    with pytest.raises(VoxScatterError, match="appears twice"):
        api.solve_particles([op, op], None, [Bd.data_ptr()] * 2, [X.data_ptr()] * 2, [1, 1])
    with pytest.raises(VoxScatterError, match="appears twice"):
        api.solve_particles([op, op2], [pr, pr], [Bd.data_ptr()] * 2, [X.data_ptr()] * 2, [1, 1])
    other = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep, ctx=api.Context(0))
    with pytest.raises(VoxScatterError, match="one context"):
        api.solve_particles([op, other], None, [Bd.data_ptr()] * 2, [X.data_ptr()] * 2, [1, 1])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_solve_profile_inside_the_graph(api, precision):
    """vs_solve_opts.profile_ms: a BiCGSTAB solve with CUDA events between the
    launches of its captured iterations gives the same solution bit for bit as
    the plain solve (the events change no arithmetic), a positive duration for
    every preconditioner and matvec pass and for the solver kernels, counted
    over whole graph launches (multiples of iters_per_graph), and the FP64
    residual per call; a plain solve afterwards captures its own graph again."""
    import torch
    p = W.small_hex(m=1.31 + 0.05j, diameter=2.5, nper=4)
    L, M, N, idx3, Toep, alpha, dV, b, Aor = _system(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    bd = torch.from_numpy(b.astype(np.complex128)).cuda()
    xs = []
    for profile in (False, True, False):
        xd = torch.zeros_like(bd)
        torch.cuda.synchronize()
        info = api.solve_device(op, bd.data_ptr(), xd.data_ptr(), pr, tol=1e-6 if precision == "mixed" else 1e-10,
                                precision=precision, iters_per_graph=2, profile=profile)
        op.ctx.synchronize()
        assert info["flag"] == 0, info
        xs.append(xd.cpu().numpy())
        if profile:
            prof = info["profile"]
            assert all(prof[k] > 0 for k in api.PROFILE_KEYS), prof
            assert prof["solver_kernels_per_iter"] > 0
            assert prof["iterations"] >= 2 and prof["iterations"] % 2 == 0, prof
            assert prof["iterations"] <= info["iter"] + 1
            assert prof["fp64_residual"] > 0 and prof["fp64_residual_calls"] >= 1
            # one pass takes less than the whole solve
            assert max(prof[k] for k in api.PROFILE_KEYS) < info["time_ms"]
    assert np.array_equal(xs[0], xs[1]) and np.array_equal(xs[0], xs[2])


@pytest.mark.parametrize("precision,tol", [("mixed", 1e-6), ("fp64", 1e-10)])
@pytest.mark.parametrize("nrhs", [1, 3])
def test_folded_vector_steps_match_separate_kernels(api, precision, tol, nrhs):
    """BiCGSTAB with its vector steps folded into the x passes (p and s formed
    in the preconditioner's forward x pass, rt^H v and t^H s, t^H t added in the
    matvec's inverse x pass, the scalar steps taken from the passes' partial
    sums) against the separate kernels, on the 27 x 23 x 7 hex plate with
    both x passes forced to the two-level kernels (the folded form needs
    them): both converge with the oracle's FP64 MVP confirming
    ||b - A x|| <= tol ||b||, the solutions agree to the tolerance, the
    iteration counts to a half step, and the launch counts show which form
    ran (23 against 26 kernels per iteration)."""
    p = W.config1()
    L, M, N, idx3, Toep, alpha, dV, b, Aor = _system(p)
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep)
    pr = api.Preconditioner(op, shift=1 / alpha, d=dV)
    for prec in ("c64", "c128"):
        op.set_shape(prec, x_reg=1)
        pr.set_shape(prec, x_reg=1, fuse_xy=0)
    rng = np.random.default_rng(7)
    B = np.stack([b] + [b * np.exp(1j * rng.uniform(0, 2 * np.pi)) + 0.3 * (rng.normal(size=b.size) +
                                                                              1j * rng.normal(size=b.size))
                        for _ in range(nrhs - 1)])
    out = {}
    for fold in (True, False):
        X, infos = api.solve_batch(op, B, pr, tol=tol, precision=precision, fold=fold)
        for r in range(nrhs):
            assert infos[r]["flag"] == 0, (fold, r, infos[r])
            true_rel = np.linalg.norm(B[r] - Aor(X[r])) / np.linalg.norm(B[r])
            assert true_rel <= tol * 1.01, (fold, r, true_rel)
        out[fold] = (X, infos)
    Xf, inf_f = out[True]
    Xs, inf_s = out[False]
    for r in range(nrhs):
        assert np.linalg.norm(Xf[r] - Xs[r]) / np.linalg.norm(Xs[r]) < 20 * tol, r
        assert abs(inf_f[r]["iter"] - inf_s[r]["iter"]) <= 0.5, (r, inf_f[r]["iter"], inf_s[r]["iter"])
    # per graph launch: 23 kernels per iteration folded, 26 separate
    assert inf_f[0]["launches"] < inf_s[0]["launches"], (inf_f[0]["launches"], inf_s[0]["launches"])
