"""Krylov solvers with MATLAB's calling conventions.  FP64 restatement (test
infrastructure only).

The reference calls MATLAB's built-in ``bicgstab``/``gmres`` (closed MathWorks
code, version unpinned) at main_DDA.m:82,89,120-121,128-129 and
scatteringHumanHead.m:109,205, and ships its own restarted GMRES in
src/src_numeric/src_iterative/pgmres.m:70-181 + pgmres_iter.m:22-150.

* ``bicgstab`` is the preconditioned BiCGSTAB of van der Vorst (1992) in the
  form of Barrett et al., "Templates for the Solution of Linear Systems" (1994),
  with MATLAB's documented outputs [x, flag, relres, iter, resvec]: the
  preconditioner handle returns M\\x, convergence is tested on the unpreconditioned
  residual at every half step, ``iter`` may be a half integer and ``resvec`` holds
  the residual norm at every half step (length 2*iter+1).
* ``gmres`` is restarted GMRES (Saad & Schultz 1986) with modified Gram-Schmidt
  and Givens rotations, left preconditioned as MATLAB documents: it stops on the
  preconditioned residual norm(M\\(b-Ax))/norm(M\\b) and reports iter=[outer, inner].
* ``pgmres`` restates pgmres.m / pgmres_iter.m (classical Gram-Schmidt, dense
  least squares per step).
* ``pgmres_dr`` restates pgmresDR.m / pgmresDR_iter.m / getHarmVecs1.m /
  getHarmVecs2.m (GCRO-DR with harmonic Ritz recycling), with
  ``numpy.linalg.eig`` / ``scipy.linalg.eig`` for MATLAB's ``eig``.

Iteration counts cannot be pinned to MATLAB's closed built-ins.
"""
import numpy as np


def _as_fun(A):
    if callable(A):
        return A
    A = np.asarray(A)
    return lambda x: A @ x


def bicgstab(A, b, tol=1e-6, maxit=None, M1=None, M2=None, x0=None):
    afun = _as_fun(A)
    b = np.asarray(b, dtype=complex).ravel()
    n = b.size
    if maxit is None:
        maxit = min(n, 20)
    prec = [f for f in (M1, M2) if f is not None]

    def minv(v):
        for f in prec:
            v = _as_fun(f)(v)
        return v

    x = np.zeros(n, dtype=complex) if x0 is None else np.asarray(x0, dtype=complex).copy()
    nb = np.linalg.norm(b)
    if nb == 0:
        return np.zeros(n, dtype=complex), 0, 0.0, 0, np.array([0.0])
    r = b - afun(x) if np.any(x) else b.copy()
    rt = r.copy()
    resvec = [np.linalg.norm(r)]
    if resvec[0] <= tol * nb:
        return x, 0, resvec[0] / nb, 0, np.array(resvec)
    rho_prev = alpha = omega = 1.0
    p = np.zeros(n, dtype=complex); v = np.zeros(n, dtype=complex)
    flag = 1
    it = 0.0
    for i in range(1, maxit + 1):
        rho = np.vdot(rt, r)
        if rho == 0:
            flag = 4; break
        if i == 1:
            p = r.copy()
        else:
            beta = (rho / rho_prev) * (alpha / omega)
            p = r + beta * (p - omega * v)
        ph = minv(p)
        v = afun(ph)
        rtv = np.vdot(rt, v)
        if rtv == 0:
            flag = 4; break
        alpha = rho / rtv
        s = r - alpha * v
        ns = np.linalg.norm(s)
        resvec.append(ns)
        if ns <= tol * nb:
            x = x + alpha * ph
            flag = 0; it = i - 0.5
            break
        sh = minv(s)
        t = afun(sh)
        tt = np.vdot(t, t)
        if tt == 0:
            flag = 4; break
        omega = np.vdot(t, s) / tt
        if omega == 0:
            flag = 4; break
        x = x + alpha * ph + omega * sh
        r = s - omega * t
        nr = np.linalg.norm(r)
        resvec.append(nr)
        it = float(i)
        if nr <= tol * nb:
            flag = 0; break
        rho_prev = rho
    relres = np.linalg.norm(b - afun(x)) / nb
    return x, flag, relres, it, np.array(resvec)


def gmres(A, b, restart=None, tol=1e-6, maxit=None, M1=None, M2=None, x0=None):
    afun = _as_fun(A)
    b = np.asarray(b, dtype=complex).ravel()
    n = b.size
    if restart is None or restart > n:
        restart = n
    if maxit is None:
        maxit = min(int(np.ceil(n / restart)), 10)
    prec = [f for f in (M1, M2) if f is not None]

    def minv(v):
        for f in prec:
            v = _as_fun(f)(v)
        return v

    x = np.zeros(n, dtype=complex) if x0 is None else np.asarray(x0, dtype=complex).copy()
    nb_prec = np.linalg.norm(minv(b))
    if np.linalg.norm(b) == 0:
        return np.zeros(n, dtype=complex), 0, 0.0, [0, 0], np.array([0.0])
    resvec = []
    flag = 1
    outer = inner = 0
    for outer in range(1, maxit + 1):
        r = minv(b - afun(x))
        beta = np.linalg.norm(r)
        if not resvec:
            resvec.append(beta)
        if beta <= tol * nb_prec:
            flag = 0; inner = 0; outer -= 1
            break
        V = np.zeros((n, restart + 1), dtype=complex)
        H = np.zeros((restart + 1, restart), dtype=complex)
        cs = np.zeros(restart, dtype=complex); sn = np.zeros(restart, dtype=complex)
        g = np.zeros(restart + 1, dtype=complex); g[0] = beta
        V[:, 0] = r / beta
        k_done = 0
        for k in range(restart):
            w = minv(afun(V[:, k]))
            for j in range(k + 1):  # modified Gram-Schmidt
                H[j, k] = np.vdot(V[:, j], w)
                w = w - H[j, k] * V[:, j]
            H[k + 1, k] = np.linalg.norm(w)
            if H[k + 1, k] != 0:
                V[:, k + 1] = w / H[k + 1, k]
            for j in range(k):  # apply previous rotations
                t = cs[j] * H[j, k] + sn[j] * H[j + 1, k]
                H[j + 1, k] = -np.conj(sn[j]) * H[j, k] + cs[j] * H[j + 1, k]
                H[j, k] = t
            a, bb = H[k, k], H[k + 1, k]
            den = np.sqrt(abs(a) ** 2 + abs(bb) ** 2)
            if a == 0:
                cs[k], sn[k] = 0.0, 1.0
            else:
                cs[k] = abs(a) / den
                sn[k] = (a / abs(a)) * np.conj(bb) / den
            H[k, k] = cs[k] * a + sn[k] * bb
            H[k + 1, k] = 0.0
            g[k + 1] = -np.conj(sn[k]) * g[k]
            g[k] = cs[k] * g[k]
            resvec.append(abs(g[k + 1]))
            k_done = k + 1
            if abs(g[k + 1]) <= tol * nb_prec:
                break
        y = np.linalg.solve(np.triu(H[:k_done, :k_done]), g[:k_done])
        x = x + V[:, :k_done] @ y
        inner = k_done
        if abs(g[k_done]) <= tol * nb_prec:
            flag = 0
            break
    relres = np.linalg.norm(minv(b - afun(x))) / nb_prec
    if flag == 0 and relres > tol:
        flag = 1
    return x, flag, relres, [outer, inner], np.array(resvec)


def pgmres(A, b, restart=50, tol=1e-3, maxit=10, L1=None, L2=None, R1=None, R2=None, x0=None):
    """[x,flag,relres,iter,resvec] = pgmres(A,b,restart,tol,maxit,L1,L2,R1,R2,x0),
    pgmres.m:70-181; inner loop pgmres_iter.m:22-150."""
    afun = _as_fun(A)
    b = np.asarray(b, dtype=complex).ravel()
    x = np.zeros_like(b) if x0 is None else np.asarray(x0, dtype=complex).copy()
    r = b - afun(x) if np.any(x) else b.copy()
    bp = b.copy()
    for Lf in (L1, L2):
        if Lf is not None:
            r = _as_fun(Lf)(r); bp = _as_fun(Lf)(bp)
    bnorm = np.linalg.norm(bp)
    resvec = [np.linalg.norm(r) / bnorm]
    outit = 0
    p = 0
    while resvec[-1] > tol and outit < maxit:
        outit += 1
        x, r, p, rin = _pgmres_iter(afun, x, r, restart, L1, L2, R1, R2, tol * bnorm)
        resvec.extend(list(np.asarray(rin) / bnorm))
    relres = np.linalg.norm(b - afun(x)) / np.linalg.norm(b)
    flag = 0 if relres <= tol else 1
    return x, flag, relres, [p, outit], np.array(resvec)


def _pgmres_iter(afun, x, r, m, L1, L2, R1, R2, tol):
    n = r.size
    V = np.zeros((n, m + 1), dtype=complex)
    V[:, 0] = r / np.linalg.norm(r)
    H = np.zeros((m + 1, m), dtype=complex)
    resvec = []
    k = 0
    y = None; res = None
    for k in range(1, m + 1):
        w = V[:, k - 1]
        for Rf in (R1, R2):
            if Rf is not None:
                w = _as_fun(Rf)(w)
        w = afun(w)
        for Lf in (L1, L2):
            if Lf is not None:
                w = _as_fun(Lf)(w)
        H[:k, k - 1] = V[:, :k].conj().T @ w  # classical Gram-Schmidt, pgmres_iter.m:106-107
        w = w - V[:, :k] @ H[:k, k - 1]
        H[k, k - 1] = np.linalg.norm(w)
        V[:, k] = w / H[k, k - 1]
        rhs = np.zeros(k + 1, dtype=complex); rhs[0] = np.linalg.norm(r)
        Hc = H[:k + 1, :k]
        y = np.linalg.lstsq(Hc, rhs, rcond=None)[0]
        res = rhs - Hc @ y
        resvec.append(np.linalg.norm(res))
        if resvec[-1] < tol:
            break
    xupd = V[:, :k] @ y
    for Rf in (R1, R2):
        if Rf is not None:
            xupd = _as_fun(Rf)(xupd)
    x = x + xupd
    r = V[:, :k + 1] @ res
    return x, r, k, resvec


def pgmres_dr(A, b, restart=50, tol=1e-3, maxit=10, ritz=None, L1=None, L2=None, R1=None, R2=None, x0=None):
    """[x,flag,relres,iter,resvec] = pgmresDR(A,b,restart,tol,maxit,ritz,L1,L2,R1,R2,x0),
    src/src_numeric/src_iterative/pgmresDR.m:73-281 with its cycle
    pgmresDR_iter.m:1-142 and the harmonic Ritz selections getHarmVecs1.m /
    getHarmVecs2.m.  GCRO-DR (Parks, de Sturler, Mackey, Johnson, Maiti 2006):
    after each cycle of ``restart`` Arnoldi steps the ``ritz`` harmonic Ritz
    vectors of smallest magnitude span a recycled space U with C = A U
    orthonormal, and the next cycle runs Arnoldi on (I - C C^H) A.  The
    Arnoldi steps use classical Gram-Schmidt once against C and once against V
    (pgmresDR_iter.m:99-107).  ``iter`` = [steps of the last cycle, outer
    cycles after the first]; ``resvec`` holds the residual estimate of every
    Arnoldi step relative to norm(L2\\(L1\\b))."""
    afun = _as_fun(A)
    b = np.asarray(b, dtype=complex).ravel()
    n = b.size
    if ritz is None:
        ritz = min(10, int(round(restart / 2)))
    else:
        ritz = min(ritz, restart - 1)
    x0 = np.zeros(n, dtype=complex) if x0 is None else np.asarray(x0, dtype=complex).ravel()
    r = b - afun(x0)
    bp = b.copy()
    for Lf in (L1, L2):
        if Lf is not None:
            r = _as_fun(Lf)(r); bp = _as_fun(Lf)(bp)
    bnorm = np.linalg.norm(bp)
    resvec = [np.linalg.norm(r) / bnorm]

    def right(v):
        for Rf in (R2, R1):          # pgmresDR_iter.m:58-71: R2 first, then R1
            if Rf is not None:
                v = _as_fun(Rf)(v)
        return v

    def left(v):
        for Lf in (L1, L2):
            if Lf is not None:
                v = _as_fun(Lf)(v)
        return v

    def cycle(r, C):
        m = restart
        V = np.zeros((n, m + 1), dtype=complex)
        V[:, 0] = r / np.linalg.norm(r)
        kc = 0 if C is None else C.shape[1]
        B = np.zeros((kc, m), dtype=complex)
        H = np.zeros((m + 1, m), dtype=complex)
        rin = []
        for k in range(1, m + 1):
            w = left(afun(right(V[:, k - 1])))
            if kc:
                B[:, k - 1] = C.conj().T @ w
                w = w - C @ B[:, k - 1]
            H[:k, k - 1] = V[:, :k].conj().T @ w
            w = w - V[:, :k] @ H[:k, k - 1]
            H[k, k - 1] = np.linalg.norm(w)
            V[:, k] = w / H[k, k - 1]
            rhs = np.zeros(k + 1, dtype=complex); rhs[0] = np.linalg.norm(r)
            Hk = H[:k + 1, :k]
            y = np.linalg.lstsq(Hk, rhs, rcond=None)[0]
            rin.append(np.linalg.norm(rhs - Hk @ y))
            if rin[-1] < tol * bnorm:
                return V[:, :k + 1], H[:k + 1, :k], B[:, :k], k, rin
        return V, H, B, m, rin

    # first cycle: plain GMRES, then the first recycled space (pgmresDR.m:181-221)
    V, H, _, p, rin = cycle(r, None)
    resvec.extend(np.asarray(rin) / bnorm)
    y = np.linalg.lstsq(H, V.conj().T @ r, rcond=None)[0]
    x = V[:, :p] @ y
    r = r - V @ (H @ y)
    U = C = None
    if resvec[-1] > tol:
        P = harm_vecs1(p, min(ritz, p - 1), H)
        U = V[:, :p] @ P
        Q, R = np.linalg.qr(H @ P)
        C = V @ Q
        U = np.linalg.solve(R.T, U.T).T      # U / R
    outit = 0
    while resvec[-1] > tol and outit < maxit:  # pgmresDR.m:226-260
        outit += 1
        V, H, B, p, rin = cycle(r, C)
        resvec.extend(np.asarray(rin) / bnorm)
        k = U.shape[1]
        d = np.linalg.norm(U, axis=0)
        D = np.diag(1.0 / d)
        U = U @ D
        H2 = np.block([[D.astype(complex), B], [np.zeros((H.shape[0], k), dtype=complex), H]])
        CV = np.hstack([C, V])
        y = np.linalg.lstsq(H2, CV.conj().T @ r, rcond=None)[0]
        x = x + np.hstack([U, V[:, :p]]) @ y
        r = r - CV @ (H2 @ y)
        if resvec[-1] > tol:
            P = harm_vecs2(p + k, k, H2, V, U, C)
            U = np.hstack([U, V[:, :p]]) @ P
            Q, R = np.linalg.qr(H2 @ P)
            C = CV @ Q
            U = np.linalg.solve(R.T, U.T).T
    x = x0 + right(x)
    relres = np.linalg.norm(b - afun(x)) / np.linalg.norm(b)
    flag = 0 if relres <= tol else 1
    return x, flag, relres, [p, outit], np.array(resvec)


def _sorted_eig(M):
    """Eigenpairs of M ordered by ascending |lambda| (sortrows on
    [abs(lambda) vecs'], getHarmVecs1.m:15-19)."""
    lam, X = np.linalg.eig(M)
    order = np.argsort(np.abs(lam), kind="stable")
    return lam[order], X[:, order]


def harm_vecs1(m, k, H):
    """getHarmVecs1.m: the k harmonic Ritz vectors of smallest magnitude of the
    (m+1) x m Hessenberg H: eig(H_m + h_{m+1,m}^2 H_m^{-H} e_m e_m^T)."""
    Hm = H[:m, :]
    f = np.linalg.solve(Hm.conj().T, np.eye(m, dtype=complex)[:, m - 1])
    M = Hm.copy()
    M[:, m - 1] += H[m, m - 1] ** 2 * f
    return _sorted_eig(M)[1][:, :k]


def harm_vecs2(m, k, H2, V, U, C):
    """getHarmVecs2.m: eig(H2^H W, H2^H H2) with W = [C V]^H [U V_{m-k}],
    keeping the k eigenvectors of largest |lambda| (the harmonic Ritz values
    of smallest magnitude)."""
    W = np.zeros((m + 1, m), dtype=complex)
    W[:k, :k] = C.conj().T @ U
    W[k:, :k] = V.conj().T @ U
    W[k:m, k:m] = np.eye(m - k)
    import scipy.linalg as sl
    lam, X = sl.eig(H2.conj().T @ W, H2.conj().T @ H2)
    order = np.argsort(np.abs(lam), kind="stable")
    return X[:, order][:, m - k:]
