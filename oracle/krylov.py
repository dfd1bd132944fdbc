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
