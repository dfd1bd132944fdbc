"""Excitation, extinction cross section, its adjoint gradient and Mie theory.
FP64 restatement / published methods (test infrastructure only).

* PlaneWavePointWise: src/src_vie/src_fields/src_excitations/PlaneWavePointWise.m:7-19.
* C_ext: absent from the reference (README.md:35 lists far-field routines as a
  to-do); Draine & Flatau, JOSA A 11 (1994) 1491, eq. (8):
  C_ext = 4 pi k / |E0|^2 sum_j Im(E_inc,j^* . p_j), with p_j = dV * P_j because the
  reference's unknown is the dipole moment per unit volume (main_DDA.m:75,139-140).
* Gradient: adjoint method on A(eps) P = E_inc with A = diag(1/alpha_LDR(eps)) - dV*G;
  A is complex symmetric, so the adjoint system is A^T lam = conj(E_inc).
* Mie: Bohren & Huffman (1983) BHMIE series for the extinction efficiency.
* Whole-domain field: main_DDA.m:136-148 (Pout/Eout on the grid, MVP over idxAll
  with Mr = 1, Mc = dV, Gram = 1/alpha, E = Einc - Etemp + Eout).
* Far field: absent from the reference (README.md:35); the far zone of the DDA
  Green tensor (getOPERATOR_DDA.m:99-113), E_sca -> exp(ik r)/r F(n) with
  F(n) = k^2 (I - n n) sum_j p_j exp(-ik n.r_j), p_j = dV P_j.
"""
import numpy as np

from .mvp import MVP
from .operators import alpha_ldr, dalpha_inv_deps


def PlaneWavePointWise(Eo, kvec, r):
    """Einc(L,M,N,3) = Eo * exp(i k.r), PlaneWavePointWise.m:7-19."""
    r = np.asarray(r, dtype=float)
    kr = kvec[0] * r[..., 0] + kvec[1] * r[..., 1] + kvec[2] * r[..., 2]
    e = np.exp(1j * kr)
    return np.stack([Eo[0] * e, Eo[1] * e, Eo[2] * e], axis=-1)


def cext_dda(P, Einc, ko, dV, Eo):
    """Extinction cross section from the polarisation P (3*nnz, idx3 order) and
    the incident field at the same entries."""
    return 4.0 * np.pi * ko * dV * np.sum(np.imag(np.conj(Einc) * P)) / np.sum(np.abs(np.asarray(Eo)) ** 2)


def cext_grad_dda(P, lam, eps_vox, ko, d, kvec, Eo):
    """dC_ext/dRe(eps) and dC_ext/dIm(eps) per voxel, given the forward solution P
    and the adjoint solution lam of A^T lam = conj(E_inc) (both 3*nnz, idx3 order)."""
    nnz = len(eps_vox)
    dV = d ** 3
    c = 4.0 * np.pi * ko * dV / np.sum(np.abs(np.asarray(Eo)) ** 2)
    lp = (lam * P).reshape(3, nnz).sum(axis=0)
    g = dalpha_inv_deps(eps_vox, ko, d, kvec, Eo) * lp
    return -c * np.imag(g), -c * np.real(g)


def mie_qext(x, m, nstop=None):
    """Extinction efficiency of a homogeneous sphere, size parameter x, relative
    index m (BHMIE recurrences, Bohren & Huffman 1983, appendix A)."""
    m = complex(m)
    if nstop is None:
        nstop = int(np.ceil(x + 4.05 * x ** (1.0 / 3.0) + 2.0))
    y = m * x
    nmx = int(max(nstop, abs(y)) + 15)
    D = np.zeros(nmx + 1, dtype=complex)
    for n in range(nmx, 0, -1):
        D[n - 1] = n / y - 1.0 / (D[n] + n / y)
    psi0, psi1 = np.cos(x), np.sin(x)
    chi0, chi1 = -np.sin(x), np.cos(x)
    xi1 = complex(psi1, -chi1)
    q = 0.0
    for n in range(1, nstop + 1):
        psi = (2.0 * n - 1.0) * psi1 / x - psi0
        chi = (2.0 * n - 1.0) * chi1 / x - chi0
        xi = complex(psi, -chi)
        an = ((D[n] / m + n / x) * psi - psi1) / ((D[n] / m + n / x) * xi - xi1)
        bn = ((D[n] * m + n / x) * psi - psi1) / ((D[n] * m + n / x) * xi - xi1)
        q += (2.0 * n + 1.0) * (an.real + bn.real)
        psi0, psi1 = psi1, psi
        chi0, chi1 = chi1, chi
        xi1 = complex(psi1, -chi1)
    return 2.0 / x ** 2 * q


def field_dda(P, idx3, Einc_grid, fN, alpha, dV, chi, L, M, N):
    """E on the whole (L,M,N,3) grid (column-major flat), main_DDA.m:136-148."""
    nD = L * M * N
    Pout = np.zeros(3 * nD, dtype=complex)
    Pout[np.asarray(idx3)] = P
    idx_all = np.arange(3 * nD)
    temp = MVP(Pout, fN, np.ones((L, M, N)), dV, 1.0 / alpha, "notransp", idx_all)
    return np.asarray(Einc_grid, dtype=complex) - temp + Pout / chi


def far_field(P, idx3, r, ko, dV, dirs):
    """F(n) (ndir, 3) by the direct sum over the unknowns (P in idx3 order)."""
    r = np.asarray(r, dtype=float)
    L, M, N = r.shape[:3]
    nD = L * M * N
    idx3 = np.asarray(idx3)
    vox = idx3[: len(idx3) // 3] % nD
    pos = r.reshape(nD, 3, order="F")[vox]  # (nvox, 3)
    Pv = np.asarray(P, dtype=complex).reshape(3, -1)  # (3, nvox)
    out = []
    for n in np.asarray(dirs, dtype=float).reshape(-1, 3):
        ph = np.exp(-1j * ko * (pos @ n))
        s = Pv @ ph
        out.append(ko ** 2 * dV * (s - n * (n @ s)))
    return np.array(out)


def polarisation_basis(k):
    """Two orthonormal linear polarisations of a unit direction k:
    e1 = k x z / |k x z| (k x x when k is along z), e2 = k x e1."""
    k = np.asarray(k, dtype=float)
    a = np.cross(k, [0.0, 0.0, 1.0])
    if np.linalg.norm(a) < 1e-6:
        a = np.cross(k, [1.0, 0.0, 0.0])
    e1 = a / np.linalg.norm(a)
    return e1, np.cross(k, e1)


def orientation_average_cext(solve, Einc_of, ko, dV, dirs, weights=None, psi=None):
    """Random-orientation averaging (absent from the reference, README.md:37):
    the particle stays fixed and the incident wave runs over the orientations
    (unit direction dirs[j], polarisation pair of polarisation_basis turned by
    psi[j] about it) with weights; solve(kvec, e) returns the polarisation P
    of that incidence (the system with that incidence's alpha_LDR) and
    Einc_of(kvec, e) its incident field at the unknowns.  C_ext (|E0| = 1) is
    averaged over the two polarisations and then over the orientations.
    Returns (average, (ndir, 2))."""
    dirs = np.asarray(dirs, dtype=float).reshape(-1, 3)
    w = np.ones(len(dirs)) if weights is None else np.asarray(weights, dtype=float)
    psi = np.zeros(len(dirs)) if psi is None else np.asarray(psi, dtype=float)
    each = np.zeros((len(dirs), 2))
    for j, d in enumerate(dirs):
        k = d / np.linalg.norm(d)
        b1, b2 = polarisation_basis(k)
        c, s_ = np.cos(psi[j]), np.sin(psi[j])
        for pol, e in enumerate((c * b1 + s_ * b2, -s_ * b1 + c * b2)):
            kvec = ko * k
            P = solve(kvec, e)
            each[j, pol] = cext_dda(P, Einc_of(kvec, e), ko, dV, e)
    return float(np.sum(w * each.mean(axis=1)) / np.sum(w)), each
