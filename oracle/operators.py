"""DDA operator assembly: LDR polarisability, Draine-Flatau Toeplitz tensor,
circulant embedding and its FFT.  FP64 restatement (test infrastructure only).

Follows src/src_vie/src_operators/getOPERATOR_DDA.m:1-122,
circulant_nop_const.m:1-40, gperiodic_coeff_nop.m:1-33, fft_operator.m:1-8.
"""
import numpy as np

from . import _fft as _F

# Lattice-dispersion-relation coefficients, getOPERATOR_DDA.m:7-9
B1 = -1.8915316
B2 = 0.1648469
B3 = -1.7700004

# Tensor component order xx, xy, xz, yy, yz, zz (getOPERATOR_DDA.m:107-112)
COMP_PAIRS = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]


def ldr_S(kvec, Eo):
    """S = sum_j (a_hat_j e_hat_j)^2, getOPERATOR_DDA.m:15-20."""
    kvec = np.asarray(kvec, dtype=float)
    Eo = np.asarray(Eo, dtype=float)
    a_hat = kvec / np.linalg.norm(kvec)
    e_hat = Eo / np.linalg.norm(Eo)
    S = 0.0
    for j in range(3):
        S = S + (a_hat[j] * e_hat[j]) ** 2
    return S


def alpha_ldr(refInd_or_eps, ko, d, kvec, Eo, is_eps=False):
    """alpha_LDR, getOPERATOR_DDA.m:10-26.

    ``refInd_or_eps`` is the refractive index m (or, with ``is_eps``, the
    permittivity eps = m^2); scalar or array.  Returns the dimensionless
    polarisability (dipole polarisability divided by d^3).
    """
    msqr = np.asarray(refInd_or_eps, dtype=complex)
    if not is_eps:
        msqr = msqr ** 2
    S = ldr_S(kvec, Eo)
    dcube = d ** 3
    alpha_CM = 3.0 / (4.0 * np.pi) * (msqr - 1.0) / (msqr + 2.0)
    return alpha_CM / (1.0 + alpha_CM * ((B1 + msqr * B2 + msqr * B3 * S) * (ko * d) ** 2
                                         - 2.0 / 3.0 * 1j * ko ** 3 * dcube))


def dalpha_inv_deps(eps, ko, d, kvec, Eo):
    """d(1/alpha_LDR)/d(eps), the derivative of the inverse of getOPERATOR_DDA.m:26
    with msqr = eps (holomorphic in eps)."""
    eps = np.asarray(eps, dtype=complex)
    S = ldr_S(kvec, Eo)
    return -4.0 * np.pi / (eps - 1.0) ** 2 + (B2 + B3 * S) * (ko * d) ** 2


def _dda_tensor(R, ko):
    """Draine-Flatau interaction tensor at offsets R (..., 3); getOPERATOR_DDA.m:99-113.
    Returns (..., 6) with G(0) = 0."""
    R = np.asarray(R, dtype=float)
    rjk = np.sqrt(np.sum(R * R, axis=-1))
    out = np.zeros(R.shape[:-1] + (6,), dtype=complex)
    nz = np.abs(rjk) > 1e-15
    r = rjk[nz]
    rh = R[nz] / r[:, None]
    pre = np.exp(1j * ko * r) / r
    c1 = ko ** 2
    c2 = (1j * ko * r - 1.0) / r ** 2
    for c, (a, b) in enumerate(COMP_PAIRS):
        I = 1.0 if a == b else 0.0
        rr = rh[:, a] * rh[:, b]
        out[nz, c] = pre * (c1 * (I - rr) + c2 * (I - 3.0 * rr))
    return out


def green_toeplitz(r, ko, nearby_quad="off"):
    """Toep(L,M,N,6): the tensor at every offset r(i,j,k)-r(1,1,1),
    getOPERATOR_DDA.m:29-119.  ``nearby_quad='on'`` averages the kernel over the
    target voxel with a 10^3 Gauss-Legendre rule for 0 < |R| < 5 dx
    (getOPERATOR_DDA.m:35-79)."""
    r = np.asarray(r, dtype=float)
    L, M, N, _ = r.shape
    dx = r[1, 0, 0, 0] - r[0, 0, 0, 0] if L > 1 else 0.0
    R0 = r[0, 0, 0, :]
    Roff = r - R0
    Toep = _dda_tensor(Roff, ko)
    if nearby_quad == "on":
        xg, wg = np.polynomial.legendre.leggauss(10)
        XG, YG, ZG = np.meshgrid(xg, xg, xg, indexing="ij")
        W = np.einsum("i,j,k->ijk", wg * 0.5, wg * 0.5, wg * 0.5)
        rjk = np.sqrt(np.sum(Roff * Roff, axis=-1))
        near = (rjk < 5 * dx) & (rjk > 1e-15)
        for (i, j, k) in zip(*np.nonzero(near)):
            R1 = r[i, j, k, :]
            pts = np.stack([R1[0] + dx / 2 * XG, R1[1] + dx / 2 * YG,
                            R1[2] + dx / 2 * ZG], axis=-1) - R0
            vals = _dda_tensor(pts, ko)
            Toep[i, j, k, :] = np.einsum("abcz,abc->z", vals, W)
    return Toep


def gperiodic_coeff_nop(cube):
    """Parity signs per tensor component for each reflected octant,
    gperiodic_coeff_nop.m:4-31."""
    table = {
        "L": [+1, -1, -1, +1, +1, +1],
        "M": [+1, -1, +1, +1, -1, +1],
        "N": [+1, +1, -1, +1, -1, +1],
        "LM": [+1, +1, -1, +1, -1, +1],
        "LN": [+1, -1, +1, +1, -1, +1],
        "MN": [+1, -1, -1, +1, +1, +1],
        "LMN": [+1, +1, +1, +1, +1, +1],
    }
    return np.array(table[cube], dtype=float)


def circulant_nop_const(G):
    """(L,M,N,6) -> (2L,2M,2N,6) parity-signed reflection embedding,
    circulant_nop_const.m:1-40."""
    L, M, N, _ = G.shape
    Gp = np.zeros((2 * L, 2 * M, 2 * N, 6), dtype=complex)
    Gp[:L, :M, :N, :] = G
    sL, sM, sN = (gperiodic_coeff_nop(c) for c in ("L", "M", "N"))
    sLM, sLN, sMN = (gperiodic_coeff_nop(c) for c in ("LM", "LN", "MN"))
    rL = slice(L - 1, 0, -1)
    rM = slice(M - 1, 0, -1)
    rN = slice(N - 1, 0, -1)
    for ii in range(6):
        Gp[L + 1:, :M, :N, ii] = G[rL, :, :, ii] * sL[ii]
        Gp[:L, M + 1:, :N, ii] = G[:, rM, :, ii] * sM[ii]
        Gp[:L, :M, N + 1:, ii] = G[:, :, rN, ii] * sN[ii]
        Gp[L + 1:, M + 1:, :N, ii] = G[rL, rM, :, ii] * sLM[ii]
        Gp[L + 1:, :M, N + 1:, ii] = G[rL, :, rN, ii] * sLN[ii]
        Gp[:L, M + 1:, N + 1:, ii] = G[:, rM, rN, ii] * sMN[ii]
    Gp[L + 1:, M + 1:, N + 1:, :] = G[rL, rM, rN, :]
    return Gp


def fft_operator(A):
    """3-D FFT of each component, fft_operator.m:1-8."""
    return _F.fftn(A, axes=(0, 1, 2))


def getOPERATOR_DDA(r, ko, refInd, kvec, Eo, nearby_quad="off"):
    """[op_out, Toep, alpha_LDR] = getOPERATOR_DDA(...), getOPERATOR_DDA.m:1-122."""
    r = np.asarray(r, dtype=float)
    dx = r[1, 0, 0, 0] - r[0, 0, 0, 0]
    alpha = alpha_ldr(refInd, ko, dx, kvec, Eo)
    Toep = green_toeplitz(r, ko, nearby_quad)
    op_out = fft_operator(circulant_nop_const(Toep))
    return op_out, Toep, alpha
