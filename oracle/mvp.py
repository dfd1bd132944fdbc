"""FFT matvec of the VIE / DDA operator and dense direct-sum checks.
FP64 restatement (test infrastructure only).

Follows src/src_vie/src_mvp/MVP.m:38-145 (identical to mv_AN_const.m).
"""
import numpy as np

from . import _fft as _F

from .operators import COMP_PAIRS, _dda_tensor

# Output component a accumulates fN component PAIR[a][b] times input b (MVP.m:108-123)
PAIR = [[0, 1, 2], [1, 3, 4], [2, 4, 5]]


def _grid(a, shape):
    a = np.asarray(a)
    if a.ndim == 0:
        return np.full(shape, a, dtype=complex)
    return a.astype(complex).reshape(shape, order="F")


def MVP(JIn0, fN, Mr, Mc, Gram, transp_flag, idx, GPU_flag=0):
    """JOut = MVP(JIn0, fN, Mr, Mc, Gram, transp_flag, idx, GPU_flag), MVP.m:1-145.

    ``idx`` are 0-based linear indices into the column-major (L,M,N,3) grid
    (MATLAB's idx3 minus one).  ``Mr`` fixes (L,M,N); ``Mc``/``Gram`` are
    scalars or (L,M,N) arrays.  GPU_flag is accepted and ignored (the oracle is
    CPU only)."""
    fN = np.asarray(fN)
    P, Q, R = fN.shape[:3]
    Mr = np.asarray(Mr)
    L, M, N = Mr.shape
    Mr = _grid(Mr, (L, M, N))
    Mc = _grid(Mc, (L, M, N))
    Gram = _grid(Gram, (L, M, N))
    idx = np.asarray(idx, dtype=np.int64)
    JInf = np.zeros(3 * L * M * N, dtype=complex)
    JInf[idx] = np.asarray(JIn0, dtype=complex).ravel()
    JIn = JInf.reshape((L, M, N, 3), order="F")
    JOut = np.zeros((L, M, N, 3), dtype=complex)
    if transp_flag == "transp":  # MVP.m:65-99
        Mcc = np.conj(Mc)
        fJ = [_F.fftn(np.conj(Mcc * JIn[..., b]), s=(P, Q, R), axes=(0, 1, 2)) for b in range(3)]
        for a in range(3):
            acc = sum(fN[..., PAIR[a][b]] * fJ[b] for b in range(3))
            J = _F.ifftn(acc, axes=(0, 1, 2))
            JOut[..., a] = Gram * np.conj(Mr) * JIn[..., a] - np.conj(J[:L, :M, :N])
    elif transp_flag == "notransp":  # MVP.m:101-133
        fJ = [_F.fftn(JIn[..., b], s=(P, Q, R), axes=(0, 1, 2)) for b in range(3)]
        for a in range(3):
            acc = sum(fN[..., PAIR[a][b]] * fJ[b] for b in range(3))
            J = _F.ifftn(acc, axes=(0, 1, 2))
            JOut[..., a] = Gram * Mr * JIn[..., a] - Mc * J[:L, :M, :N]
    else:
        raise ValueError("transp_flag must be 'transp' or 'notransp'")
    return JOut.ravel(order="F")[idx]


mv_AN_const = MVP  # src/src_vie/src_mvp/mv_AN_const.m is the same function


def MVP_plain_transpose(JIn0, fN, Mr, Mc, Gram, idx):
    """Plain (unconjugated) transpose A^T x = Gram*Mr*x - N(Mc*x) of the
    'notransp' operator: the complex-symmetric adjoint needed for gradients
    (N^T = N because the Green tensor is symmetric)."""
    fN = np.asarray(fN)
    P, Q, R = fN.shape[:3]
    Mr = np.asarray(Mr)
    L, M, N = Mr.shape
    Mr = _grid(Mr, (L, M, N)); Mc = _grid(Mc, (L, M, N)); Gram = _grid(Gram, (L, M, N))
    JInf = np.zeros(3 * L * M * N, dtype=complex)
    JInf[np.asarray(idx)] = np.asarray(JIn0, dtype=complex).ravel()
    JIn = JInf.reshape((L, M, N, 3), order="F")
    JOut = np.zeros((L, M, N, 3), dtype=complex)
    fJ = [_F.fftn(Mc * JIn[..., b], s=(P, Q, R), axes=(0, 1, 2)) for b in range(3)]
    for a in range(3):
        acc = sum(fN[..., PAIR[a][b]] * fJ[b] for b in range(3))
        J = _F.ifftn(acc, axes=(0, 1, 2))
        JOut[..., a] = Gram * Mr * JIn[..., a] - J[:L, :M, :N]
    return JOut.ravel(order="F")[np.asarray(idx)]


def dense_dda_matrix(r, vox_idx, ko, Gram, Mc, Mr=1.0):
    """Dense O(n^2) DDA matrix on the voxels ``vox_idx`` (0-based linear, column
    major): A[(a,al),(b,be)] = Gram*Mr*delta - Mc_a * G_al,be(r_a - r_b), with the
    Draine-Flatau tensor evaluated directly at each pair offset (no Toeplitz
    storage, no embedding).  Unknown ordering matches idx3 (component-major)."""
    r = np.asarray(r, dtype=float)
    L, M, N, _ = r.shape
    pts = r.reshape((-1, 3), order="F")[np.asarray(vox_idx)]
    n = len(pts)
    D = pts[:, None, :] - pts[None, :, :]
    Gt = _dda_tensor(D, ko)  # (n, n, 6)
    A = np.zeros((3 * n, 3 * n), dtype=complex)
    g = np.broadcast_to(np.asarray(Gram, dtype=complex) * np.asarray(Mr, dtype=complex), (n,)) \
        if np.ndim(Gram) == 0 or np.size(Gram) == 1 else np.asarray(Gram).ravel(order="F")[vox_idx] * \
        (np.asarray(Mr) if np.ndim(Mr) == 0 else np.asarray(Mr).ravel(order="F")[vox_idx])
    mc = np.broadcast_to(np.asarray(Mc, dtype=complex), (n,)) if np.ndim(Mc) == 0 \
        else np.asarray(Mc).ravel(order="F")[vox_idx]
    for c, (a, b) in enumerate(COMP_PAIRS):
        blk = -mc[:, None] * Gt[:, :, c]
        A[a * n:(a + 1) * n, b * n:(b + 1) * n] += blk
        if a != b:
            A[b * n:(b + 1) * n, a * n:(a + 1) * n] += blk
    A[np.arange(3 * n), np.arange(3 * n)] += np.tile(g, 3)
    return A


def dense_from_toeplitz(Toep, vox_idx, Gram, Mc, Mr=1.0):
    """Dense matrix built from the stored first-octant Toeplitz tensor by
    explicit per-axis parity (gperiodic_coeff_nop.m), without any FFT."""
    from .operators import gperiodic_coeff_nop
    L, M, N, _ = Toep.shape
    ii, jj, kk = np.unravel_index(np.asarray(vox_idx), (L, M, N), order="F")
    n = len(ii)
    sL, sM, sN = (gperiodic_coeff_nop(c) for c in ("L", "M", "N"))
    di = ii[:, None] - ii[None, :]
    dj = jj[:, None] - jj[None, :]
    dk = kk[:, None] - kk[None, :]
    A = np.zeros((3 * n, 3 * n), dtype=complex)
    mc = np.broadcast_to(np.asarray(Mc, dtype=complex), (n,)) if np.ndim(Mc) == 0 \
        else np.asarray(Mc).ravel(order="F")[vox_idx]
    for c, (a, b) in enumerate(COMP_PAIRS):
        s = np.where(di < 0, sL[c], 1.0) * np.where(dj < 0, sM[c], 1.0) * np.where(dk < 0, sN[c], 1.0)
        blk = -mc[:, None] * s * Toep[np.abs(di), np.abs(dj), np.abs(dk), c]
        A[a * n:(a + 1) * n, b * n:(b + 1) * n] += blk
        if a != b:
            A[b * n:(b + 1) * n, a * n:(a + 1) * n] += blk
    g = np.asarray(Gram, dtype=complex) * np.asarray(Mr, dtype=complex)
    g = np.broadcast_to(g, (n,)) if g.ndim == 0 else g.ravel(order="F")[vox_idx]
    A[np.arange(3 * n), np.arange(3 * n)] += np.tile(g, 3)
    return A
