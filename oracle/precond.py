"""Chan-Olkin 1- and 2-level circulant preconditioners.  FP64 restatement
(test infrastructure only).

Follows src/src_preconditioning/circ_1_level.m:1-259, circ_2_level.m:1-155,
mvp_circ_2_level.m:1-23, chan_mvp_idx.m:1-17 and the block inversion inlined at
main_DDA.m:107-111 (DDA) / scatteringHumanHead.m:179-184 (JVIE).

The reference's per-component sign conventions are kept exactly, including the
ones that only cancel out for operators whose odd components vanish at zero
offset (circ_1_level.m:29,42 negate the xy/xz averages; circ_2_level.m:44
stores -CC3 while the block uses CC3).
"""
import numpy as np

from . import _fft as _F

# sign applied to the (L+1-i)/L term in circ_1_level.m:14,29,42,55,69,84
_S1 = [+1, -1, -1, +1, +1, +1]
# sign applied to the (M+1-i)/M term in circ_2_level.m:14,27,38,51,63,76
_S2 = [+1, -1, +1, +1, -1, +1]
# sign of the stored circ_M_opToep component, circ_2_level.m:20,31,44,55,67,80
_STORE2 = [+1, +1, -1, +1, +1, +1]


def _chan_average(A, s):
    """T. Chan optimal-circulant first column along axis 0 with the reference's
    sign convention: c(1)=A(1); c(i) = s*(n+1-i)/n*A(i) + (i-1)/n*A(n-i+2)."""
    n = A.shape[0]
    c = np.zeros_like(A)
    c[0] = A[0]
    for i0 in range(1, n):
        c[i0] = s * (n - i0) / n * A[i0] + i0 / n * A[n - i0]
    return c


def circ_1_level(opToeplitz, L, M, N, parallel_prec=0, on_off="off"):
    """[circ, circ_L_opToep] = circ_1_level(...), circ_1_level.m:1-93.
    With on_off='on' the dense 3MN x 3MN blocks are assembled too
    (circ_1_level.m:96-259; tiny grids only)."""
    T = np.asarray(opToeplitz, dtype=complex)
    out = np.zeros((L, M, N, 6), dtype=complex)
    for c in range(6):
        out[..., c] = _F.fft(_chan_average(T[..., c], _S1[c]), axis=0)
    circ = circ_1_level_blocks(out, L, M, N) if on_off != "off" else None
    return circ, out


def _toeplitz(col, row):
    """MATLAB toeplitz(c, r): T(i,j) = c(i-j+1) for i>=j, r(j-i+1) for j>i."""
    col = np.asarray(col); row = np.asarray(row)
    n = len(col); m = len(row)
    i = np.arange(n)[:, None]; j = np.arange(m)[None, :]
    return np.where(i >= j, col[np.clip(i - j, 0, n - 1)], row[np.clip(j - i, 0, m - 1)])


def circ_1_level_blocks(circL, L, M, N):
    """Dense 1-level blocks, circ_1_level.m:181-257 (serial branch).  Returns
    (L, 3MN, 3MN); rows/cols ordered (y, z, comp) with y fastest."""
    MN = M * N
    blocks = np.zeros((L, 3 * MN, 3 * MN), dtype=complex)
    zt = np.abs(np.arange(N)[:, None] - np.arange(N)[None, :])

    def blk(c, i_loop, negcol):
        chans = []
        for k in range(N):
            v = circL[i_loop, :, k, c]
            colv = np.concatenate([v[:1], -v[1:]]) if negcol else v
            chans.append(_toeplitz(colv, v))
        return np.block([[chans[zt[p, q]] for q in range(N)] for p in range(N)])

    for i_loop in range(L):
        t = np.zeros((3 * MN, 3 * MN), dtype=complex)
        t[:MN, :MN] = blk(0, i_loop, False)
        r2 = blk(1, i_loop, True)
        t[:MN, MN:2 * MN] = r2; t[MN:2 * MN, :MN] = r2
        r3 = blk(2, i_loop, False)
        U = np.triu(r3); r3 = U - U.T + np.diag(np.diag(U))
        t[:MN, 2 * MN:] = r3; t[2 * MN:, :MN] = r3
        t[MN:2 * MN, MN:2 * MN] = blk(3, i_loop, False)
        r5 = blk(4, i_loop, True)
        U = np.triu(r5); r5 = U + U.T - np.diag(np.diag(U))
        t[MN:2 * MN, 2 * MN:] = r5; t[2 * MN:, MN:2 * MN] = r5
        t[2 * MN:, 2 * MN:] = blk(5, i_loop, False)
        blocks[i_loop] = t
    return blocks


def circ_2_level(circ_L_opToep, L, M, N):
    """[circ_M_opToep, circ] = circ_2_level(...), circ_2_level.m:1-155.
    ``circ`` is returned as an (L, M, 3N, 3N) array (the reference's cell{L,M});
    rows/cols ordered (z, comp) with z fastest."""
    C = np.asarray(circ_L_opToep, dtype=complex)
    lev2 = np.zeros((L, M, N, 6), dtype=complex)
    for c in range(6):
        lev2[..., c] = _F.fft(_chan_average(np.moveaxis(C[..., c], 1, 0), _S2[c]), axis=0).swapaxes(0, 1)
    circ_M = lev2 * np.array(_STORE2)[None, None, None, :]
    blocks = np.zeros((L, M, 3 * N, 3 * N), dtype=complex)
    for i in range(L):
        for j in range(M):
            cc, CC, CC3, C4, C5, C6 = (lev2[i, j, :, c] for c in range(6))
            t = np.zeros((3 * N, 3 * N), dtype=complex)
            t[:N, :N] = _toeplitz(cc, cc)
            b2 = _toeplitz(CC, CC)
            t[:N, N:2 * N] = b2; t[N:2 * N, :N] = b2
            b3 = _toeplitz(np.concatenate([CC3[:1], -CC3[1:]]), CC3)
            t[:N, 2 * N:] = b3; t[2 * N:, :N] = b3
            t[N:2 * N, N:2 * N] = _toeplitz(C4, C4)
            b5 = _toeplitz(np.concatenate([C5[:1], -C5[1:]]), C5)
            t[N:2 * N, 2 * N:] = b5; t[2 * N:, N:2 * N] = b5
            t[2 * N:, 2 * N:] = _toeplitz(C6, C6)
            blocks[i, j] = t
    return circ_M, blocks


def invert_blocks(blocks, shift, diag):
    """inv(shift*I - diag(d)*C) for every block: main_DDA.m:109 with
    shift=1/alpha_LDR, d=dV; scatteringHumanHead.m:181-182 with shift=Gram and
    d=face3_2 (a 3N vector)."""
    n = blocks.shape[-1]
    d = np.broadcast_to(np.asarray(diag, dtype=complex), (n,))
    A = np.asarray(shift, dtype=complex) * np.eye(n) - d[:, None] * blocks
    return np.linalg.inv(A)


def mvp_circ_2_level(inv_blocks, JIn, L, M, N, idx):
    """mvp = mvp_circ_2_level(inv_blocks, JIn, L, M, N, idx), mvp_circ_2_level.m:1-23.
    ``idx`` is 0-based into the column-major (L,M,N,3) grid."""
    V = np.zeros(3 * L * M * N, dtype=complex)
    V[np.asarray(idx)] = np.asarray(JIn, dtype=complex).ravel()
    V = V.reshape((L, M, N, 3), order="F")
    V = _F.fft(_F.fft(V, axis=0), axis=1)
    vec = V.transpose(0, 1, 3, 2).reshape(L, M, 3 * N)  # index comp*N + z
    out = np.einsum("ijab,ijb->ija", inv_blocks, vec)
    V = out.reshape(L, M, 3, N).transpose(0, 1, 3, 2)
    V = _F.ifft(_F.ifft(V, axis=1), axis=0)
    return V.ravel(order="F")[np.asarray(idx)]


def chan_mvp_idx(inv_blocks, JIn, L, M, N, idx):
    """1-level apply, chan_mvp_idx.m:1-17; ``inv_blocks`` is (L, 3MN, 3MN)."""
    V = np.zeros(3 * L * M * N, dtype=complex)
    V[np.asarray(idx)] = np.asarray(JIn, dtype=complex).ravel()
    temp = _F.fft(V.reshape((L, 3 * M * N), order="F"), axis=0)
    temp = np.einsum("iab,ib->ia", inv_blocks, temp)
    temp = _F.ifft(temp, axis=0)
    return temp.ravel(order="F")[np.asarray(idx)]


def eps_layer_average(eps_r):
    """face3_2 of scatteringHumanHead.m:157-177: average eps_r over x, then over
    y, per z layer; (t - 1)/t repeated for the three components."""
    e = np.asarray(eps_r, dtype=complex)
    hey = e.sum(axis=0) / e.shape[0]          # (M, N): sum(epsilon_r, 1) ./ L
    kk = hey.sum(axis=0) / e.shape[1]         # (N,): sum(er_av_x, 2) ./ M
    face_2 = (kk - 1) / kk
    return np.concatenate([face_2, face_2, face_2])
