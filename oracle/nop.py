"""Galerkin N-operator (JVIE) Toeplitz assembly, far and medium cells.  FP64
restatement (test infrastructure only).

Follows src/src_vie/src_operators/assembly_nop_const.m:1-174:
* cube_faces.m:1-50           -- the 6 faces of the voxel [0,dx]^3 (4 vertices each)
* cubatures/gauss_2d.m:1-20   -- tensor Gauss-Legendre rule on [0,1]^2 (gauss_1d.m)
* mexcubatures/cubature_nop_const.cpp:8-124 -- 4-D face-pair cubature of
  exp(-i ko R)/R over the 21 distinct face pairs, scaled by dx^4
* vector_projection.m:1-30    -- P(k,l,c) = (k x e_a).(l x e_b) for the 6 components
* assembly_nop_const.m:44-92  -- far cells (4x4 rule) everywhere, then the
  medium cells (offset < 5 per axis) again with the 10x10 rule
* assembly_nop_const.m:150-165 -- G(:,:,:,c) = sum_kl J(:,:,:,k,l) P(k,l,c) / (4 pi)
The near cells (offsets < 2 per axis) need the singular DIRECTFN/DEMCEM
corrections (assembly_nop_const.m:94-146); they are taken from the caller
(``near_J``), as the GPU entry point does, and are zero without it.

``reference_cubature()`` binds the reference's own cubature_nop, compiled from
its source by oracle/build_ref.py, which pins ``cubature_nop`` here.
"""
import ctypes

import numpy as np

# cubature_nop_const.cpp:32-35: the 21 distinct (observation, source) face pairs
_OBS = [0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 4, 4, 5]
_SRC = [0, 1, 2, 3, 4, 5, 0, 2, 3, 4, 5, 2, 3, 4, 5, 2, 4, 5, 4, 5, 4]
# cubature_nop_const.cpp:100-118: the remaining entries copied from those
_COPIES = [((1, 1), (0, 0)), ((2, 0), (1, 3)), ((2, 1), (0, 3)), ((3, 0), (1, 2)), ((3, 1), (0, 2)),
           ((3, 3), (2, 2)), ((4, 0), (1, 5)), ((4, 1), (0, 5)), ((4, 2), (3, 5)), ((4, 3), (2, 5)),
           ((5, 0), (1, 4)), ((5, 1), (0, 4)), ((5, 2), (3, 4)), ((5, 3), (2, 4)), ((5, 5), (4, 4))]

NP_FAR, NP_MEDIUM, N_MEDIUM = 4, 10, 5  # assembly_nop_const.m:20-26


def cube_faces(dx, dy=None, dz=None):
    """R_faces[coord, vertex, face] (cube_faces.m:1-50): faces -x,+x,-y,+y,-z,+z."""
    dy = dx if dy is None else dy
    dz = dx if dz is None else dz
    F = np.array([
        [[0, 0, 0], [0, dy, 0], [0, dy, dz], [0, 0, dz]],
        [[dx, 0, 0], [dx, dy, 0], [dx, dy, dz], [dx, 0, dz]],
        [[0, 0, 0], [dx, 0, 0], [dx, 0, dz], [0, 0, dz]],
        [[0, dy, 0], [dx, dy, 0], [dx, dy, dz], [0, dy, dz]],
        [[0, 0, 0], [dx, 0, 0], [dx, dy, 0], [0, dy, 0]],
        [[0, 0, dz], [dx, 0, dz], [dx, dy, dz], [0, dy, dz]]], dtype=float)  # [face, vertex, coord]
    return np.transpose(F, (2, 1, 0)).copy()


def gauss_2d(n):
    """(w, u, v) of the n*n tensor Gauss-Legendre rule on [0,1]^2, point I*n+J
    = (x_I, x_J) (gauss_2d.m:1-20)."""
    x, w = np.polynomial.legendre.leggauss(n)
    W = (np.outer(w, w) / 4.0).ravel()
    U = np.repeat((x + 1) / 2, n)
    V = np.tile((x + 1) / 2, n)
    return W, U, V


def cubature_nop(W, U, V, r_m, r_n, R_faces, ko, dx):
    """I_mn[6,6] (cubature_nop_const.cpp:8-124)."""
    I = np.zeros((6, 6), dtype=complex)
    r_m = np.asarray(r_m, float)
    r_n = np.asarray(r_n, float)
    for po, ps in zip(_OBS, _SRC):
        p1, p2, p4 = R_faces[:, 0, po], R_faces[:, 1, po], R_faces[:, 3, po]
        q1, q2, q4 = R_faces[:, 0, ps], R_faces[:, 1, ps], R_faces[:, 3, ps]
        rp = p1[None, :] + np.outer(U, p2 - p1) + np.outer(V, p4 - p1) + r_m[None, :]
        rq = q1[None, :] + np.outer(U, q2 - q1) + np.outer(V, q4 - q1) + r_n[None, :]
        R = np.sqrt(((rq[None, :, :] - rp[:, None, :]) ** 2).sum(-1))
        I[po, ps] = (np.outer(W, W) * np.exp(-1j * ko * R) / R).sum()
    for (a, b), (c, d) in _COPIES:
        I[a, b] = I[c, d]
    return dx ** 4 * I


def vector_projection():
    """P[k, l, comp] (vector_projection.m:1-30)."""
    e = np.eye(3)
    KL = np.array([-e[0], e[0], -e[1], e[1], -e[2], e[2]])
    pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    P = np.zeros((6, 6, 6))
    for k in range(6):
        for l in range(6):
            for c, (a, b) in enumerate(pairs):
                P[k, l, c] = np.dot(np.cross(KL[k], e[a]), np.cross(KL[l], e[b]))
    return P


def near_extent(L, M, N):
    """Extent of the near block: offsets < 2 per axis within the grid."""
    return min(2, L), min(2, M), min(2, N)


def assembly_nop(L, M, N, ko, dx, near_J=None, cubature=None):
    """G_mn (L, M, N, 6) of assembly_nop_const.m with the near block (offsets < 2
    per axis, ``near_extent``) taken from near_J (near_extent + (6, 6)), or zero
    without it.  ``cubature`` replaces cubature_nop (same signature)."""
    cub = cubature or cubature_nop
    Rf = cube_faces(dx)
    J = np.zeros((L, M, N, 6, 6), dtype=complex)
    rn = np.zeros(3)
    a, b, c = near_extent(L, M, N)
    near = lambda mx, my, mz: mx < a and my < b and mz < c  # noqa: E731  (replaced below)
    W, U, V = gauss_2d(NP_FAR)
    for mx in range(L):
        for my in range(M):
            for mz in range(N):
                if not near(mx, my, mz):
                    J[mx, my, mz] = cub(W, U, V, np.array([mx, my, mz]) * dx, rn, Rf, ko, dx)
    W, U, V = gauss_2d(NP_MEDIUM)
    for mx in range(min(N_MEDIUM, L)):
        for my in range(min(N_MEDIUM, M)):
            for mz in range(min(N_MEDIUM, N)):
                if not near(mx, my, mz):
                    J[mx, my, mz] = cub(W, U, V, np.array([mx, my, mz]) * dx, rn, Rf, ko, dx)
    J[:a, :b, :c] = 0 if near_J is None else np.asarray(near_J).reshape(a, b, c, 6, 6)
    P = vector_projection()
    return np.einsum("xyzkl,klc->xyzc", J, P) / (4 * np.pi)


def reference_cubature():
    """The reference's cubature_nop (same signature as ``cubature_nop``), or None
    when it cannot be compiled here (no reference checkout or no g++)."""
    from oracle import build_ref
    path = build_ref.build()
    if path is None:
        return None
    lib = ctypes.CDLL(path)
    dp = ctypes.POINTER(ctypes.c_double)
    lib.ref_cubature_nop.argtypes = [ctypes.c_int, dp, dp, dp, dp, dp, dp, ctypes.c_double, ctypes.c_double, dp]
    lib.ref_cubature_nop.restype = None

    def p(a):
        return a.ctypes.data_as(dp)

    def cub(W, U, V, r_m, r_n, R_faces, ko, dx):
        W, U, V = (np.ascontiguousarray(a, dtype=float) for a in (W, U, V))
        rm = np.ascontiguousarray(r_m, dtype=float)
        rn = np.ascontiguousarray(r_n, dtype=float)
        F = np.asfortranarray(R_faces, dtype=float).ravel(order="F")
        out = np.zeros(72)
        lib.ref_cubature_nop(len(W), p(W), p(U), p(V), p(rm), p(rn), p(F), float(ko), float(dx), p(out))
        return (out[0::2] + 1j * out[1::2]).reshape(6, 6, order="F")
    return cub
