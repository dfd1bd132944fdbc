"""Host-side mirror of the reference's MATLAB interface on libvoxscatter.

Function names, argument order and meaning follow the reference:
  getOPERATOR_DDA   src/src_vie/src_operators/getOPERATOR_DDA.m:1-2
  MVP / mv_AN_const src/src_vie/src_mvp/MVP.m:1
  circ_1_level      src/src_preconditioning/circ_1_level.m:1
  circ_2_level      src/src_preconditioning/circ_2_level.m:1
  mvp_circ_2_level  src/src_preconditioning/mvp_circ_2_level.m:2
  bicgstab          MATLAB bicgstab as called at main_DDA.m:82,120-121
Indices are 0-based (MATLAB idx - 1).  The long-lived objects (Context,
Operator) are the handle-based fast path; the MATLAB-named functions build
them per call, as the reference's handles re-pass fN on every call.
"""
import ctypes as C

import numpy as np

from . import _lib as L


class Context:
    """A CUDA device + stream owned by libvoxscatter."""

    def __init__(self, device=0):
        self._lib = L.load()
        h = C.c_void_p()
        L.check(self._lib.vs_ctx_create(int(device), C.byref(h)))
        self.h = h
        self.device = device

    def synchronize(self):
        L.check(self._lib.vs_ctx_synchronize(self.h), self.h)

    def stream_ptr(self):
        """The context's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        ptr = C.c_void_p()
        L.check(self._lib.vs_ctx_stream(self.h, C.byref(ptr)), self.h)
        return ptr.value or 0

    def close(self):
        if getattr(self, "h", None):
            self._lib.vs_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _offsets(r):
    r = np.asarray(r, dtype=float)
    ox = np.ascontiguousarray(r[:, 0, 0, 0] - r[0, 0, 0, 0])
    oy = np.ascontiguousarray(r[0, :, 0, 1] - r[0, 0, 0, 1])
    oz = np.ascontiguousarray(r[0, 0, :, 2] - r[0, 0, 0, 2])
    return ox, oy, oz


def green_dda(r, ko, nearby_quad="off", ctx=None):
    """Toep (L,M,N,6) on the device in FP64 (getOPERATOR_DDA.m:29-119)."""
    ctx = ctx or default_context()
    Lx, My, Nz = np.asarray(r).shape[:3]
    ox, oy, oz = _offsets(r)
    out = np.zeros(Lx * My * Nz * 6, dtype=np.complex128)
    L.check(ctx._lib.vs_green_dda(ctx.h, Lx, My, Nz, L.dptr(ox), L.dptr(oy), L.dptr(oz), float(ko),
                                  1 if nearby_quad == "on" else 0, L.dptr(out)), ctx.h)
    return out.reshape((Lx, My, Nz, 6), order="F")


def alpha_ldr(m, ko, d, kvec, Eo, is_eps=False):
    """alpha_LDR (getOPERATOR_DDA.m:7-26), elementwise over m (or eps)."""
    lib = L.load()
    arr = np.atleast_1d(np.asarray(m, dtype=np.complex128)).ravel()
    arr = np.ascontiguousarray(arr)
    out = np.zeros_like(arr)
    kv = np.ascontiguousarray(np.asarray(kvec, dtype=float))
    e0 = np.ascontiguousarray(np.asarray(Eo, dtype=float))
    L.check(lib.vs_alpha_ldr(L.dptr(arr), arr.size, 1 if is_eps else 0, float(ko), float(d), L.dptr(kv),
                             L.dptr(e0), L.dptr(out)))
    return out[0] if np.ndim(m) == 0 else out.reshape(np.shape(m))


def eps_layer_average(eps_r):
    """face3 (3N) of the JVIE 2-level preconditioner from the relative
    permittivity grid eps_r (L, M, N): (t - 1)/t with t the x- then y-average of
    each z layer, repeated for the three components (scatteringHumanHead.m:157-177)."""
    lib = L.load()
    e = np.asarray(eps_r, dtype=np.complex128)
    L_, M_, N_ = e.shape
    ef = np.ascontiguousarray(e.ravel(order="F"))
    out = np.zeros(3 * N_, dtype=np.complex128)
    L.check(lib.vs_eps_layer_average(L_, M_, N_, L.dptr(ef), L.dptr(out)))
    return out


def nop_assemble(L_, M_, N_, ko, dx, near_J=None, ctx=None):
    """Galerkin N-operator Toeplitz tensor G (L, M, N, 6) of assembly_nop_const.m
    (far and medium cells on the device); near_J: the singular near block
    (min(2,L), min(2,M), min(2,N), 6, 6) or None (those cells zero)."""
    ctx = ctx or default_context()
    G = np.zeros(L_ * M_ * N_ * 6, dtype=np.complex128)
    nj = None
    if near_J is not None:
        shape = (min(2, L_), min(2, M_), min(2, N_), 6, 6)
        nj = np.ascontiguousarray(np.asarray(near_J, dtype=np.complex128).reshape(shape).ravel(order="F"))
    L.check(ctx._lib.vs_nop_assemble(ctx.h, L_, M_, N_, float(ko), float(dx), L.dptr(nj) if nj is not None else None,
                                     L.dptr(G)), ctx.h)
    return G.reshape((L_, M_, N_, 6), order="F")


def circulant_fft(Toep, P=None, Q=None, R=None, ctx=None):
    """fN = fft_operator(circulant_nop_const(Toep)) for (P,Q,R) = (2L,2M,2N) by default."""
    ctx = ctx or default_context()
    Lx, My, Nz = Toep.shape[:3]
    P = P or 2 * Lx; Q = Q or 2 * My; R = R or 2 * Nz
    t = L.cplx_flat(Toep)
    out = np.zeros(P * Q * R * 6, dtype=np.complex128)
    L.check(ctx._lib.vs_circulant_fft(ctx.h, Lx, My, Nz, L.dptr(t), P, Q, R, L.dptr(out)), ctx.h)
    return out.reshape((P, Q, R, 6), order="F")


def getOPERATOR_DDA(r, ko, refInd, kvec, Eo, nearby_quad="off", ctx=None):
    """[op_out, Toep, alpha_LDR] = getOPERATOR_DDA(r, ko, refInd, kvec, Eo, nearby_quad)."""
    r = np.asarray(r, dtype=float)
    dx = r[1, 0, 0, 0] - r[0, 0, 0, 0]
    Toep = green_dda(r, ko, nearby_quad, ctx)
    fN = circulant_fft(Toep, ctx=ctx)
    return fN, Toep, alpha_ldr(refInd, ko, dx, kvec, Eo)


_TRANSP = {"notransp": L.VS_NOTRANSP, "transp": L.VS_CONJTRANSP, "plain_transp": L.VS_TRANSP}


class Operator:
    """Handle on a device operator A x = Gram.*Mr.*x - Mc.*N(x) on idx3."""

    def __init__(self, L_, M_, N_, idx3, Mr=1.0, Mc=1.0, Gram=1.0, toep=None, fN=None, PQR=(0, 0, 0), ctx=None):
        self.ctx = ctx or default_context()
        lib = self.ctx._lib
        keep = []
        idx = np.ascontiguousarray(np.asarray(idx3, dtype=np.int64).ravel())
        keep.append(idx)
        dMr, dMc, dG = L.make_diag(Mr, keep), L.make_diag(Mc, keep), L.make_diag(Gram, keep)
        h = C.c_void_p()
        if fN is not None:
            P, Q, R = fN.shape[:3]
            f = L.cplx_flat(fN)
            L.check(lib.vs_op_create_fN(self.ctx.h, L_, M_, N_, L.dptr(f), P, Q, R,
                                        idx.ctypes.data_as(L._pi64), idx.size, dMr, dMc, dG, C.byref(h)), self.ctx.h)
        else:
            t = L.cplx_flat(toep)
            L.check(lib.vs_op_create(self.ctx.h, L_, M_, N_, L.dptr(t), int(PQR[0]), int(PQR[1]), int(PQR[2]),
                                     idx.ctypes.data_as(L._pi64), idx.size, dMr, dMc, dG, C.byref(h)), self.ctx.h)
        self.h = h
        self.n3 = idx.size
        lmn = (C.c_int64 * 3)(); pqr = (C.c_int64 * 3)()
        L.check(lib.vs_op_info(h, lmn, pqr, None))
        self.LMN = tuple(lmn); self.PQR = tuple(pqr)

    def apply(self, x, transp_flag="notransp", precision="c64", gram=None):
        """y = A x for nrhs = x.size / n3 right-hand sides.  ``gram``: None (the
        operator's Gram) or one Gram per right-hand side in its place, as an
        (nrhs,) array of scalars or an (nrhs, L, M, N) array of grids (MVP.m
        called with each right-hand side's Gram)."""
        x = np.ascontiguousarray(np.asarray(x, dtype=np.complex128))
        nrhs = x.size // self.n3
        assert nrhs * self.n3 == x.size
        y = np.empty_like(x)
        prec = L.VS_C64 if precision == "c64" else L.VS_C128
        if gram is None:
            L.check(self.ctx._lib.vs_op_apply(self.h, L.dptr(x), L.dptr(y), nrhs, _TRANSP[transp_flag], prec),
                    self.ctx.h)
            return y
        g, gn = _gram_array(gram, nrhs, self.LMN)
        L.check(self.ctx._lib.vs_op_apply_gram(self.h, L.dptr(x), L.dptr(y), nrhs, _TRANSP[transp_flag], prec,
                                               L.dptr(g), gn), self.ctx.h)
        return y

    def apply_device(self, x, y, transp_flag="notransp"):
        """x, y: CUDA torch tensors (complex64 or complex128), n3*nrhs elements."""
        import torch
        prec = L.VS_C64 if x.dtype == torch.complex64 else L.VS_C128
        torch.cuda.synchronize()
        L.check(self.ctx._lib.vs_op_apply_device(self.h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                                 x.numel() // self.n3, _TRANSP[transp_flag], prec), self.ctx.h)
        self.ctx.synchronize()
        return y

    def time_passes(self, x_ptr, y_ptr, nrhs=1, precision="c64", nrep=20):
        """Per-launch milliseconds of the 5 pipeline passes (CUDA events)."""
        out = (C.c_float * 5)()
        L.check(self.ctx._lib.vs_op_time_passes(self.h, C.c_void_p(x_ptr), C.c_void_p(y_ptr), nrhs,
                                                L.VS_C64 if precision == "c64" else L.VS_C128, nrep, out), self.ctx.h)
        return list(out)

    def shape(self, precision="c64"):
        sh = L.vs_shape()
        L.check(self.ctx._lib.vs_op_get_shape(self.h, L.VS_C64 if precision == "c64" else L.VS_C128, C.byref(sh)))
        return dict(lg_lines_x=sh.lg_lines_x, lg_tile_y=sh.lg_tile_y, lg_tile_z=sh.lg_tile_z, z_reg=sh.z_reg,
                    y_reg=sh.y_reg, x_reg=sh.x_reg, z_df=sh.z_df)

    def set_shape(self, precision="c64", **kw):
        cur = self.shape(precision)
        cur.update(kw)
        sh = L.vs_shape(**cur)
        L.check(self.ctx._lib.vs_op_set_shape(self.h, L.VS_C64 if precision == "c64" else L.VS_C128, C.byref(sh)),
                self.ctx.h)

    def close(self):
        if getattr(self, "h", None):
            self.ctx._lib.vs_op_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _gram_array(gram, nrhs, LMN):
    """(flat complex array, entries per right-hand side) of a Gram per
    right-hand side: nrhs scalars, or nrhs column-major (L, M, N) grids."""
    g = np.asarray(gram, dtype=np.complex128)
    V = int(np.prod(LMN))
    if g.size == nrhs:
        return np.ascontiguousarray(g.ravel()), 1
    if g.size == nrhs * V:
        flat = np.ascontiguousarray(g.reshape(nrhs, -1, order="C") if g.ndim == 2 else
                                    np.stack([gi.ravel(order="F") for gi in g.reshape((nrhs,) + tuple(LMN))]))
        return flat.ravel(), V
    raise ValueError(f"gram must hold {nrhs} scalars or {nrhs} grids of {LMN}")


def MVP(JIn0, fN, Mr, Mc, Gram, transp_flag, idx, GPU_flag=1, precision="c128", ctx=None):
    """JOut = MVP(JIn0, fN, Mr, Mc, Gram, transp_flag, idx, GPU_flag) (MVP.m:1).
    The device pipeline runs in ``precision`` ('c128' matches the reference's
    FP64; 'c64' is the mixed-precision inner kernel)."""
    Mr = np.asarray(Mr)
    L_, M_, N_ = Mr.shape
    op = Operator(L_, M_, N_, idx, Mr, Mc, Gram, fN=np.asarray(fN), ctx=ctx)
    try:
        return op.apply(JIn0, transp_flag, precision)
    finally:
        op.close()


mv_AN_const = MVP


def _precisions(precisions):
    m = 0
    for p in precisions:
        m |= L.VS_BUILD_C64 if p == "c64" else L.VS_BUILD_C128
    return m


def circ_levels(opToeplitz, Lx, My, Nz, want_blocks=True, ctx=None):
    """(circ_L_opToep, circ_M_opToep, blocks[L,M,3N,3N]) computed on the device."""
    ctx = ctx or default_context()
    t = L.cplx_flat(opToeplitz)
    V = Lx * My * Nz
    c1 = np.zeros(6 * V, dtype=np.complex128)
    c2 = np.zeros(6 * V, dtype=np.complex128)
    n = 3 * Nz
    blk = np.zeros(Lx * My * n * n, dtype=np.complex128) if want_blocks else None
    L.check(ctx._lib.vs_circ_levels(ctx.h, Lx, My, Nz, L.dptr(t), L.dptr(c1), L.dptr(c2),
                                    L.dptr(blk) if want_blocks else None), ctx.h)
    shp = (Lx, My, Nz, 6)
    blocks = None
    if want_blocks:
        # block b = i + L*j, each column-major n x n  ->  [i, j, p, q]
        blocks = blk.reshape(My, Lx, n, n).transpose(1, 0, 3, 2)
    return c1.reshape(shp, order="F"), c2.reshape(shp, order="F"), blocks


def circ_1_level(opToeplitz, Lx, My, Nz, parallel_prec=0, on_off="off", ctx=None):
    """[circ, circ_L_opToep] = circ_1_level(...) with on_off = 'off' (circ_1_level.m:1-93)."""
    if on_off != "off":
        raise NotImplementedError("dense 1-level blocks (on_off='on') are not built on the device")
    c1, _, _ = circ_levels(opToeplitz, Lx, My, Nz, want_blocks=False, ctx=ctx)
    return None, c1


def circ_2_level(circ_L_opToep, Lx, My, Nz, opToeplitz=None, ctx=None):
    """[circ_M_opToep, circ] = circ_2_level(circ_L_opToep, L, M, N).

    The device pipeline starts from the Toeplitz tensor (both levels in one
    call); pass it as ``opToeplitz``.  ``circ`` is returned as an
    (L, M, 3N, 3N) array (the reference's cell{L,M})."""
    if opToeplitz is None:
        raise ValueError("the device path needs the Toeplitz tensor (opToeplitz=...)")
    _, c2, blocks = circ_levels(opToeplitz, Lx, My, Nz, want_blocks=True, ctx=ctx)
    return c2, blocks


class Preconditioner:
    """Handle on a device 2-level circulant preconditioner (y = M^-1 x)."""

    def __init__(self, op=None, shift=None, d=None, inv_blocks=None, LMN=None, idx3=None,
                 precisions=("c64", "c128"), ctx=None, lu="auto"):
        """lu: how the FP32 blocks are inverted -- "auto" (shared-memory kernel up
        to 3N = 168, tensor cores up to 256, then CUDA cores), "tc" (tcgen05
        trailing updates, 3N <= 256) or "cuda" (CUDA-core kernels)."""
        h = C.c_void_p()
        mask = _precisions(precisions) | {"auto": 0, "tc": L.VS_BUILD_LU_TC, "cuda": L.VS_BUILD_LU_CUDA}[lu]
        if op is not None:
            self.ctx = op.ctx
            sh = np.array([complex(shift)], dtype=np.complex128)
            dd = np.ascontiguousarray(np.atleast_1d(np.asarray(d, dtype=np.complex128)).ravel())
            L.check(self.ctx._lib.vs_prec_create(op.h, L.dptr(sh), L.dptr(dd), dd.size, mask, C.byref(h)), self.ctx.h)
            self.n3 = op.n3
        else:
            self.ctx = ctx or default_context()
            Lx, My, Nz = LMN
            n = 3 * Nz
            # [i, j, p, q] -> block i + L*j, column-major
            flat = np.ascontiguousarray(np.asarray(inv_blocks, dtype=np.complex128).transpose(1, 0, 3, 2).ravel())
            idx = np.ascontiguousarray(np.asarray(idx3, dtype=np.int64).ravel())
            L.check(self.ctx._lib.vs_prec_create_blocks(self.ctx.h, Lx, My, Nz, L.dptr(flat),
                                                        idx.ctypes.data_as(L._pi64), idx.size, mask, C.byref(h)),
                    self.ctx.h)
            self.n3 = idx.size
        self.h = h

    def apply(self, x, precision="c64"):
        x = np.ascontiguousarray(np.asarray(x, dtype=np.complex128))
        nrhs = x.size // self.n3
        y = np.empty_like(x)
        L.check(self.ctx._lib.vs_prec_apply(self.h, L.dptr(x), L.dptr(y), nrhs,
                                            L.VS_C64 if precision == "c64" else L.VS_C128), self.ctx.h)
        return y

    def time_passes(self, x_ptr, y_ptr, nrhs=1, precision="c64", nrep=20):
        out = (C.c_float * 5)()
        L.check(self.ctx._lib.vs_prec_time_passes(self.h, C.c_void_p(x_ptr), C.c_void_p(y_ptr), nrhs,
                                                  L.VS_C64 if precision == "c64" else L.VS_C128, nrep, out),
                self.ctx.h)
        return list(out)

    def shape(self, precision="c64"):
        sh = L.vs_prec_shape()
        L.check(self.ctx._lib.vs_prec_get_shape(self.h, L.VS_C64 if precision == "c64" else L.VS_C128,
                                                C.byref(sh)))
        return dict(lg_lines_x=sh.lg_lines_x, lg_tile_y=sh.lg_tile_y, gemv_blocks=sh.gemv_blocks,
                    gemv_threads=sh.gemv_threads, gemv_mode=sh.gemv_mode, gemv_chunk=sh.gemv_chunk, y_reg=sh.y_reg,
                    x_reg=sh.x_reg, fuse_xy=sh.fuse_xy, wait_polls=sh.wait_polls)

    def set_shape(self, precision="c64", **kw):
        cur = self.shape(precision)
        cur.update(kw)
        sh = L.vs_prec_shape(**cur)
        L.check(self.ctx._lib.vs_prec_set_shape(self.h, L.VS_C64 if precision == "c64" else L.VS_C128,
                                                C.byref(sh)), self.ctx.h)

    def blocks(self, Lx, My, Nz, precision="c128"):
        n = 3 * Nz
        out = np.zeros(Lx * My * n * n, dtype=np.complex128)
        L.check(self.ctx._lib.vs_prec_get_blocks(self.h, L.VS_C64 if precision == "c64" else L.VS_C128,
                                                 L.dptr(out)), self.ctx.h)
        return out.reshape(My, Lx, n, n).transpose(1, 0, 3, 2)

    def close(self):
        if getattr(self, "h", None):
            self.ctx._lib.vs_prec_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def invert_blocks_device(mats_ptr, n, nmat, method="auto", ctx=None):
    """In-place FP32 inversion of nmat complex n x n matrices at the device
    address mats_ptr (complex64, either storage order): "auto" (tensor cores
    for n <= 256, else CUDA cores), "tc" or "cuda"."""
    ctx = ctx or default_context()
    code = {"auto": 0, "tc": L.VS_BUILD_LU_TC, "cuda": L.VS_BUILD_LU_CUDA}[method]
    L.check(ctx._lib.vs_invert_blocks_device(ctx.h, C.c_void_p(mats_ptr), int(n), int(nmat), code), ctx.h)


def mvp_circ_2_level(inv_blocks, JIn, Lx, My, Nz, idx, precision="c128", ctx=None):
    """mvp = mvp_circ_2_level(inv_blocks, JIn, L, M, N, idx) with inv_blocks as an
    (L, M, 3N, 3N) array."""
    pr = Preconditioner(inv_blocks=inv_blocks, LMN=(Lx, My, Nz), idx3=idx,
                        precisions=(precision,), ctx=ctx)
    try:
        return pr.apply(JIn, precision)
    finally:
        pr.close()


_METHODS = {"bicgstab": L.VS_BICGSTAB, "gmres": L.VS_GMRES, "gmres_dr": L.VS_GMRES_DR}


def _method(name):
    if name not in _METHODS:
        raise ValueError(f"unknown method {name!r}; expected one of {sorted(_METHODS)}")
    return _METHODS[name]


def solve(op, b, prec=None, tol=1e-6, maxit=2000, precision="mixed", x0=None, inner_tol=0.0, max_refine=10,
          iters_per_graph=4, want_resvec=True, transpose=False, method="bicgstab", restart=50, ritz=10, gram=None):
    """Device Krylov solve; returns (x, info dict, resvec).  ``gram``: None or
    this solve's Gram in place of the operator's (a scalar or an (L, M, N) grid)."""
    lib = op.ctx._lib
    b = np.ascontiguousarray(np.asarray(b, dtype=np.complex128).ravel())
    x = np.zeros_like(b) if x0 is None else np.ascontiguousarray(np.asarray(x0, dtype=np.complex128).ravel()).copy()
    o = L.vs_solve_opts()
    lib.vs_solve_opts_default(C.byref(o))
    o.precision = L.VS_SOLVE_MIXED if precision == "mixed" else L.VS_SOLVE_FP64
    o.tol = float(tol); o.maxit = int(maxit); o.inner_tol = float(inner_tol); o.max_refine = int(max_refine)
    o.iters_per_graph = int(iters_per_graph)
    o.transpose = 1 if transpose else 0
    o.method = _method(method)
    o.restart = int(restart)
    o.ritz = int(ritz)
    rv = np.zeros(4 * int(maxit) + 64 if want_resvec else 1)
    if want_resvec:
        o.resvec = L.dptr(rv); o.resvec_cap = rv.size
    if gram is not None:
        g, o.gram_n = _gram_array(gram, 1, op.LMN)
        o.gram = L.dptr(g)
    info = L.vs_solve_info()
    L.check(lib.vs_solve(op.h, prec.h if prec is not None else None, L.dptr(b), L.dptr(x), C.byref(o),
                         C.byref(info)), op.ctx.h)
    d = dict(flag=info.flag, relres=info.relres, iter=info.iter, refinements=info.refinements,
             time_ms=info.time_ms, launches=info.kernel_launches)
    return x, d, rv[:info.n_resvec].copy()


PROFILE_KEYS = ("prec_x_fwd", "prec_y_fwd", "prec_gemv", "prec_y_inv", "prec_x_inv",
                "mv_x_fwd", "mv_y_fwd", "mv_z", "mv_y_inv", "mv_x_inv")


def solve_device(op, b_ptr, x_ptr, prec=None, tol=1e-6, maxit=2000, precision="mixed", inner_tol=0.0,
                 max_refine=10, iters_per_graph=4, method="bicgstab", restart=50, ritz=10, profile=False,
                 fold=True):
    """vs_solve_device on device buffers (double2, n3 each); returns the info
    dict.  profile=True (BiCGSTAB) adds "profile": the in-solve durations of
    vs_solve_opts.profile_ms in ms (each pass, the solver's kernels per
    iteration, the FP64 residual per call) and the counts they average over.
    fold=False keeps BiCGSTAB's vector steps as separate kernels
    (vs_solve_opts.unfused)."""
    lib = op.ctx._lib
    o = L.vs_solve_opts()
    lib.vs_solve_opts_default(C.byref(o))
    o.precision = L.VS_SOLVE_MIXED if precision == "mixed" else L.VS_SOLVE_FP64
    o.tol = float(tol); o.maxit = int(maxit); o.inner_tol = float(inner_tol); o.max_refine = int(max_refine)
    o.iters_per_graph = int(iters_per_graph)
    o.method = _method(method)
    o.restart = int(restart)
    o.ritz = int(ritz)
    o.unfused = 0 if fold else 1
    prof = (C.c_float * 16)() if profile else None
    if profile:
        o.profile_ms = C.cast(prof, C.POINTER(C.c_float))
    info = L.vs_solve_info()
    L.check(lib.vs_solve_device(op.h, prec.h if prec is not None else None, C.c_void_p(b_ptr), C.c_void_p(x_ptr),
                                C.byref(o), C.byref(info)), op.ctx.h)
    out = dict(flag=info.flag, relres=info.relres, iter=info.iter, refinements=info.refinements,
               time_ms=info.time_ms, launches=info.kernel_launches)
    if profile:
        p = list(prof)
        out["profile"] = dict(zip(PROFILE_KEYS, p[:10]), solver_kernels_per_iter=p[10], iterations=int(p[11]),
                              fp64_residual=p[12], fp64_residual_calls=int(p[13]))
    return out


def solve_host_ptr(op, b_ptr, x_ptr, prec=None, tol=1e-6, maxit=2000, precision="mixed", iters_per_graph=4,
                   method="bicgstab", restart=50, ritz=10):
    """vs_solve on host buffers given as raw pointers (e.g. pinned torch tensors)."""
    lib = op.ctx._lib
    o = L.vs_solve_opts()
    lib.vs_solve_opts_default(C.byref(o))
    o.precision = L.VS_SOLVE_MIXED if precision == "mixed" else L.VS_SOLVE_FP64
    o.tol = float(tol); o.maxit = int(maxit); o.iters_per_graph = int(iters_per_graph)
    o.method = _method(method)
    o.restart = int(restart)
    o.ritz = int(ritz)
    info = L.vs_solve_info()
    L.check(lib.vs_solve(op.h, prec.h if prec is not None else None, C.cast(C.c_void_p(b_ptr), L._pd),
                         C.cast(C.c_void_p(x_ptr), L._pd), C.byref(o), C.byref(info)), op.ctx.h)
    return dict(flag=info.flag, relres=info.relres, iter=info.iter, refinements=info.refinements,
                time_ms=info.time_ms, launches=info.kernel_launches)


def gmres(A, b, restart=None, tol=1e-6, maxit=None, M1=None, M2=None, x0=None, precision="mixed"):
    """[x, flag, relres, iter, resvec] = gmres(A, b, restart, tol, maxit, M1, M2, x0)
    with A an Operator and M1 a Preconditioner.  Left preconditioned and
    restarted like MATLAB's gmres; iter = [outer, inner]; resvec holds the
    preconditioned residual norms relative to ||M^-1 b|| scaled to ||b||.
    relres is the true FP64 relative residual."""
    if M2 is not None:
        raise NotImplementedError("a second preconditioner factor is not supported")
    n = A.n3
    restart = n if restart is None else min(int(restart), n)
    maxit = min(int(np.ceil(n / restart)), 10) if maxit is None else int(maxit)
    total = min(restart * maxit, 1 << 30)
    x, info, rv = solve(A, b, prec=M1, tol=tol, maxit=total, precision=precision, x0=x0, method="gmres",
                        restart=min(restart, 2048))
    steps = int(info["iter"])
    outer = max(1, -(-steps // restart))
    inner = steps - (outer - 1) * restart
    nb = np.linalg.norm(np.asarray(b))
    return x, info["flag"], info["relres"], [outer, inner], rv * nb


def pgmresDR(A, b, restart=50, tol=1e-3, maxit=10, ritz=None, L1=None, L2=None, R1=None, R2=None, x0=None,
             precision="mixed"):
    """[x, flag, relres, iter, resvec] = pgmresDR(A, b, restart, tol, maxit, ritz, L1, L2, R1, R2, x0)
    (src/src_numeric/src_iterative/pgmresDR.m:73) with A an Operator and R1 a
    Preconditioner (right preconditioning, as JVIE_Solver_const_GPU.m:400-427
    passes it).  GCRO-DR on the device: every cycle of ``restart`` Arnoldi
    steps recycles the ``ritz`` harmonic Ritz vectors of smallest magnitude;
    ``maxit`` counts the cycles after the first, as pgmresDR.m does.  iter =
    [steps of the last cycle, cycles after the first] (with precision "mixed"
    these count the Arnoldi steps of all refinement solves together); resvec
    holds the Arnoldi residual estimates relative to ||b||; relres is the
    true FP64 relative residual.  Left preconditioners and a second right factor are
    not supported."""
    if L1 is not None or L2 is not None or R2 is not None:
        raise NotImplementedError("pgmresDR here takes the preconditioner as R1 only")
    ritz = min(10, int(round(restart / 2))) if ritz is None else min(int(ritz), int(restart) - 1)
    total = int(restart) * (int(maxit) + 1)
    x, info, rv = solve(A, b, prec=R1, tol=tol, maxit=total, precision=precision, x0=x0, method="gmres_dr",
                        restart=int(restart), ritz=ritz)
    steps = int(info["iter"])
    cycles = max(1, -(-steps // int(restart)))
    last = steps - (cycles - 1) * int(restart)
    return x, info["flag"], info["relres"], [last, cycles - 1], rv


def bicgstab(A, b, tol=1e-6, maxit=20, M1=None, M2=None, x0=None, precision="mixed"):
    """[x, flag, relres, iter, resvec] = bicgstab(A, b, tol, maxit, M1, M2, x0)
    with A an Operator and M1 a Preconditioner (M2 must be None).  resvec holds
    absolute residual norms at every half step, like MATLAB's."""
    if M2 is not None:
        raise NotImplementedError("a second preconditioner factor is not supported")
    x, info, rv = solve(A, b, prec=M1, tol=tol, maxit=maxit, precision=precision, x0=x0)
    nb = np.linalg.norm(np.asarray(b))
    return x, info["flag"], info["relres"], info["iter"], rv * nb


def _solve_opts(lib, tol, maxit, precision):
    o = L.vs_solve_opts()
    lib.vs_solve_opts_default(C.byref(o))
    o.precision = L.VS_SOLVE_MIXED if precision == "mixed" else L.VS_SOLVE_FP64
    o.tol = float(tol)
    o.maxit = int(maxit)
    return o


def plane_wave(op, r, kvec, Eo):
    """Einc(idx3) = PlaneWavePointWise(Eo, kvec, r)(idx3) on the device (FP64)."""
    r = np.asarray(r, dtype=float)
    x = np.ascontiguousarray(r[:, 0, 0, 0]); y = np.ascontiguousarray(r[0, :, 0, 1])
    z = np.ascontiguousarray(r[0, 0, :, 2])
    kv = np.ascontiguousarray(np.asarray(kvec, dtype=float))
    e0 = np.ascontiguousarray(np.asarray(Eo, dtype=np.complex128))
    b = np.zeros(op.n3, dtype=np.complex128)
    L.check(op.ctx._lib.vs_plane_wave(op.h, L.dptr(x), L.dptr(y), L.dptr(z), L.dptr(kv), L.dptr(e0), L.dptr(b)),
            op.ctx.h)
    return b


def cext(op, P, Einc, ko, dV, Eo):
    """Extinction cross section of the polarisation P."""
    P = np.ascontiguousarray(np.asarray(P, dtype=np.complex128))
    E = np.ascontiguousarray(np.asarray(Einc, dtype=np.complex128))
    out = C.c_double()
    L.check(op.ctx._lib.vs_cext(op.h, L.dptr(P), L.dptr(E), float(ko), float(dV),
                                float(np.sum(np.abs(np.asarray(Eo)) ** 2)), C.byref(out)), op.ctx.h)
    return out.value


def _prec_code(precision):
    return {"c64": L.VS_C64, "c128": L.VS_C128}[precision]


def apply_domain(op, x_grid, a, b, precision="c128"):
    """y = a x + b crop(G * x) on every entry of the (L,M,N,3) grid (column-major
    flattening, one right-hand side per row of a 2-D x_grid): the whole-domain
    MVP of main_DDA.m:142-145 (a = 1/alpha, b = -dV) and mv_L_const.m (a = -Gram,
    b = 1) with op's operator spectrum."""
    X = np.ascontiguousarray(np.asarray(x_grid, dtype=np.complex128))
    nrhs = 1 if X.ndim == 1 else X.shape[0]
    Y = np.zeros_like(X)
    av = np.array([complex(a).real, complex(a).imag]); bv = np.array([complex(b).real, complex(b).imag])
    L.check(op.ctx._lib.vs_op_apply_domain(op.h, L.dptr(X), L.dptr(Y), nrhs, L.dptr(av), L.dptr(bv),
                                           _prec_code(precision)), op.ctx.h)
    return Y


def field_dda(op, P, Einc_grid, alpha, dV, chi, precision="c128"):
    """Total field on the whole grid after a DDA solve, main_DDA.m:136-148:
    E = Einc - (Pout/alpha - dV crop(G * Pout)) + Pout/chi with Pout = P on the
    unknowns and 0 elsewhere.  P: n3 (or nrhs x n3); Einc_grid: 3LMN (or
    nrhs x 3LMN), column-major (L,M,N,3).  Returns E in the layout of Einc_grid."""
    Pa = np.ascontiguousarray(np.asarray(P, dtype=np.complex128))
    Ea = np.ascontiguousarray(np.asarray(Einc_grid, dtype=np.complex128))
    nrhs = 1 if Pa.ndim == 1 else Pa.shape[0]
    out = np.zeros_like(Ea)
    al = np.array([complex(alpha).real, complex(alpha).imag]); ch = np.array([complex(chi).real, complex(chi).imag])
    L.check(op.ctx._lib.vs_field_dda(op.h, L.dptr(Pa), L.dptr(Ea), nrhs, L.dptr(al), float(dV), L.dptr(ch),
                                     L.dptr(out), _prec_code(precision)), op.ctx.h)
    return out


def far_field(op, P, r, ko, dV, dirs):
    """Far-field amplitude F(n) = ko^2 dV (I - n n^T) sum_j P_j exp(-i ko n.r_j)
    for the unit directions dirs (ndir x 3); returns (ndir, 3), or (nrhs, ndir, 3)
    for a 2-D P.  E_sca -> exp(i ko r)/r F(n); the optical theorem gives
    C_ext = 4 pi / ko Im(conj(E0).F(k_inc)) / |E0|^2."""
    Pa = np.ascontiguousarray(np.asarray(P, dtype=np.complex128))
    nrhs = 1 if Pa.ndim == 1 else Pa.shape[0]
    r = np.asarray(r, dtype=float)
    x = np.ascontiguousarray(r[:, 0, 0, 0]); y = np.ascontiguousarray(r[0, :, 0, 1])
    z = np.ascontiguousarray(r[0, 0, :, 2])
    D = np.ascontiguousarray(np.asarray(dirs, dtype=float).reshape(-1, 3))
    F = np.zeros((nrhs, D.shape[0], 3), dtype=np.complex128)
    L.check(op.ctx._lib.vs_far_field(op.h, L.dptr(Pa), nrhs, L.dptr(x), L.dptr(y), L.dptr(z), float(ko), float(dV),
                                     L.dptr(D), D.shape[0], L.dptr(F)), op.ctx.h)
    return F[0] if Pa.ndim == 1 else F


def orientation_average(op, prec, m, r, ko, d, dirs, weights=None, psi=None, tol=1e-6, maxit=2000,
                        precision="mixed", method="bicgstab", restart=50):
    """Orientation-averaged C_ext over the orientations (unit incident
    direction dirs[j], polarisation pair turned by psi[j] about it; weights or
    equal weights), two orthogonal linear polarisations each, every incidence
    with its own alpha_LDR; m: refractive index (scalar or one per voxel in idx
    order).  Returns (cext_avg, cext_each (ndir, 2), infos)."""
    lib = op.ctx._lib
    mv = np.ascontiguousarray(np.atleast_1d(np.asarray(m, dtype=np.complex128)).ravel())
    r = np.asarray(r, dtype=float)
    x = np.ascontiguousarray(r[:, 0, 0, 0]); y = np.ascontiguousarray(r[0, :, 0, 1])
    z = np.ascontiguousarray(r[0, 0, :, 2])
    D = np.ascontiguousarray(np.asarray(dirs, dtype=float).reshape(-1, 3))
    nd = D.shape[0]
    wv = None if weights is None else np.ascontiguousarray(np.asarray(weights, dtype=float).ravel())
    pv = None if psi is None else np.ascontiguousarray(np.asarray(psi, dtype=float).ravel())
    o = _solve_opts(lib, tol, maxit, precision)
    o.method = _method(method)
    o.restart = int(restart)
    avg = C.c_double()
    each = np.zeros((nd, 2))
    infos = (L.vs_solve_info * (2 * nd))()
    L.check(lib.vs_orientation_average(op.h, prec.h if prec is not None else None, L.dptr(mv), mv.size, L.dptr(x),
                                       L.dptr(y), L.dptr(z), float(ko), float(d), L.dptr(D),
                                       L.dptr(pv) if pv is not None else None,
                                       L.dptr(wv) if wv is not None else None, nd, C.byref(o), C.byref(avg),
                                       L.dptr(each), infos), op.ctx.h)
    return avg.value, each, [dict(flag=i.flag, relres=i.relres, iter=i.iter) for i in infos]


def cext_grad(op, prec, Einc, eps, ko, d, kvec, Eo, tol=1e-6, maxit=2000, precision="mixed"):
    """(C_ext, dC/dRe(eps), dC/dIm(eps), P, info_fwd, info_adj) by the adjoint method."""
    lib = op.ctx._lib
    E = np.ascontiguousarray(np.asarray(Einc, dtype=np.complex128))
    ep = np.ascontiguousarray(np.asarray(eps, dtype=np.complex128))
    kv = np.ascontiguousarray(np.asarray(kvec, dtype=float))
    e0 = np.ascontiguousarray(np.asarray(Eo, dtype=float))
    o = _solve_opts(lib, tol, maxit, precision)
    c = C.c_double()
    gre = np.zeros(ep.size); gim = np.zeros(ep.size)
    P = np.zeros(op.n3, dtype=np.complex128)
    i1, i2 = L.vs_solve_info(), L.vs_solve_info()
    L.check(lib.vs_cext_grad(op.h, prec.h if prec is not None else None, L.dptr(E), L.dptr(ep), float(ko), float(d),
                             L.dptr(kv), L.dptr(e0), C.byref(o), C.byref(c), L.dptr(gre), L.dptr(gim), L.dptr(P),
                             C.byref(i1), C.byref(i2)), op.ctx.h)
    info = lambda i: dict(flag=i.flag, relres=i.relres, iter=i.iter, time_ms=i.time_ms)
    return c.value, gre, gim, P, info(i1), info(i2)


def solve_batch(op, B, prec=None, tol=1e-6, maxit=2000, precision="mixed", method="bicgstab", restart=50,
                iters_per_graph=4, ritz=10, gram=None, fold=True):
    """Solve A_r x_r = b_r for every row b_r of B (nrhs x n3) as one batch; returns
    (X, list of info dicts).  ``gram``: None (every A_r is the operator) or the
    Gram of each right-hand side (nrhs scalars or nrhs (L, M, N) grids), e.g.
    1/alpha_LDR of each incident direction and polarisation.  fold=False keeps
    BiCGSTAB's vector steps as separate kernels (vs_solve_opts.unfused)."""
    lib = op.ctx._lib
    B = np.ascontiguousarray(np.asarray(B, dtype=np.complex128))
    nrhs = B.shape[0]
    X = np.zeros_like(B)
    o = _solve_opts(lib, tol, maxit, precision)
    o.method = _method(method)
    o.restart = int(restart)
    o.ritz = int(ritz)
    o.iters_per_graph = int(iters_per_graph)
    o.unfused = 0 if fold else 1
    if gram is not None:
        g, o.gram_n = _gram_array(gram, nrhs, op.LMN)
        o.gram = L.dptr(g)
    infos = (L.vs_solve_info * nrhs)()
    L.check(lib.vs_solve_batch(op.h, prec.h if prec is not None else None, L.dptr(B), L.dptr(X), nrhs, C.byref(o),
                               infos), op.ctx.h)
    return X, [dict(flag=i.flag, relres=i.relres, iter=i.iter, refinements=i.refinements, time_ms=i.time_ms,
                    launches=i.kernel_launches) for i in infos]


def solve_particles_device(ops, precs, b_ptrs, x_ptrs, nrhs, tol=1e-6, maxit=2000, precision="mixed",
                           iters_per_graph=4):
    """vs_solve_particles_device: several particles' batched solves at once
    (device buffers, double2, nrhs[i]*n3 each).  Particles whose operators
    live on different Contexts run concurrently, one host thread per context;
    returns one list of info dicts per particle."""
    if not ops:
        return []
    lib = ops[0].ctx._lib
    k = len(ops)
    o = _solve_opts(lib, tol, maxit, precision)
    o.iters_per_graph = int(iters_per_graph)
    raw = lambda v: v.value if isinstance(v, C.c_void_p) else v
    arr = lambda vals: (C.c_void_p * k)(*[C.c_void_p(raw(v)) for v in vals])
    pops = arr([op.h for op in ops])
    ppr = arr([pr.h if pr is not None else None for pr in precs])
    nr = (C.c_int64 * k)(*[int(v) for v in nrhs])
    infos = (L.vs_solve_info * int(sum(nrhs)))()
    L.check(lib.vs_solve_particles_device(k, pops, ppr, arr(b_ptrs), arr(x_ptrs), nr, C.byref(o), infos))
    out, at = [], 0
    for v in nrhs:
        out.append([dict(flag=i.flag, relres=i.relres, iter=i.iter, refinements=i.refinements, time_ms=i.time_ms,
                         launches=i.kernel_launches) for i in infos[at:at + int(v)]])
        at += int(v)
    return out


def solve_particles(ops, precs, b_ptrs, x_ptrs, nrhs, grams=None, tol=1e-6, maxit=2000, precision="mixed",
                    iters_per_graph=4):
    """vs_solve_particles: several particles (distinct operators on one
    Context) solved in lockstep, one CUDA graph launch per inner iteration of
    all of them.  b_ptrs / x_ptrs: device buffers (complex128, nrhs[i]*n3
    each; x starts from zero); grams: None or per particle None / the Gram of
    each right-hand side (nrhs[i] scalars or grids).  Returns one list of
    info dicts per particle."""
    if not ops:
        return []
    lib = ops[0].ctx._lib
    k = len(ops)
    o = _solve_opts(lib, tol, maxit, precision)
    o.iters_per_graph = int(iters_per_graph)
    raw = lambda v: v.value if isinstance(v, C.c_void_p) else v
    arr = lambda vals: (C.c_void_p * k)(*[C.c_void_p(raw(v)) for v in vals])
    keep = []
    gptr = (L._pd * k)()
    gn = (C.c_int64 * k)()
    for i in range(k):
        if grams is not None and grams[i] is not None:
            g, n_ = _gram_array(grams[i], int(nrhs[i]), ops[i].LMN)
            keep.append(g)
            gptr[i] = L.dptr(g)
            gn[i] = n_
    nr = (C.c_int64 * k)(*[int(v) for v in nrhs])
    infos = (L.vs_solve_info * int(sum(nrhs)))()
    L.check(lib.vs_solve_particles(k, arr([op.h for op in ops]),
                                   arr([pr.h if pr is not None else None for pr in (precs or [None] * k)]),
                                   arr(b_ptrs), arr(x_ptrs), nr, gptr if grams is not None else None, gn,
                                   C.byref(o), infos), ops[0].ctx.h)
    out, at = [], 0
    for v in nrhs:
        out.append([dict(flag=i.flag, relres=i.relres, iter=i.iter, refinements=i.refinements, time_ms=i.time_ms,
                         launches=i.kernel_launches) for i in infos[at:at + int(v)]])
        at += int(v)
    return out


def solve_batch_device(op, b_ptr, x_ptr, nrhs, prec=None, tol=1e-6, maxit=2000, precision="mixed",
                       iters_per_graph=4, gram=None, fold=True):
    """vs_solve_batch_device on device buffers (double2, nrhs*n3 each); ``gram``
    and ``fold`` as in solve_batch."""
    lib = op.ctx._lib
    o = _solve_opts(lib, tol, maxit, precision)
    o.iters_per_graph = int(iters_per_graph)
    o.unfused = 0 if fold else 1
    if gram is not None:
        g, o.gram_n = _gram_array(gram, nrhs, op.LMN)
        o.gram = L.dptr(g)
    infos = (L.vs_solve_info * nrhs)()
    L.check(lib.vs_solve_batch_device(op.h, prec.h if prec is not None else None, C.c_void_p(b_ptr),
                                      C.c_void_p(x_ptr), nrhs, C.byref(o), infos), op.ctx.h)
    return [dict(flag=i.flag, relres=i.relres, iter=i.iter, refinements=i.refinements, time_ms=i.time_ms,
                 launches=i.kernel_launches) for i in infos]
