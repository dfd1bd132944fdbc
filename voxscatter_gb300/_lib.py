"""ctypes binding of libvoxscatter.so (include/voxscatter.h).

The library is loaded from this package directory; there is no fallback: a
missing or unloadable library raises immediately.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvoxscatter.so")

VS_OK, VS_ERR_ARG, VS_ERR_CUDA, VS_ERR_OOM, VS_ERR_NONFINITE, VS_ERR_UNSUPPORTED, VS_ERR_TIMEOUT = range(7)
VS_NOTRANSP, VS_TRANSP, VS_CONJTRANSP = 0, 1, 2
VS_C64, VS_C128 = 0, 1

_pd = C.POINTER(C.c_double)
_pi64 = C.POINTER(C.c_int64)
_vp = C.c_void_p
_i64 = C.c_int64


class vs_diag(C.Structure):
    _fields_ = [("v", _pd), ("n", _i64)]


# name -> (restype, argtypes); every function declared in include/voxscatter.h
SIGNATURES = {
    "vs_ctx_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "vs_ctx_destroy": (C.c_int, [_vp]),
    "vs_last_error": (C.c_char_p, [_vp]),
    "vs_ctx_synchronize": (C.c_int, [_vp]),
    "vs_ctx_stream": (C.c_int, [_vp, C.POINTER(_vp)]),
    "vs_green_dda": (C.c_int, [_vp, _i64, _i64, _i64, _pd, _pd, _pd, C.c_double, C.c_int, _pd]),
    "vs_alpha_ldr": (C.c_int, [_pd, _i64, C.c_int, C.c_double, C.c_double, _pd, _pd, _pd]),
    "vs_circulant_fft": (C.c_int, [_vp, _i64, _i64, _i64, _pd, _i64, _i64, _i64, _pd]),
    "vs_nop_assemble": (C.c_int, [_vp, _i64, _i64, _i64, C.c_double, C.c_double, _pd, _pd]),
    "vs_op_create": (C.c_int, [_vp, _i64, _i64, _i64, _pd, _i64, _i64, _i64, _pi64, _i64, vs_diag, vs_diag,
                               vs_diag, C.POINTER(_vp)]),
    "vs_op_create_fN": (C.c_int, [_vp, _i64, _i64, _i64, _pd, _i64, _i64, _i64, _pi64, _i64, vs_diag, vs_diag,
                                  vs_diag, C.POINTER(_vp)]),
    "vs_op_destroy": (C.c_int, [_vp]),
    "vs_op_info": (C.c_int, [_vp, _pi64, _pi64, _pi64]),
    "vs_op_apply": (C.c_int, [_vp, _pd, _pd, _i64, C.c_int, C.c_int]),
    "vs_op_apply_device": (C.c_int, [_vp, _vp, _vp, _i64, C.c_int, C.c_int]),
    "vs_op_apply_gram": (C.c_int, [_vp, _pd, _pd, _i64, C.c_int, C.c_int, _pd, _i64]),
    "vs_op_apply_device_noalloc": (C.c_int, [_vp, _vp, _vp, _i64, C.c_int, C.c_int]),
    "vs_circ_levels": (C.c_int, [_vp, _i64, _i64, _i64, _pd, _pd, _pd, _pd]),
    "vs_prec_create": (C.c_int, [_vp, _pd, _pd, _i64, C.c_int, C.POINTER(_vp)]),
    "vs_prec_create_blocks": (C.c_int, [_vp, _i64, _i64, _i64, _pd, _pi64, _i64, C.c_int, C.POINTER(_vp)]),
    "vs_prec_destroy": (C.c_int, [_vp]),
    "vs_invert_blocks_device": (C.c_int, [_vp, _vp, _i64, _i64, C.c_int]),
    "vs_prec_apply": (C.c_int, [_vp, _pd, _pd, _i64, C.c_int]),
    "vs_prec_apply_device": (C.c_int, [_vp, _vp, _vp, _i64, C.c_int]),
    "vs_prec_get_blocks": (C.c_int, [_vp, C.c_int, _pd]),
}
VS_BUILD_C64, VS_BUILD_C128, VS_BUILD_LU_TC, VS_BUILD_LU_CUDA = 1, 2, 4, 8
VS_BICGSTAB, VS_GMRES, VS_GMRES_DR = 0, 1, 2
VS_SOLVE_MIXED, VS_SOLVE_FP64 = 0, 1


class vs_solve_opts(C.Structure):
    _fields_ = [("method", C.c_int), ("precision", C.c_int), ("tol", C.c_double), ("maxit", C.c_int),
                ("inner_tol", C.c_double), ("max_refine", C.c_int), ("iters_per_graph", C.c_int),
                ("resvec", _pd), ("resvec_cap", _i64), ("transpose", C.c_int), ("restart", C.c_int),
                ("ritz", C.c_int), ("gram", _pd), ("gram_n", _i64), ("profile_ms", C.POINTER(C.c_float)),
                ("unfused", C.c_int)]


class vs_solve_info(C.Structure):
    _fields_ = [("flag", C.c_int), ("relres", C.c_double), ("iter", C.c_double), ("refinements", C.c_int),
                ("n_resvec", _i64), ("time_ms", C.c_double), ("kernel_launches", _i64)]


class vs_shape(C.Structure):
    _fields_ = [("lg_lines_x", C.c_int), ("lg_tile_y", C.c_int), ("lg_tile_z", C.c_int), ("z_reg", C.c_int),
                ("y_reg", C.c_int), ("x_reg", C.c_int), ("z_df", C.c_int)]


class vs_prec_shape(C.Structure):
    _fields_ = [("lg_lines_x", C.c_int), ("lg_tile_y", C.c_int), ("gemv_blocks", C.c_int), ("gemv_threads", C.c_int),
                ("gemv_mode", C.c_int), ("gemv_chunk", C.c_int), ("y_reg", C.c_int), ("x_reg", C.c_int),
                ("fuse_xy", C.c_int), ("wait_polls", C.c_int)]


SIGNATURES.update({
    "vs_prec_get_shape": (C.c_int, [_vp, C.c_int, C.POINTER(vs_prec_shape)]),
    "vs_prec_set_shape": (C.c_int, [_vp, C.c_int, C.POINTER(vs_prec_shape)]),
    "vs_op_get_shape": (C.c_int, [_vp, C.c_int, C.POINTER(vs_shape)]),
    "vs_op_set_shape": (C.c_int, [_vp, C.c_int, C.POINTER(vs_shape)]),
    "vs_solve_batch": (C.c_int, [_vp, _vp, _pd, _pd, _i64, C.POINTER(vs_solve_opts), C.POINTER(vs_solve_info)]),
    "vs_solve_batch_device": (C.c_int, [_vp, _vp, _vp, _vp, _i64, C.POINTER(vs_solve_opts),
                                        C.POINTER(vs_solve_info)]),
    "vs_solve_particles_device": (C.c_int, [_i64, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp),
                                            C.POINTER(_i64), C.POINTER(vs_solve_opts), C.POINTER(vs_solve_info)]),
    "vs_solve_particles": (C.c_int, [_i64, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp),
                                     C.POINTER(_i64), C.POINTER(_pd), C.POINTER(_i64), C.POINTER(vs_solve_opts),
                                     C.POINTER(vs_solve_info)]),
    "vs_orientation_average": (C.c_int, [_vp, _vp, _pd, _i64, _pd, _pd, _pd, C.c_double, C.c_double, _pd, _pd,
                                         _pd, _i64, C.POINTER(vs_solve_opts), C.POINTER(C.c_double), _pd,
                                         C.POINTER(vs_solve_info)]),
    "vs_plane_wave": (C.c_int, [_vp, _pd, _pd, _pd, _pd, _pd, _pd]),
    "vs_cext": (C.c_int, [_vp, _pd, _pd, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double)]),
    "vs_op_apply_domain": (C.c_int, [_vp, _pd, _pd, C.c_int64, _pd, _pd, C.c_int]),
    "vs_eps_layer_average": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, _pd, _pd]),
    "vs_field_dda": (C.c_int, [_vp, _pd, _pd, C.c_int64, _pd, C.c_double, _pd, _pd, C.c_int]),
    "vs_far_field": (C.c_int, [_vp, _pd, C.c_int64, _pd, _pd, _pd, C.c_double, C.c_double, _pd, C.c_int64, _pd]),
    "vs_cext_grad": (C.c_int, [_vp, _vp, _pd, _pd, C.c_double, C.c_double, _pd, _pd, C.POINTER(vs_solve_opts),
                               C.POINTER(C.c_double), _pd, _pd, _pd, C.POINTER(vs_solve_info),
                               C.POINTER(vs_solve_info)]),
    "vs_op_time_passes": (C.c_int, [_vp, _vp, _vp, _i64, C.c_int, C.c_int, C.POINTER(C.c_float)]),
    "vs_prec_time_passes": (C.c_int, [_vp, _vp, _vp, _i64, C.c_int, C.c_int, C.POINTER(C.c_float)]),
    "vs_solve_opts_default": (None, [C.POINTER(vs_solve_opts)]),
    "vs_solve": (C.c_int, [_vp, _vp, _pd, _pd, C.POINTER(vs_solve_opts), C.POINTER(vs_solve_info)]),
    "vs_solve_device": (C.c_int, [_vp, _vp, _vp, _vp, C.POINTER(vs_solve_opts), C.POINTER(vs_solve_info)]),
})

_lib = None


class VoxScatterError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"libvoxscatter status {status}: {msg}")
        self.status = status


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise VoxScatterError(VS_ERR_ARG, f"{LIB_PATH} not built; run voxscatter_gb300.build.build()")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def check(status, ctx=None):
    if status != VS_OK:
        msg = load().vs_last_error(ctx)
        raise VoxScatterError(status, msg.decode() if msg else "")


def dptr(a):
    """double* view of a contiguous float64/complex128 numpy array."""
    assert a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"]
    return a.ctypes.data_as(_pd)


def cplx_flat(a, order="F"):
    return np.ascontiguousarray(np.asarray(a, dtype=np.complex128).ravel(order=order))


def make_diag(v, keep):
    """vs_diag from a scalar or a grid array; ``keep`` collects the buffers."""
    arr = np.asarray(v, dtype=np.complex128)
    flat = cplx_flat(arr) if arr.ndim > 0 else np.array([complex(arr)], dtype=np.complex128)
    keep.append(flat)
    return vs_diag(dptr(flat), flat.size)
