"""The C-ABI library builds, loads without a GPU and exports every function
declared in include/voxscatter.h (no compute calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "voxscatter.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(vs_[A-Za-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from voxscatter_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_header(lib):
    from voxscatter_gb300 import _lib
    assert set(_declared()) == set(_lib.SIGNATURES)


def test_no_gpu_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from voxscatter_gb300 import _lib
    h = ctypes.c_void_p()
    st = lib.vs_ctx_create(0, ctypes.byref(h))
    assert st != _lib.VS_OK
    assert lib.vs_last_error(None)


def test_eps_layer_average_host(lib):
    """vs_eps_layer_average is host arithmetic: against the restatement of
    scatteringHumanHead.m:157-177 without a GPU (<= 1e-14 relative)."""
    import numpy as np
    import oracle as O
    from voxscatter_gb300 import api
    rng = np.random.default_rng(4)
    eps = 2.0 + rng.normal(size=(7, 5, 4)) + 0.1j * rng.normal(size=(7, 5, 4))
    f = api.eps_layer_average(eps)
    f_o = O.eps_layer_average(eps)
    assert f.shape == (12,)
    assert np.abs(f - f_o).max() <= 1e-14 * np.abs(f_o).max()


def test_particles_entry_rejects_bad_arguments_without_a_gpu(lib):
    """vs_solve_particles_device checks its arguments before any CUDA call."""
    import ctypes as C
    from voxscatter_gb300 import _lib as L
    o = L.vs_solve_opts()
    lib.vs_solve_opts_default(C.byref(o))
    info = (L.vs_solve_info * 1)()
    nul = (C.c_void_p * 1)(None)
    nr = (C.c_int64 * 1)(1)
    assert lib.vs_solve_particles_device(0, nul, nul, nul, nul, nr, C.byref(o), info) == L.VS_ERR_ARG
    assert lib.vs_solve_particles_device(1, nul, nul, nul, nul, nr, C.byref(o), info) == L.VS_ERR_ARG
    assert b"NULL operator" in lib.vs_last_error(None)
