"""GPU parity of the Galerkin N-operator Toeplitz assembly (far and medium
cells of assembly_nop_const.m) against fixtures made with the reference's own
cubature_nop_const.cpp and against the oracle; and the assembled tensor
through the JVIE operator pipeline.  Tolerances: 1e-12 relative (FP64)."""
import os

import numpy as np
import pytest

import oracle as O
from oracle import nop

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "nop_assembly.npz")


@pytest.fixture(scope="module")
def api():
    from voxscatter_gb300 import build
    build.build()
    from voxscatter_gb300 import api as A
    return A


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def test_nop_assembly_matches_reference_fixtures(api):
    g = np.load(GOLDEN)
    ko, dx = float(g["ko"]), float(g["dx"])
    for name, shape in (("G_7x6x5", (7, 6, 5)), ("G_1x1x6", (1, 1, 6))):
        assert rel(api.nop_assemble(*shape, ko, dx), g[name]) < 1e-12, name


@pytest.mark.parametrize("shape", [(13, 9, 6), (6, 1, 11), (2, 7, 3)])
def test_nop_assembly_with_near_block_matches_oracle(api, shape):
    rng = np.random.default_rng(sum(shape))
    ko, dx = 2 * np.pi * 1.1, 0.04
    near = rng.normal(size=nop.near_extent(*shape) + (6, 6)) + 1j * rng.normal(size=nop.near_extent(*shape) + (6, 6))
    near *= dx ** 3
    G = api.nop_assemble(*shape, ko, dx, near_J=near)
    G_o = nop.assembly_nop(*shape, ko, dx, near_J=near)
    assert rel(G, G_o) < 1e-12


def test_nop_tensor_through_the_jvie_operator(api):
    """JVIE matvec Gram*x - Mc*N(x) (JVIE_Solver_const.m:140-141, MVP.m) with the
    device-assembled N tensor against the oracle MVP of the same tensor."""
    L, M, N = 8, 7, 5
    ko, dx = 2 * np.pi, 0.05
    rng = np.random.default_rng(3)
    near = (rng.normal(size=(2, 2, 2, 6, 6)) + 1j * rng.normal(size=(2, 2, 2, 6, 6))) * dx ** 3
    G = api.nop_assemble(L, M, N, ko, dx, near_J=near)
    idx3 = np.arange(3 * L * M * N)
    eps = 2.0 + 0.1j
    Mc = (eps - 1) / eps
    Gram = dx ** 3
    op = api.Operator(L, M, N, idx3, 1.0, Mc, Gram, toep=G)
    fN = O.fft_operator(O.circulant_nop_const(G))
    x = rng.normal(size=idx3.size) + 1j * rng.normal(size=idx3.size)
    y_o = O.MVP(x, fN, np.ones((L, M, N)), Mc, Gram, "notransp", idx3)
    assert rel(op.apply(x, "notransp", "c128"), y_o) < 1e-11
