"""Generate tests/golden/nop_assembly.npz with the reference's own face-pair
cubature (src/src_vie/src_operators/mexcubatures/cubature_nop_const.cpp,
compiled from the reference checkout by oracle/build_ref.py).

Contents: raw 6x6 face-pair integrals for a few offsets under the far (4x4),
medium (10x10) and near (20x20) rules, and the far + medium N-operator
Toeplitz tensor G (assembly_nop_const.m, near block zero) of two small grids.
Run from the repository root:  python tests/golden/make_nop_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import nop  # noqa: E402


def main():
    ref = nop.reference_cubature()
    if ref is None:
        raise SystemExit("the reference cubature could not be compiled (no reference checkout or g++)")
    out = {}
    ko, dx = 2 * np.pi * 1.3, 0.05
    Rf = nop.cube_faces(dx)
    offs = np.array([[3, 2, 1], [0, 1, 1], [7, 0, 4], [1, 1, 0], [12, 9, 3]])
    for n in (4, 10, 20):
        W, U, V = nop.gauss_2d(n)
        out[f"J_rule{n}"] = np.array([ref(W, U, V, o * dx, np.zeros(3), Rf, ko, dx) for o in offs])
    out["J_offsets"] = offs
    out["ko"], out["dx"] = ko, dx
    for name, (L, M, N) in (("G_7x6x5", (7, 6, 5)), ("G_1x1x6", (1, 1, 6))):
        out[name] = nop.assembly_nop(L, M, N, ko, dx, near_J=None, cubature=ref)
    np.savez_compressed(os.path.join(HERE, "nop_assembly.npz"), **out)
    print("wrote", os.path.join(HERE, "nop_assembly.npz"))


if __name__ == "__main__":
    main()
