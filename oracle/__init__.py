"""CPU FP64 oracle for the VoxScatter DDA / Galerkin-JVIE hot path.

TEST INFRASTRUCTURE ONLY.  This package is imported by ``tests/``, by
``__graft_entry__.smoke()`` (as the checker) and by the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py``.  The product path
(``voxscatter_gb300``) never imports it.

It is a NumPy/SciPy restatement of the reference MATLAB code, one function per
reference function, each citing the file:line it follows (paths relative to the
VoxScatter repository root).  All arithmetic is complex FP64, as in the
reference.  Arrays use the MATLAB column-major convention: a grid array of
shape (L, M, N[, c]) is flattened with ``order='F'`` and voxel indices are
0-based column-major linear indices ``i + L*(j + M*k)``.

Parity status: UNPINNED against the reference's own outputs.  The reference is
MATLAB (no MATLAB/Octave is available to run it) and ships no golden vectors,
known-answer tests or fixtures for this path.  The restatement is instead
pinned by independent mathematics: a dense O(n^2) direct-sum DDA operator (which
checks the circulant embedding and its sign tables), explicit dense circulant
matrices (which check the Chan-Olkin levels), direct dense solves (which check
the Krylov solvers) and Mie theory (which checks the extinction cross section).
"""
from .operators import (alpha_ldr, green_toeplitz, circulant_nop_const,
                        gperiodic_coeff_nop, fft_operator, getOPERATOR_DDA,
                        dalpha_inv_deps)
from .mvp import MVP, mv_AN_const, dense_dda_matrix, dense_from_toeplitz
from .precond import (circ_1_level, circ_2_level, eps_layer_average, invert_blocks,
                      mvp_circ_2_level, chan_mvp_idx, circ_1_level_blocks)
from .krylov import bicgstab, gmres, pgmres, pgmres_dr, harm_vecs1, harm_vecs2
from .physics import (PlaneWavePointWise, cext_dda, cext_grad_dda, far_field, field_dda, mie_qext,
                      polarisation_basis, orientation_average_cext)

__all__ = [n for n in dir() if not n.startswith("_")]
