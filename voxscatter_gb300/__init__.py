"""GB300-native (sm_103a) FFT-accelerated DDA / Galerkin-JVIE solver.

The compute path is ``libvoxscatter.so`` (hand-written CUDA behind a C ABI,
declared in include/voxscatter.h); this package is the host-side mirror of the
reference's MATLAB interface (MVP, getOPERATOR_DDA, circ_1_level,
circ_2_level, mvp_circ_2_level, bicgstab, gmres) on top of it.
"""
