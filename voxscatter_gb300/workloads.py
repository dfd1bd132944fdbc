"""Seeded synthetic scattering problems with the shapes of the five benchmark
configurations (hexagonal plates, a batch of plates, a random-permittivity slab
and an extruded Koch snowflake).  Host-side input generation only.

A problem is a dict with keys: r (L,M,N,3), idx (0-based voxels), L, M, N, d,
ko, kvec, Eo, eps (per-voxel permittivity at idx, complex), refInd (scalar or
None), label.
"""
import math

import numpy as np

from .geometry import geometry, koch_vertices, points_in_polygon, grid3d, matlab_colon


def hex_plate(diameter_lam, m, n_per_lam=10, aspect_ratio=0.5, direction=(0, 0, 1), pol=(1, 0, 0)):
    """Hexagonal prism plate of the given diameter (in wavelengths), thickness
    aspect_ratio*diameter/2, voxelised with geometry('hex', ...) rules
    (geometry.m:18-62).  Lengths are in units of the plate radius a=1."""
    size_param = math.pi * diameter_lam  # 2*pi*a/lambda with a=1, lambda=2/D
    r, idx, res, _, lam_ext, _ = geometry("hex", m, size_param, n_per_lam, aspect_ratio)
    ko = 2 * math.pi / lam_ext
    L, M, N, _ = r.shape
    kvec = ko * np.asarray(direction, float) / np.linalg.norm(direction)
    return dict(r=r, idx=idx, L=L, M=M, N=N, d=res, ko=ko, kvec=kvec,
                Eo=np.asarray(pol, float), eps=np.full(len(idx), complex(m) ** 2),
                refInd=complex(m), label=f"hex D={diameter_lam}lam m={m} grid {L}x{M}x{N}")


def config1():
    """Hex plate, diameter 2 lambda, thickness 0.5 lambda, m=1.31, +z, x-pol."""
    return hex_plate(2.0, 1.31)


def config2():
    """Hex plate, diameter 8 lambda, thickness 2 lambda, m=1.31+0.01i."""
    return hex_plate(8.0, 1.31 + 0.01j)


def config3_particles(seed=0, n_particles=32):
    """32 hex plates, diameter ~ U[1,6] lambda, thickness D/4, m=1.31+0.01i, each
    with 8 incident directions x 2 polarisations (directions seeded)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_particles):
        D = float(rng.uniform(1.0, 6.0))
        p = hex_plate(D, 1.31 + 0.01j)
        dirs = []
        for _ in range(8):
            v = rng.normal(size=3); v /= np.linalg.norm(v)
            a = np.cross(v, [0, 0, 1.0] if abs(v[2]) < 0.9 else [1.0, 0, 0]); a /= np.linalg.norm(a)
            b = np.cross(v, a)
            dirs.append((v, a)); dirs.append((v, b))
        p["rhs"] = dirs
        out.append(p)
    return out


def config4(seed=0, L=64, M=64, N=16):
    """64x64x16 slab, eps=(1.5+0.02i)^2 (1 + 0.1 g), g a Gaussian random field of
    correlation length 4 voxels (white noise convolved with a sigma=4 Gaussian,
    normalised to unit standard deviation), z-incidence, x-polarisation,
    10 voxels per interior wavelength."""
    rng = np.random.default_rng(seed)
    m0 = 1.5 + 0.02j
    lam = 1.0
    d = lam / (10 * m0.real)
    x = (np.arange(L) - (L - 1) / 2) * d
    y = (np.arange(M) - (M - 1) / 2) * d
    z = (np.arange(N) - (N - 1) / 2) * d
    r = grid3d(x, y, z)
    w = rng.normal(size=(L, M, N))
    g = _gauss_filter(w, 4.0)
    g = (g - g.mean()) / g.std()
    eps_grid = m0 ** 2 * (1 + 0.1 * g)
    idx = np.arange(L * M * N)
    ko = 2 * math.pi / lam
    return dict(r=r, idx=idx, L=L, M=M, N=N, d=d, ko=ko, kvec=np.array([0, 0, ko]),
                Eo=np.array([1.0, 0, 0]), eps=eps_grid.ravel(order="F").astype(complex),
                refInd=None, label=f"slab {L}x{M}x{N} random eps")


def _gauss_filter(w, sigma):
    out = w
    for ax in range(3):
        n = w.shape[ax]
        k = np.fft.fftfreq(n)
        filt = np.exp(-2 * (math.pi * sigma * k) ** 2)
        out = np.fft.ifft(np.fft.fft(out, axis=ax) * filt.reshape([-1 if a == ax else 1 for a in range(3)]), axis=ax).real
    return out


def config5(level=3, L=256, M=256, N=64, layers=16):
    """Koch snowflake (given level), circumradius 16 lambda on a 256x256x64 grid
    with d = lambda/8, extruded over the central ``layers`` z-layers (2 lambda);
    the remaining layers are air.  m = 1.78+0.005i."""
    m = 1.78 + 0.005j
    lam = 1.0
    d = lam / 8
    poly = koch_vertices(level)
    poly = poly * (16.0 / np.max(np.hypot(poly[:, 0], poly[:, 1])))
    x = (np.arange(L) - (L - 1) / 2) * d
    y = (np.arange(M) - (M - 1) / 2) * d
    z = (np.arange(N) - (N - 1) / 2) * d
    r = grid3d(x, y, z)
    inpoly = points_in_polygon(r[:, :, 0, 0].ravel(), r[:, :, 0, 1].ravel(), poly).reshape(L, M)
    zmask = np.abs(np.arange(N) - (N - 1) / 2) < layers / 2
    mask = inpoly[:, :, None] & zmask[None, None, :]
    idx = np.nonzero(mask.ravel(order="F"))[0]
    ko = 2 * math.pi / lam
    return dict(r=r, idx=idx, L=L, M=M, N=N, d=d, ko=ko, kvec=np.array([0, 0, ko]),
                Eo=np.array([1.0, 0, 0]), eps=np.full(len(idx), m ** 2), refInd=m,
                label=f"koch level {level} grid {L}x{M}x{N}")


def small_hex(m=1.31 + 0.05j, nper=3, aspect_ratio=0.5, diameter=2.0):
    """A few-hundred-voxel hex plate for oracle-speed parity tests."""
    return hex_plate(diameter, m, n_per_lam=nper, aspect_ratio=aspect_ratio)
