"""Voxel grids and particle shapes (host-side input generation).

Restates src/src_geometry/geometry.m:1-71, src_domain/generatedomain_new.m:41-104,
src_domain/grid3d.m:35-61 and koch_snowflake.m:7-101.  Grids are returned as
``r`` of shape (L, M, N, 3) and ``idx`` as sorted 0-based column-major linear
voxel indices (MATLAB's ``find`` minus one).
"""
import math

import numpy as np


def matlab_colon(a, d, b):
    """MATLAB ``a:d:b``: count by floor with a relative tolerance, elements
    evaluated from both ends (a + k*d in the first half, b' - (n-k)*d after)."""
    n = int(math.floor((b - a) / d + 1e-10))
    if n < 0:
        return np.zeros(0)
    k = np.arange(n + 1, dtype=float)
    end = a + n * d
    out = np.where(k <= n / 2, a + k * d, end - (n - k) * d)
    return out


def grid3d(x, y, z):
    """r(L,M,N,3) from coordinate vectors, grid3d.m:41-61."""
    X, Y, Z = np.meshgrid(np.asarray(x, float), np.asarray(y, float),
                          np.asarray(z, float), indexing="ij")
    return np.stack([X, Y, Z], axis=-1)


def generatedomain_new(res, x, y=None, z=None):
    """Centred voxel grid of resolution ``res`` covering [-x,x]x[-y,y]x[-z,z],
    generatedomain_new.m:45-104."""
    if y is None:
        y = x
    if z is None:
        z = x
    vecs = []
    for v in (x, y, z):
        v = np.atleast_1d(np.asarray(v, dtype=float))
        if v.size == 1:
            v = np.array([-v[0], v[0]])
        D = v.max() - v.min()
        n = max(1, int(np.round(D / res)))
        C = (v.max() + v.min()) / 2
        vecs.append(matlab_colon(C - (n / 2 - 0.5) * res, res, C + (n / 2 - 0.5) * res))
    return grid3d(*vecs)


def geometry(geom, refInd, sizeParam, nPerLam, aspect_ratio=0.1):
    """[r, idx, res, P, lambda_ext, lambda_int] = geometry(...), geometry.m:1-71.
    ``aspect_ratio`` is the hexagon's thickness/width, hard-coded to 1/10 at
    geometry.m:21."""
    if geom == "spheroid":
        a, c = 1.0, 0.5
        dom = (2 * a, 2 * a, 2 * c); P = math.pi * a * c
    elif geom == "sphere":
        a = c = 1.0
        dom = (2 * a, 2 * a, 2 * a); P = math.pi * a ** 2
    elif geom == "hex":
        a = 1.0
        b = math.sqrt(3) / 2 * a
        dom = (2 * a, 2 * b, a * aspect_ratio); P = dom[1] * dom[2]
    elif geom == "cube":
        a = 1.0
        dom = (2 * a, 2 * a, 2 * a); P = 4 * a ** 2
    else:
        raise ValueError(geom)
    lambda_ext = 2 * math.pi * a / sizeParam
    h_pref = dom[0]
    lambda_int = lambda_ext / complex(refInd).real
    res_temp = lambda_int / nPerLam
    Nn = math.ceil(h_pref / res_temp)
    res = h_pref / Nn
    r = generatedomain_new(res, dom[0] / 2, dom[1] / 2, dom[2] / 2)
    L, M, N, _ = r.shape
    X, Y = r[..., 0], r[..., 1]
    if geom == "hex":
        s3 = math.sqrt(3)
        l1 = Y - s3 * (a - X)
        l2 = Y - s3 * (X + a)
        l3 = Y - s3 * (-a - X)
        l4 = Y - s3 * (X - a)
        mask = (l1 < 0) & (l2 < 0) & (l3 > 0) & (l4 > 0)
    elif geom in ("spheroid", "sphere"):
        mask = (X ** 2 + Y ** 2) / a ** 2 + r[..., 2] ** 2 / c ** 2 <= 1
    else:
        mask = np.ones((L, M, N), dtype=bool)
    idx = np.nonzero(mask.ravel(order="F"))[0]
    return r, idx, res, P, lambda_ext, lambda_int


def koch_vertices(iterations):
    """Closed polygon of the Koch snowflake, koch_snowflake.m:7-21, centred and
    scaled to unit half-height (koch_snowflake.m:26-37)."""
    P = np.array([[0.0, 0.0], [1.0, 0.0], [math.cos(-math.pi / 3), math.sin(-math.pi / 3)], [0.0, 0.0]])
    for _ in range(iterations):
        n = P.shape[0]
        newP = np.zeros((4 * n + 1, 2))
        for i in range(n - 1):
            newP[4 * i + 0] = P[i]
            newP[4 * i + 1] = (2 * P[i] + P[i + 1]) / 3
            link = P[i + 1] - P[i]
            ang = math.atan2(link[1], link[0])
            leng = math.hypot(link[0], link[1])
            newP[4 * i + 2] = newP[4 * i + 1] + (leng / 3) * np.array([math.cos(ang + math.pi / 3), math.sin(ang + math.pi / 3)])
            newP[4 * i + 3] = (P[i] + 2 * P[i + 1]) / 3
        newP[4 * n] = P[n - 1]
        P = newP[:4 * (n - 1)].tolist() + [P[n - 1].tolist()]
        P = np.array(P)
    xmin, ymin = P.min(axis=0); xmax, ymax = P.max(axis=0)
    P = P - np.array([(xmax + xmin) / 2, (ymax + ymin) / 2])
    return P / ((ymax - ymin) / 2)


def points_in_polygon(px, py, poly):
    """Even-odd rule with boundary points counted as inside (the ``in`` output of
    MATLAB's inpolygon, koch_snowflake.m:101)."""
    px = np.asarray(px, float); py = np.asarray(py, float)
    inside = np.zeros(px.shape, dtype=bool)
    on = np.zeros(px.shape, dtype=bool)
    x1, y1 = poly[:-1, 0], poly[:-1, 1]
    x2, y2 = poly[1:, 0], poly[1:, 1]
    for a1, b1, a2, b2 in zip(x1, y1, x2, y2):
        cond = (b1 > py) != (b2 > py)
        with np.errstate(divide="ignore", invalid="ignore"):
            xint = a1 + (py - b1) * (a2 - a1) / (b2 - b1)
        inside ^= cond & (px < xint)
        cross = (px - a1) * (b2 - b1) - (py - b1) * (a2 - a1)
        seg = (np.abs(cross) <= 1e-12) & (px >= min(a1, a2) - 1e-12) & (px <= max(a1, a2) + 1e-12) \
            & (py >= min(b1, b2) - 1e-12) & (py <= max(b1, b2) + 1e-12)
        on |= seg
    return inside | on
