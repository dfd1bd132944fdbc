"""The five configurations, generated by the reference's voxelisation rules
(geometry.m:42-62, generatedomain_new.m:86-98; koch_snowflake.m for the
snowflake), have the grid sizes, dipole counts and material parameters the
benchmark and the tests are quoted on."""
import numpy as np

from voxscatter_gb300 import workloads as W


def test_config1_hex_plate_cpu_case():
    p = W.config1()
    assert (p["L"], p["M"], p["N"]) == (27, 23, 7)          # the ceil rule of geometry.m
    assert p["refInd"] == 1.31
    assert np.isclose(p["d"], 2.0 / 27)


def test_config2_hex_plate_bench_workload():
    p = W.config2()
    assert (p["L"], p["M"], p["N"]) == (105, 91, 26)
    assert len(p["idx"]) == 186238                         # 558,714 unknowns
    assert p["refInd"] == 1.31 + 0.01j
    assert np.allclose(p["kvec"] / np.linalg.norm(p["kvec"]), [0, 0, 1]) and np.allclose(p["Eo"], [1, 0, 0])


def test_config3_thirty_two_plates_sixteen_rhs_each():
    ps = W.config3_particles(seed=0)
    assert len(ps) == 32 and all(len(q["rhs"]) == 16 for q in ps)
    sizes = [q["L"] for q in ps]
    assert min(sizes) >= 10 and max(sizes) <= 90             # diameters U[1, 6] lambda
    for q in ps:
        for v, pol in q["rhs"]:                               # unit directions, transverse polarisations
            assert np.isclose(np.linalg.norm(v), 1) and abs(np.dot(v, pol)) < 1e-12
    assert W.config3_particles(seed=0)[5]["L"] == ps[5]["L"]  # seeded


def test_config4_random_permittivity_slab():
    p = W.config4(seed=0)
    assert (p["L"], p["M"], p["N"]) == (64, 64, 16) and len(p["idx"]) == 64 * 64 * 16
    eps0 = (1.5 + 0.02j) ** 2
    assert abs(np.mean(p["eps"]) - eps0) < 0.02 * abs(eps0)
    rel = np.real(p["eps"] / eps0) - 1                        # 0.1 g, g of unit standard deviation
    assert 0.07 < np.std(rel) < 0.13


def test_config5_koch_snowflake_grid():
    p = W.config5()
    assert (p["L"], p["M"], p["N"]) == (256, 256, 64)
    assert p["refInd"] == 1.78 + 0.005j and np.isclose(p["d"], 0.125)
    nz = np.unique(p["idx"] // (256 * 256))
    assert len(nz) == 16                                      # 2 lambda of thickness at d = lambda/8


def test_config5_snowflake_area_matches_koch_formula():
    """Each filled layer of the level-3 snowflake (circumradius 16 lambda at
    d = lambda/8) holds as many voxels as the Koch area formula
    A_n = A_0 (8/5 - 3/5 (4/9)^n), A_0 = 3 sqrt(3)/4 R^2, predicts, to the
    staircase error of the voxelisation."""
    p = W.config5()
    per_layer = len(p["idx"]) / 16
    R, d, n = 16.0, 0.125, 3
    area = 3 * np.sqrt(3) / 4 * R ** 2 * (8 / 5 - 3 / 5 * (4 / 9) ** n)
    assert abs(per_layer - area / d ** 2) < 0.01 * area / d ** 2
