"""Host-side crystallography: space-group decomposition, reflection sets,
conventions, radial integrals and harmonics of the oracle."""
import math

import numpy as np
import pytest

from discamb_gb300 import crystal as X
from discamb_gb300 import workloads as W
from oracle import oracle as O


@pytest.mark.parametrize("sym,n_total,n_sub,centro,cent", [
    ("P1", 1, 1, False, "P"), ("P-1", 2, 1, True, "P"), ("P21", 2, 2, False, "P"),
    ("P21/c", 4, 2, True, "P"), ("P212121", 4, 4, False, "P"), ("C2/c", 8, 2, True, "C"),
    ("P43212", 8, 8, False, "P"), ("P-1(shift)", 2, 1, True, "P"), ("I2/m-like", 8, 2, True, "I")])
def test_space_group_decomposition(sym, n_total, n_sub, centro, cent):
    g = X.space_group(sym)
    assert g.n_total == n_total and g.n_subset == n_sub
    assert g.centrosymmetric == centro and g.centering == cent
    assert g.point_group_order * {"P": 1, "C": 2, "I": 2}[cent] == n_total


def test_operations_must_form_a_group():
    with pytest.raises(ValueError):
        X.SpaceGroup("bad", ["x,y,z", "-x,y+1/3,-z"])


def test_config1_reflection_count():
    cell = (60.0, 70.0, 80.0, 90.0, 90.0, 90.0)
    hkl = X.unique_hkl(cell, X.space_group("P212121"), d_min=1.5)
    assert len(hkl) == 54704
    assert (hkl >= 0).all()


def test_unique_reflections_are_unique_and_complete():
    g = X.space_group("P21/c")
    cell = (9.0, 11.0, 13.0, 90.0, 101.0, 90.0)
    hkl = X.unique_hkl(cell, g, d_min=1.0)
    orbits = set()
    for h in hkl:
        orb = {tuple(int(v) for v in s * (h @ r)) for r in g.rot for s in (1, -1)}
        assert not (orb & orbits)
        orbits |= orb
    full = X.unique_hkl(cell, X.space_group("P1"), d_min=1.0)
    assert sum(1 for h in full if tuple(h) in orbits) + sum(1 for h in full if tuple(-h) in orbits) >= len(full)


def test_centering_absences_removed():
    g = X.space_group("C2/c")
    hkl = X.unique_hkl((12.0, 9.0, 14.0, 90.0, 100.0, 90.0), g, d_min=1.2)
    assert np.all((hkl[:, 0] + hkl[:, 1]) % 2 == 0)


@pytest.mark.parametrize("src,dst", [("U_cif", "U_cart"), ("U_cif", "U_star"), ("U_cart", "U_star")])
def test_adp_conventions_round_trip(src, dst):
    cell = (8.1, 9.3, 10.7, 82.0, 101.0, 95.0)
    u = np.array([0.03, 0.02, 0.04, 0.004, -0.003, 0.002])
    v = X.convert_adp(cell, X.convert_adp(cell, u, src, dst), dst, src)
    assert np.allclose(u, v, rtol=0, atol=1e-15)
    # gradient conversion is the adjoint of the parameter map
    g = np.array([0.3, -1.2, 0.7, 0.11, 0.5, -0.2])
    du = np.array([1e-3, 2e-3, -1e-3, 5e-4, 1e-4, -3e-4])
    dv = X.convert_adp(cell, u + du, src, dst) - X.convert_adp(cell, u, src, dst)
    gd = X.convert_adp_gradient(cell, g, dst, src)
    assert abs(np.dot(g, dv) - np.dot(gd, du)) < 1e-14


@pytest.mark.parametrize("l,n", [(0, 2), (0, 5), (1, 3), (1, 6), (2, 4), (2, 8), (3, 5), (3, 9), (4, 6), (4, 10)])
def test_radial_integral_matches_quadrature(l, n):
    from scipy import integrate, special
    z = 6.3
    for h in (0.05, 0.4, 1.1):
        k = 2 * math.pi * h
        val, _ = integrate.quad(lambda r: r ** n * math.exp(-z * r) * special.spherical_jn(l, k * r), 0, 60,
                                limit=400, epsabs=1e-15, epsrel=1e-12)
        assert abs(O.g_function(l, n, h, z) - val) <= 1e-10 * max(abs(val), 1e-12)


def test_harmonics_are_density_normalised():
    # (2 - delta_l0) = int |d_lm| dOmega, checked with a Fibonacci-sphere average
    n = 200000
    k = np.arange(n)
    z = 1 - (2 * k + 1) / n
    r = np.sqrt(1 - z * z)
    phi = math.pi * (3 - math.sqrt(5)) * k
    u = np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)
    vals = np.array([O.dlm(v) for v in u[::20]])
    integ = np.abs(vals).mean(axis=0) * 4 * math.pi
    target = np.array([1.0] + [2.0] * 24)
    assert np.allclose(integ, target, rtol=2e-3)


def test_workload_generator_is_seeded():
    a = W.config0(seed=0)
    b = W.config0(seed=0)
    assert np.array_equal(a.xyz, b.xyz) and np.array_equal(a.dtdf, b.dtdf)
    assert a.n_atoms == 32 and 3500 < a.n_hkl < 6000
