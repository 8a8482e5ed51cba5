"""Quadrature generated here (Gauss-Legendre restated, Lebedev solved from the
moment equations) against the reference's own rules (golden fixture)."""
import numpy as np
import pytest

from openmmcustomgbintegralforce_gb300 import quadrature as Q
from tests.conftest import golden


def test_gauss_legendre_bit_identical_to_reference():
    g = golden("quadrature.npz")
    for n in (24, 32):
        x, w = Q.gauss_legendre(0.05, 2.0, n)
        assert np.array_equal(x, g[f"gl{n}_x"])
        assert np.array_equal(w, g[f"gl{n}_w"])


@pytest.mark.parametrize("order", [26, 38, 50, 110])
def test_lebedev_matches_reference_rule(order):
    from scipy.spatial import cKDTree

    ref = golden("quadrature.npz")[f"leb{order}"]
    xyz, w = Q.lebedev(order)
    d, idx = cKDTree(xyz).query(ref[:, :3])
    assert len(set(idx.tolist())) == order
    assert d.max() < 2e-15
    assert np.abs(ref[:, 3] - w[idx]).max() < 1e-17


@pytest.mark.parametrize("order", sorted(Q.LEBEDEV_ORBITS))
def test_lebedev_exact_to_its_degree(order):
    xyz, w = Q.lebedev(order)
    degree = Q.LEBEDEV_ORBITS[order][0]
    assert abs(w.sum() - 1.0) < 1e-15
    assert np.abs(np.linalg.norm(xyz, axis=1) - 1).max() < 1e-15
    for (a, b, c, exact) in Q._moments(degree):
        for perm in ((a, b, c), (b, c, a), (c, a, b)):
            v = np.sum(w * xyz[:, 0] ** (2 * perm[0]) * xyz[:, 1] ** (2 * perm[1]) * xyz[:, 2] ** (2 * perm[2]))
            assert abs(v - exact) < 1e-15
    # odd moments vanish by symmetry
    assert abs(np.sum(w * xyz[:, 0] ** 3 * xyz[:, 1])) < 1e-16


def test_header_matches_solver():
    import os
    import re

    path = os.path.join(os.path.dirname(Q.__file__), "csrc", "lebedev_rules.h")
    text = open(path).read()
    for order in (26, 38, 50, 110):
        m = re.search(rf"kRule{order}\[{order * 4}\] = \{{(.*?)\}};", text, re.S)
        vals = np.array([float(v) for v in m.group(1).replace("\n", " ").split(",") if v.strip()])
        xyz, w = Q.lebedev(order)
        assert np.array_equal(vals.reshape(order, 4), np.column_stack([xyz, w]))


def test_tensor_layout_matches_reference_ordering():
    off, rad, w = Q.tensor_quadrature(24, 38, 0.05, 2.0)
    x, wr = Q.gauss_legendre(0.05, 2.0, 24)
    u, ws = Q.lebedev(38)
    assert off.shape == (912, 3)
    assert np.array_equal(rad[38 * 5: 38 * 6], np.full(38, x[5]))
    assert np.array_equal(w[38 * 5 + 7], wr[5] * ws[7])
    # Gauss-Legendre-24 integrates 1/r^2 on [0.05, 2] to ~1e-5 relative
    assert abs(np.sum(w / rad ** 2) / (1 / 0.05 - 1 / 2.0) - 1) < 1e-4
