"""The custom-expression oracle (oracle/custom.py) pinned to the FP64 oracle:
the canonical CHARMM set written as user expressions reproduces the
canonical evaluation (CharmmReferenceGBSW's formulas) for the GBMV-II and
GBSW-integral classes, and its forces are minus the gradient of its energy
for expression sets outside the canonical one (tabulated functions
included).  Also the library's own expression compiler on the CPU: every
set compiles, and a wrong one is refused with a message (gbx_custom_check:
no device needed)."""
import copy

import numpy as np
import pytest

from openmmcustomgbintegralforce_gb300.globule import make_globule
from openmmcustomgbintegralforce_gb300.spec import GBModel, box_for
from oracle import oracle as O
from oracle.custom import CustomOracle
from openmmcustomgbintegralforce_gb300.expression_sets import (CANONICAL, EXTENDED, FUNCTIONS, MODIFIED, TABULATED,
                                                               extended_exclusions, modified_params)


@pytest.fixture(scope="module")
def glob():
    return make_globule(150, seed=71)


@pytest.mark.parametrize("cls", ["gbmv2", "gbsw_integral"])
def test_canonical_expressions_match_canonical_oracle(glob, cls):
    g = glob
    m = GBModel.gbmv2(box=box_for(g.positions, margin=1.0)) if cls == "gbmv2" else GBModel.gbsw_integral()
    ref = O.Oracle(m).energy_forces(g.positions, g.charge, g.radius)
    got = CustomOracle(m, CANONICAL).energy_forces(g.positions, np.stack([g.charge, g.radius], axis=1))
    assert abs(got["energy"] / ref["energy"] - 1) < 1e-12
    assert np.abs(got["forces"] - ref["forces"]).max() < 1e-10 * np.abs(ref["forces"]).max()
    assert np.abs(got["values"][0] / ref["born"] - 1).max() < 1e-12


def test_modified_expressions_forces_are_energy_gradient(glob):
    g = glob
    m = GBModel.gbmv2(box=box_for(g.positions, margin=1.0))
    P = modified_params(g)
    orc = CustomOracle(m, MODIFIED)
    out = orc.energy_forces(g.positions, P)
    rng = np.random.default_rng(4)
    h = 1e-6
    F = out["forces"]
    for flat in rng.choice(3 * g.n, size=6, replace=False):
        i, d = int(flat) // 3, int(flat) % 3
        xp, xm = g.positions.copy(), g.positions.copy()
        xp[i, d] += h
        xm[i, d] -= h
        fd = -(orc.energy_forces(xp, P)["energy"] - orc.energy_forces(xm, P)["energy"]) / (2 * h)
        assert abs(fd - F[i, d]) <= 1e-6 * np.abs(F).max() + 1e-5 * abs(F[i, d]), (i, d, fd, F[i, d])


def test_extended_expressions_gradients(glob):
    """Coordinates in a computed value and a single-particle term, excluded
    pairs skipped by a ParticlePair term only, and the energy derivatives
    by globals: forces and parameter derivatives against FP64 central
    differences of the oracle's own energy."""
    g = glob
    m = GBModel.gbmv2(box=box_for(g.positions, margin=1.0))
    P = np.stack([g.charge, g.radius], axis=1)
    ext = dict(EXTENDED, exclusions=extended_exclusions(g.n))
    orc = CustomOracle(m, ext)
    out = orc.energy_forces(g.positions, P)
    rng = np.random.default_rng(5)
    h = 1e-6
    F = out["forces"]
    for flat in rng.choice(3 * g.n, size=6, replace=False):
        i, d = int(flat) // 3, int(flat) % 3
        xp, xm = g.positions.copy(), g.positions.copy()
        xp[i, d] += h
        xm[i, d] -= h
        fd = -(orc.energy_forces(xp, P)["energy"] - orc.energy_forces(xm, P)["energy"]) / (2 * h)
        assert abs(fd - F[i, d]) <= 1e-6 * np.abs(F).max() + 1e-5 * abs(F[i, d]), (i, d, fd, F[i, d])
    for k, name in enumerate(ext["param_derivs"]):
        gp, gm = dict(ext["globals"]), dict(ext["globals"])
        gp[name] += h
        gm[name] -= h
        ep = CustomOracle(m, dict(ext, globals=gp)).energy_forces(g.positions, P)["energy"]
        em = CustomOracle(m, dict(ext, globals=gm)).energy_forces(g.positions, P)["energy"]
        fd = (ep - em) / (2 * h)
        assert abs(fd - out["param_derivs"][k]) <= 1e-6 * abs(fd) + 1e-6, (name, fd, out["param_derivs"][k])
    # the exclusions change the ParticlePair term
    plain = CustomOracle(m, EXTENDED).energy_forces(g.positions, P)
    assert abs(plain["energy"] / out["energy"] - 1) > 1e-4


def test_tabulated_expressions_gradients(glob):
    """Tabulated functions (natural cubic splines) in a computed value, a
    single-particle term and a pair term: forces against FP64 central
    differences of the oracle's energy; a pair beyond the table's range
    gets nothing from it."""
    from oracle.custom import tabulated

    g = glob
    m = GBModel.gbmv2(box=box_for(g.positions, margin=1.0))
    P = np.stack([g.charge, g.radius], axis=1)
    orc = CustomOracle(m, TABULATED)
    out = orc.energy_forces(g.positions, P)
    rng = np.random.default_rng(6)
    h = 1e-6
    F = out["forces"]
    for flat in rng.choice(3 * g.n, size=6, replace=False):
        i, d = int(flat) // 3, int(flat) % 3
        xp, xm = g.positions.copy(), g.positions.copy()
        xp[i, d] += h
        xm[i, d] -= h
        fd = -(orc.energy_forces(xp, P)["energy"] - orc.energy_forces(xm, P)["energy"]) / (2 * h)
        assert abs(fd - F[i, d]) <= 1e-6 * np.abs(F).max() + 1e-5 * abs(F[i, d]), (i, d, fd, F[i, d])
    tail = tabulated(TABULATED["functions"])["tail"]
    import sympy as sp

    f = sp.lambdify([sp.Symbol("t")], tail(sp.Symbol("t")), "numpy")
    vals, lo, hi = TABULATED["functions"]["tail"]
    assert np.allclose(f(np.linspace(lo, hi, len(vals))), vals, atol=1e-12)  # through its points
    assert f(np.array([hi + 0.1, lo - 0.1])).tolist() == [0.0, 0.0]  # zero outside


def test_function_set_gradients(glob):
    """The Lepton function set (FUNCTIONS): forces against FP64 central
    differences of the oracle's energy."""
    g = glob
    m = GBModel.gbmv2(box=box_for(g.positions, margin=1.0))
    P = np.stack([g.charge, g.radius], axis=1)
    orc = CustomOracle(m, FUNCTIONS)
    F = orc.energy_forces(g.positions, P)["forces"]
    rng = np.random.default_rng(7)
    h = 1e-6
    for flat in rng.choice(3 * g.n, size=6, replace=False):
        i, d = int(flat) // 3, int(flat) % 3
        xp, xm = g.positions.copy(), g.positions.copy()
        xp[i, d] += h
        xm[i, d] -= h
        fd = -(orc.energy_forces(xp, P)["energy"] - orc.energy_forces(xm, P)["energy"]) / (2 * h)
        assert abs(fd - F[i, d]) <= 1e-6 * np.abs(F).max() + 1e-5 * abs(F[i, d]), (i, d, fd, F[i, d])


def test_library_compiles_and_refuses_expression_sets():
    from openmmcustomgbintegralforce_gb300._lib import check_custom

    for s in (CANONICAL, MODIFIED, dict(EXTENDED, exclusions=extended_exclusions(50)), TABULATED, FUNCTIONS):
        st, msg = check_custom(s)
        if st == 4 and "NVRTC" in msg:
            pytest.skip("NVRTC not available")
        assert st == 0, msg
    bad = copy.deepcopy(MODIFIED)
    bad["terms"] = [("q^2/Bx", 0)]
    st, msg = check_custom(bad)
    assert st != 0 and "Bx" in msg
    bad["terms"] = [("q^2/(B", 0)]
    st, msg = check_custom(bad)
    assert st != 0 and "expected ')'" in msg
    bad = copy.deepcopy(MODIFIED)
    bad["params"] = ["q", "s"]
    st, msg = check_custom(bad)
    assert st != 0 and "radius" in msg
    # tabulated functions: too few values, an empty range, a missing table, a wrong argument count
    bad = copy.deepcopy(TABULATED)
    bad["functions"]["scale"] = ([1.0], 0.0, 1.0)
    st, msg = check_custom(bad)
    assert st != 0 and "at least 2 values" in msg
    bad["functions"]["scale"] = ([1.0, 2.0], 1.0, 1.0)
    st, msg = check_custom(bad)
    assert st != 0 and "max > min" in msg
    bad = copy.deepcopy(TABULATED)
    del bad["functions"]["tail"]
    st, msg = check_custom(bad)
    assert st != 0 and "tail" in msg
    bad = copy.deepcopy(TABULATED)
    bad["terms"][3] = ("q1*q2*tail(r, r)", 2)
    st, msg = check_custom(bad)
    assert st != 0 and "one argument" in msg
