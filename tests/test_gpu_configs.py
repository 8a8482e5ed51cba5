"""The benchmark configurations at their own sizes against the FP64 oracle,
through the C ABI:

* GBMV-II and GBMV-I, 10,000 atoms, 24 x 50 quadrature, after a few
  MD-like jittered calls on one context (the last conformation is checked);
* GBSW, 50,000 atoms, 32 x 110 quadrature, 2.0 nm pair cutoff (the chain
  rule's cutoff quirk included);
* the GBMV-I / GBMV-II adjoint (dE/dq, dE/dR, dE/dalpha) against the
  oracle's analytic adjoint, which tests/test_oracle_adjoint.py pins to FP64
  central differences.

Tolerances (FP32 arithmetic, FP64 Born-radius assembly): energy 2e-5
relative, forces and every gradient 1e-4 relative RMS, Born radii 1e-4
maximum relative.
"""
import numpy as np
import pytest

from openmmcustomgbintegralforce_gb300._lib import Context
from openmmcustomgbintegralforce_gb300.globule import make_globule
from openmmcustomgbintegralforce_gb300.spec import GBModel, box_for
from oracle import oracle as O

pytestmark = pytest.mark.gpu

E_TOL = 2e-5
F_TOL = 1e-4
B_TOL = 1e-4
G_TOL = 1e-4


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.fixture(scope="module")
def glob10k():
    return make_globule(10000, seed=2027)


@pytest.mark.parametrize("itype", [2, 1])
def test_gbmv_10k_after_jittered_calls(glob10k, itype):
    g = glob10k
    box = box_for(g.positions, margin=1.0)
    m = (GBModel.gbmv2 if itype == 2 else GBModel.gbmv1)(box=box, lebedev=50)
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    rng = np.random.default_rng(itype)
    x = g.positions.copy()
    for _ in range(4):  # N(0, 0.01 A) per call, accumulated as in MD
        x = x + rng.normal(0.0, 0.001, size=x.shape)
        E, F = ctx.execute_host(x)
    ref = O.Oracle(m).energy_forces(x, g.charge, g.radius)
    assert abs(E / ref["energy"] - 1) < E_TOL
    assert rel_rms(F, ref["forces"]) < F_TOL
    assert np.abs(ctx.born_radii() / ref["born"] - 1).max() < B_TOL
    ctx.close()


def test_gbsw_50k_cutoff_vs_oracle():
    g = make_globule(50000, seed=2026)
    m = GBModel.charmm_gbsw(n_radial=32, lebedev=110, cutoff=2.0)
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    E, F = ctx.execute_host(g.positions)
    E2, F2 = ctx.execute_host(g.positions)
    assert E2 == E and np.array_equal(F2, F)
    ref = O.Oracle(m).energy_forces(g.positions, g.charge, g.radius)
    assert abs(E / ref["energy"] - 1) < E_TOL
    assert rel_rms(F, ref["forces"]) < F_TOL
    assert np.abs(ctx.born_radii() / ref["born"] - 1).max() < B_TOL
    ctx.close()


@pytest.mark.parametrize("itype", [1, 2])
def test_gbmv_adjoint_vs_oracle(itype):
    g = make_globule(1000, seed=43)
    box = box_for(g.positions, margin=1.0)
    m = (GBModel.gbmv2 if itype == 2 else GBModel.gbmv1)(box=box)
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    out = ctx.adjoint(g.positions)
    ref = O.Oracle(m).energy_forces(g.positions, g.charge, g.radius, adjoint=True)
    errs = {"energy": abs(out["energy"] / ref["energy"] - 1), "forces": rel_rms(out["forces"], ref["forces"]),
            "dEdq": rel_rms(out["dEdq"], ref["dEdq"]), "dEdR": rel_rms(out["dEdR"], ref["dEdR"]),
            "dEdalpha": float(np.abs(out["dEdalpha"] / ref["dEdalpha"] - 1).max())}
    print(f"GBMV-{itype} adjoint errors: {errs}")
    assert errs["energy"] < E_TOL
    assert errs["forces"] < F_TOL
    assert errs["dEdq"] < G_TOL
    assert errs["dEdR"] < G_TOL
    assert errs["dEdalpha"] < G_TOL
    ctx.close()


@pytest.mark.parametrize("itype", [1, 2])
def test_gbmv_bitwise_deterministic(itype):
    """The cell passes hand out slots by atomics; sorting each cell's points
    makes every sum's order a function of the input: repeated calls and a
    fresh context give the same bits."""
    g = make_globule(3000, seed=53)
    box = box_for(g.positions, margin=1.0)
    m = (GBModel.gbmv2 if itype == 2 else GBModel.gbmv1)(box=box, lebedev=50)
    runs = []
    for _ in range(2):
        ctx = Context(m, g.n)
        ctx.set_particle_parameters(g.charge, g.radius)
        for _ in range(2):
            runs.append(ctx.execute_host(g.positions))
        ctx.close()
    for E, F in runs[1:]:
        assert E == runs[0][0] and np.array_equal(F, runs[0][1])
