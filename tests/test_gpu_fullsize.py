"""The 50,000-atom GBSW workload (32 x 110 quadrature, full N^2 pair term)
checked through properties that hold at any size, where the FP64 oracle is
too slow to run in a test: runs are bit-identical, the total force vanishes
(the chain rule adds each contribution to the shaping atom and its negation
to the point's owner as the same fixed-point integer, the pair term applies
+g d and -g d), and a rigid translation leaves energy and forces unchanged
to rounding (the lookup table and cell grid move with the atoms)."""
import numpy as np
import pytest

from openmmcustomgbintegralforce_gb300._lib import Context
from openmmcustomgbintegralforce_gb300.globule import make_globule
from openmmcustomgbintegralforce_gb300.spec import GBModel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def full():
    g = make_globule(50000, seed=2026)
    m = GBModel.charmm_gbsw(n_radial=32, lebedev=110)
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    E, F = ctx.execute_host(g.positions)
    yield g, ctx, E, F
    ctx.close()


def test_bit_identical_runs(full):
    g, ctx, E, F = full
    for _ in range(2):
        E2, F2 = ctx.execute_host(g.positions)
        assert E2 == E and np.array_equal(F2, F)


def test_total_force_vanishes(full):
    g, ctx, E, F = full
    scale = float(np.sqrt((F ** 2).sum(axis=1).mean()))
    assert np.abs(F.sum(axis=0)).max() < 1e-6 * scale * g.n


def test_rigid_translation(full):
    g, ctx, E, F = full
    E2, F2 = ctx.execute_host(g.positions + np.array([0.731, -1.219, 2.003]))
    assert abs(E2 / E - 1) < 1e-6
    assert float(np.sqrt(((F2 - F) ** 2).sum() / (F ** 2).sum())) < 1e-5
