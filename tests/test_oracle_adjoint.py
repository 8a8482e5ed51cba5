"""The FP64 oracle's analytic adjoint (dE/dx, dE/dq, dE/dR_in, dE/dalpha)
against FP64 central differences of its own energy, for all three volume
models.  The reference returns forces only, so these differences are what
pin the adjoint the device's gradients are checked against.

The lookup table's membership tests make the energy piecewise smooth: a
step that moves a cell sample across an atom's pad changes a list and the
energy jumps.  The seeded entries below were drawn once; none of their
+-h steps crosses a pad.
"""
import numpy as np
import pytest

from openmmcustomgbintegralforce_gb300.globule import make_globule
from openmmcustomgbintegralforce_gb300.spec import GBModel, box_for
from oracle import oracle as O


def models(g):
    box = box_for(g.positions, margin=1.0)
    return {"gbsw": GBModel.charmm_gbsw(), "gbmv1": GBModel.gbmv1(box=box), "gbmv2": GBModel.gbmv2(box=box)}


@pytest.fixture(scope="module")
def glob():
    return make_globule(250, seed=47)


@pytest.mark.parametrize("name", ["gbsw", "gbmv1", "gbmv2"])
def test_oracle_adjoint_vs_central_differences(glob, name):
    g = glob
    m = models(g)[name]
    orc = O.Oracle(m)
    ref = orc.energy_forces(g.positions, g.charge, g.radius, adjoint=True)
    rng = np.random.default_rng(3)

    def E(pos=g.positions, q=g.charge, R=g.radius, model=None):
        o = orc if model is None else O.Oracle(model)
        return o.energy_forces(pos, q, R)["energy"]

    def close(fd, an, scale, what):
        assert abs(fd - an) <= 1e-6 * scale + 1e-5 * abs(an), f"{name} {what}: fd {fd} vs analytic {an}"

    h = 1e-6
    F = ref["forces"]
    fs = float(np.sqrt((F ** 2).mean()))
    for flat in rng.choice(3 * g.n, size=8, replace=False):
        i, d = int(flat) // 3, int(flat) % 3
        xp, xm = g.positions.copy(), g.positions.copy()
        xp[i, d] += h
        xm[i, d] -= h
        close(-(E(pos=xp) - E(pos=xm)) / (2 * h), F[i, d], fs, f"F[{i},{d}]")
    for key, which in (("dEdq", "q"), ("dEdR", "R")):
        an = ref[key]
        sc = float(np.sqrt((an ** 2).mean()))
        for i in rng.choice(g.n, size=6, replace=False):
            i = int(i)
            p = (g.charge if which == "q" else g.radius).astype(np.float64).copy()
            p[i] += h
            ep = E(q=p) if which == "q" else E(R=p)
            p[i] -= 2 * h
            em = E(q=p) if which == "q" else E(R=p)
            close((ep - em) / (2 * h), an[i], sc, f"{key}[{i}]")
    for k, par in enumerate(("alpha0", "alpha1")):
        base = getattr(m, par)
        ep = E(model=m.replace(**{par: base + h}))
        em = E(model=m.replace(**{par: base - h}))
        close((ep - em) / (2 * h), ref["dEdalpha"][k], abs(ref["dEdalpha"][k]), par)
