"""Finite differences of the CUDA path's own energy against its analytic
derivatives: forces (-dE/dx), and the adjoint's dE/dq, dE/dR and dE/dalpha.

The energy is evaluated in FP32 kernels with FP64 accumulation, so central
differences carry an absolute noise of a few 1e-3 kJ/mol / (2 h); the
tolerances below are that noise plus 3% of the derivative.  Entries are
drawn at random from a seeded generator (the reference's own adjoint check
uses 200 random entries with FD steps of 1e-4 A for positions)."""
import numpy as np
import pytest

from openmmcustomgbintegralforce_gb300._lib import Context
from openmmcustomgbintegralforce_gb300.globule import make_globule
from openmmcustomgbintegralforce_gb300.spec import GBModel

pytestmark = pytest.mark.gpu

REL = 3e-2


@pytest.fixture(scope="module")
def case():
    g = make_globule(400, seed=31)
    m = GBModel.charmm_gbsw()
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    out = ctx.adjoint(g.positions)
    yield g, m, ctx, out
    ctx.close()


def energy(ctx, x):
    return ctx.execute_host(x, forces=False)[0]


def check(fd, an, scale, what):
    assert abs(fd - an) <= 0.02 * scale + REL * abs(an), f"{what}: fd {fd} vs analytic {an} (scale {scale})"


def test_forces_are_minus_energy_gradient(case):
    g, _, ctx, out = case
    rng = np.random.default_rng(5)
    F = out["forces"]
    scale = float(np.sqrt((F ** 2).mean()))
    h = 1e-3
    for _ in range(16):
        i, d = int(rng.integers(g.n)), int(rng.integers(3))
        xp, xm = g.positions.copy(), g.positions.copy()
        xp[i, d] += h
        xm[i, d] -= h
        fd = -(energy(ctx, xp) - energy(ctx, xm)) / (2 * h)
        check(fd, F[i, d], scale, f"F[{i},{d}]")


def test_dEdq_and_dEdR(case):
    g, _, ctx, out = case
    rng = np.random.default_rng(6)
    for key, h, arr in (("dEdq", 1e-3, "charge"), ("dEdR", 2e-4, "radius")):
        an = out[key]
        scale = float(np.sqrt((an ** 2).mean()))
        for _ in range(8):
            i = int(rng.integers(g.n))
            q, R = g.charge.astype(np.float64).copy(), g.radius.astype(np.float64).copy()
            base = q if arr == "charge" else R
            base[i] += h
            ctx.set_particle_parameters(q, R)
            ep = energy(ctx, g.positions)
            base[i] -= 2 * h
            ctx.set_particle_parameters(q, R)
            em = energy(ctx, g.positions)
            ctx.set_particle_parameters(g.charge, g.radius)
            check((ep - em) / (2 * h), an[i], scale, f"{key}[{i}]")


def test_dEdalpha(case):
    g, m, ctx, out = case
    h = 1e-4
    for k in (0, 1):
        d0, d1 = (h, 0.0) if k == 0 else (0.0, h)
        ctx.set_global_parameters(m.alpha0 + d0, m.alpha1 + d1)
        ep = energy(ctx, g.positions)
        ctx.set_global_parameters(m.alpha0 - d0, m.alpha1 - d1)
        em = energy(ctx, g.positions)
        ctx.set_global_parameters(m.alpha0, m.alpha1)
        an = out["dEdalpha"][k]
        check((ep - em) / (2 * h), an, abs(an), f"dE/dalpha{k}")
