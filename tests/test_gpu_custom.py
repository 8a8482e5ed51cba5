"""CharmmGBMVForce expressions compiled into device code (gbx_create_custom),
through the C ABI, against the FP64 custom-expression oracle
(oracle/custom.py, itself pinned to the canonical oracle):

* the canonical set written as user expressions gives the canonical
  context's results;
* a set outside it (a second computed value, globals, a nonpolar
  single-particle term, a Lepton definition) for the GBMV-II and
  GBSW-integral classes, with and without a cutoff;
* coordinates in a computed value and a single-particle term, exclusions
  skipped by a ParticlePair term only, and energy derivatives by globals
  (addEnergyParameterDerivative);
* tabulated functions (Continuous1DFunction) in a computed value, a
  single-particle term and a pair term;
* the Lepton function set (FP64 in the values and single-particle terms,
  FP32 fast math in the pair terms);
* the pair kernel's tile edges: 1, 2, 31, 33, 64 and 97 particles with
  exclusions inside and across tiles, with and without a cutoff;
* a global parameter update, bit-reproducible calls, and a refused
  expression.

Tolerances as the parity suite: energy 2e-5 relative, forces 1e-4 relative
RMS, the first computed value (the Born radius) 1e-4 maximum relative.
"""
import copy

import numpy as np
import pytest

from openmmcustomgbintegralforce_gb300._lib import Context, CustomContext, GBXError
from openmmcustomgbintegralforce_gb300.globule import make_globule
from openmmcustomgbintegralforce_gb300.spec import GBModel, box_for
from oracle.custom import CustomOracle
from openmmcustomgbintegralforce_gb300.expression_sets import (CANONICAL, EXTENDED, FUNCTIONS, MODIFIED, TABULATED,
                                                               extended_exclusions, modified_params)

pytestmark = pytest.mark.gpu

E_TOL, F_TOL, B_TOL = 2e-5, 1e-4, 1e-4


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.fixture(scope="module")
def glob():
    return make_globule(1000, seed=73)


def model_of(cls, g, **kw):
    if cls == "gbmv2":
        return GBModel.gbmv2(box=box_for(g.positions, margin=1.0), **kw)
    return GBModel.gbsw_integral(**kw)


def test_canonical_set_matches_canonical_context(glob):
    g = glob
    m = model_of("gbmv2", g)
    ref = Context(m, g.n)
    ref.set_particle_parameters(g.charge, g.radius)
    E0, F0 = ref.execute_host(g.positions)
    ctx = CustomContext(m, g.n, CANONICAL)
    ctx.set_custom_parameters(np.stack([g.charge, g.radius], axis=1))
    E1, F1 = ctx.execute_host(g.positions)
    print(f"canonical as expressions: energy {abs(E1 / E0 - 1):.2e} forces {rel_rms(F1, F0):.2e}")
    assert abs(E1 / E0 - 1) < E_TOL
    assert rel_rms(F1, F0) < F_TOL
    assert np.abs(ctx.born_radii() / ref.born_radii() - 1).max() < B_TOL
    ctx.close()
    ref.close()


@pytest.mark.parametrize("cls,cutoff", [("gbmv2", 0.0), ("gbsw_integral", 0.0), ("gbmv2", 1.2)])
def test_modified_set_vs_oracle(glob, cls, cutoff):
    g = glob
    m = model_of(cls, g, cutoff=cutoff)
    P = modified_params(g)
    ctx = CustomContext(m, g.n, MODIFIED)
    ctx.set_custom_parameters(P)
    E, F = ctx.execute_host(g.positions)
    E2, F2 = ctx.execute_host(g.positions)
    assert E2 == E and np.array_equal(F2, F)
    ref = CustomOracle(m, MODIFIED).energy_forces(g.positions, P)
    print(f"{cls} cutoff={cutoff}: energy {abs(E / ref['energy'] - 1):.2e} forces {rel_rms(F, ref['forces']):.2e}")
    assert abs(E / ref["energy"] - 1) < E_TOL
    assert rel_rms(F, ref["forces"]) < F_TOL
    assert np.abs(ctx.born_radii() / ref["values"][0] - 1).max() < B_TOL
    ctx.close()


@pytest.mark.parametrize("cls", ["gbmv2", "gbsw_integral"])
def test_modified_set_cutoff_periodic_vs_oracle(cls):
    """The modified set under CutoffPeriodic: integrals on the box-sampled
    table with minimum-image point distances, pair terms by minimum image,
    in a box barely wider than twice the cutoff (the box changes the
    result)."""
    from openmmcustomgbintegralforce_gb300.spec import TABLE_PERIODIC

    g = make_globule(600, seed=23)
    pos = g.positions - g.positions.min(axis=0)
    box = (2.8, 2.8, 2.9)
    if cls == "gbmv2":
        m = GBModel.gbmv2(box=box, cutoff=1.3, periodic=True)
    else:
        m = GBModel.gbsw_integral(box=box, cutoff=1.3, periodic=True, table_mode=TABLE_PERIODIC)
    P = modified_params(g)
    ctx = CustomContext(m, g.n, MODIFIED)
    ctx.set_custom_parameters(P)
    E, F = ctx.execute_host(pos)
    ref = CustomOracle(m, MODIFIED).energy_forces(pos, P)
    print(f"{cls} periodic: energy {abs(E / ref['energy'] - 1):.2e} forces {rel_rms(F, ref['forces']):.2e}")
    assert abs(E / ref["energy"] - 1) < E_TOL
    assert rel_rms(F, ref["forces"]) < F_TOL
    flat = CustomOracle(m.replace(periodic=False), MODIFIED).energy_forces(pos, P)
    assert abs(flat["energy"] / ref["energy"] - 1) > 1e-4
    ctx.close()


def test_global_update(glob):
    g = glob
    m = model_of("gbmv2", g)
    P = modified_params(g)
    ctx = CustomContext(m, g.n, MODIFIED)
    ctx.set_custom_parameters(P)
    ctx.execute_host(g.positions)
    ctx.set_custom_global("eps", 4.0)
    E, F = ctx.execute_host(g.positions)
    mod = dict(MODIFIED, globals=dict(MODIFIED["globals"], eps=4.0))
    ref = CustomOracle(m, mod).energy_forces(g.positions, P)
    assert abs(E / ref["energy"] - 1) < E_TOL
    assert rel_rms(F, ref["forces"]) < F_TOL
    with pytest.raises(GBXError):
        ctx.set_custom_global("no_such", 1.0)
    ctx.close()


def test_refused_expression(glob):
    g = glob
    bad = copy.deepcopy(MODIFIED)
    bad["terms"] = [("q^2/Bx", 0)]
    with pytest.raises(GBXError):
        CustomContext(model_of("gbmv2", g), g.n, bad)


def test_kernel_mirror_compiles_a_non_canonical_force(glob):
    """The Python mirror of the GBMV kernel takes a force outside the
    canonical set through the compiled path."""
    from openmmcustomgbintegralforce_gb300 import api

    g = glob
    f = api.CharmmGBMVForce()
    for p in MODIFIED["params"]:
        f.addPerParticleParameter(p)
    for k, v in MODIFIED["globals"].items():
        f.addGlobalParameter(k, v)
    for name, order in MODIFIED["integrals"]:
        f.addGBIntegral(name, [order], [])
    for name, e in MODIFIED["values"]:
        f.addComputedValue(name, e, api.SingleParticle)
    for e, t in MODIFIED["terms"]:
        f.addEnergyTerm(e, api.SingleParticle if t == 0 else api.ParticlePairNoExclusions)
    f.setGBIntegralType(api.GBMVIntegralTypeII)
    P = modified_params(g)
    for row in P:
        f.addParticle(list(row))
    box = box_for(g.positions, margin=1.0)
    k = api.CalcCharmmGBMVForceKernel(box=box)
    k.initialize(g.n, f)
    E, F = k.execute(g.positions)
    ref = CustomOracle(GBModel.gbmv2(box=box), MODIFIED).energy_forces(g.positions, P)
    assert abs(E / ref["energy"] - 1) < E_TOL
    assert rel_rms(F, ref["forces"]) < F_TOL


@pytest.mark.parametrize("cls", ["gbmv2", "gbsw_integral"])
def test_extended_set_vs_oracle(glob, cls):
    """Coordinates, exclusions and parameter derivatives: energy, forces,
    the computed values and dE/dg against the oracle; the exclusions
    change the result; repeated calls are bit-identical."""
    g = glob
    m = model_of(cls, g)
    P = np.stack([g.charge, g.radius], axis=1)
    ext = dict(EXTENDED, exclusions=extended_exclusions(g.n))
    ctx = CustomContext(m, g.n, ext)
    ctx.set_custom_parameters(P)
    E, F = ctx.execute_host(g.positions)
    pd = ctx.param_derivs()
    E2, F2 = ctx.execute_host(g.positions)
    assert E2 == E and np.array_equal(F2, F) and np.array_equal(ctx.param_derivs(), pd)
    ref = CustomOracle(m, ext).energy_forces(g.positions, P)
    print(f"{cls} extended: energy {abs(E / ref['energy'] - 1):.2e} forces {rel_rms(F, ref['forces']):.2e} "
          f"param derivs {np.abs(pd / ref['param_derivs'] - 1).max():.2e}")
    assert abs(E / ref["energy"] - 1) < E_TOL
    assert rel_rms(F, ref["forces"]) < F_TOL
    assert np.abs(ctx.born_radii() / ref["values"][0] - 1).max() < B_TOL
    assert np.abs(pd / ref["param_derivs"] - 1).max() < E_TOL * 5
    plain = CustomOracle(m, EXTENDED).energy_forces(g.positions, P)
    assert abs(plain["energy"] / E - 1) > 1e-4
    ctx.close()


def test_kernel_mirror_exclusions_and_param_derivs(glob):
    """The GBMV kernel mirror passes the force's exclusions and energy
    parameter derivatives to the compiled path."""
    from openmmcustomgbintegralforce_gb300 import api

    g = glob
    f = api.CharmmGBMVForce()
    for p in EXTENDED["params"]:
        f.addPerParticleParameter(p)
    for k, v in EXTENDED["globals"].items():
        f.addGlobalParameter(k, v)
    for name in EXTENDED["param_derivs"]:
        f.addEnergyParameterDerivative(name)
    for name, order in EXTENDED["integrals"]:
        f.addGBIntegral(name, [order], [])
    for name, e in EXTENDED["values"]:
        f.addComputedValue(name, e, api.SingleParticle)
    kinds = {0: api.SingleParticle, 1: api.ParticlePair, 2: api.ParticlePairNoExclusions}
    for e, t in EXTENDED["terms"]:
        f.addEnergyTerm(e, kinds[t])
    excl = extended_exclusions(g.n)
    for i, j in excl:
        f.addExclusion(i, j)
    f.setGBIntegralType(api.GBMVIntegralTypeII)
    P = np.stack([g.charge, g.radius], axis=1)
    for row in P:
        f.addParticle(list(row))
    box = box_for(g.positions, margin=1.0)
    k = api.CalcCharmmGBMVForceKernel(box=box)
    k.initialize(g.n, f)
    E, F = k.execute(g.positions)
    pd = k.getEnergyParameterDerivatives()
    ref = CustomOracle(GBModel.gbmv2(box=box), dict(EXTENDED, exclusions=excl)).energy_forces(g.positions, P)
    assert abs(E / ref["energy"] - 1) < E_TOL
    assert rel_rms(F, ref["forces"]) < F_TOL
    assert sorted(pd) == sorted(EXTENDED["param_derivs"])
    for n, v in zip(EXTENDED["param_derivs"], ref["param_derivs"]):
        assert abs(pd[n] / v - 1) < E_TOL * 5


@pytest.mark.parametrize("cls", ["gbmv2", "gbsw_integral"])
def test_tabulated_set_vs_oracle(glob, cls):
    """Natural cubic splines evaluated on the device (FP64 in the values,
    FP32 in the pair terms) against scipy's in the oracle."""
    g = glob
    m = model_of(cls, g)
    P = np.stack([g.charge, g.radius], axis=1)
    ctx = CustomContext(m, g.n, TABULATED)
    ctx.set_custom_parameters(P)
    E, F = ctx.execute_host(g.positions)
    E2, F2 = ctx.execute_host(g.positions)
    assert E2 == E and np.array_equal(F2, F)
    ref = CustomOracle(m, TABULATED).energy_forces(g.positions, P)
    print(f"{cls} tabulated: energy {abs(E / ref['energy'] - 1):.2e} forces {rel_rms(F, ref['forces']):.2e}")
    assert abs(E / ref["energy"] - 1) < E_TOL
    assert rel_rms(F, ref["forces"]) < F_TOL
    assert np.abs(ctx.born_radii() / ref["values"][0] - 1).max() < B_TOL
    ctx.close()


def test_kernel_mirror_tabulated_functions(glob):
    """The GBMV kernel mirror passes Continuous1DFunction tables to the
    compiled path."""
    from openmmcustomgbintegralforce_gb300 import api

    g = glob
    f = api.CharmmGBMVForce()
    for p in TABULATED["params"]:
        f.addPerParticleParameter(p)
    for k, v in TABULATED["globals"].items():
        f.addGlobalParameter(k, v)
    for name, (vals, lo, hi) in TABULATED["functions"].items():
        f.addTabulatedFunction(name, api.Continuous1DFunction(vals, lo, hi))
    for name, order in TABULATED["integrals"]:
        f.addGBIntegral(name, [order], [])
    for name, e in TABULATED["values"]:
        f.addComputedValue(name, e, api.SingleParticle)
    for e, t in TABULATED["terms"]:
        f.addEnergyTerm(e, api.SingleParticle if t == 0 else api.ParticlePairNoExclusions)
    f.setGBIntegralType(api.GBMVIntegralTypeII)
    P = np.stack([g.charge, g.radius], axis=1)
    for row in P:
        f.addParticle(list(row))
    box = box_for(g.positions, margin=1.0)
    k = api.CalcCharmmGBMVForceKernel(box=box)
    k.initialize(g.n, f)
    E, F = k.execute(g.positions)
    ref = CustomOracle(GBModel.gbmv2(box=box), TABULATED).energy_forces(g.positions, P)
    assert abs(E / ref["energy"] - 1) < E_TOL
    assert rel_rms(F, ref["forces"]) < F_TOL


@pytest.mark.parametrize("n", [1, 2, 31, 33, 64, 97])
@pytest.mark.parametrize("cutoff", [0.0, 0.9])
def test_tile_edges_vs_oracle(n, cutoff):
    """The pair kernel's 32-particle tiles at ragged and exact sizes (a lone
    particle, part tiles, whole tiles, a diagonal tile only), with
    exclusions inside and across tiles and with a cutoff, against the
    oracle."""
    g = make_globule(max(n, 2), seed=300 + n)
    pos = g.positions[:n]
    P = np.stack([g.charge[:n], g.radius[:n]], axis=1)
    # exclusions between tiles too: every 7th particle with the one 40 places on
    excl = extended_exclusions(n) + [(i, i + 40) for i in range(0, n - 40, 7)]
    ext = dict(EXTENDED, exclusions=excl)
    m = GBModel.gbmv2(box=box_for(pos, margin=1.0), cutoff=cutoff)
    ctx = CustomContext(m, n, ext)
    ctx.set_custom_parameters(P)
    E, F = ctx.execute_host(pos)
    pd = ctx.param_derivs()
    ref = CustomOracle(m, ext).energy_forces(pos, P)
    tolE = E_TOL if cutoff == 0.0 else 1e-4  # pairs within FP32 rounding of the cutoff
    assert abs(E / ref["energy"] - 1) < tolE, (E, ref["energy"])
    assert rel_rms(F, ref["forces"]) < (F_TOL if cutoff == 0.0 else 1e-3)
    assert np.abs(pd / ref["param_derivs"] - 1).max() < 1e-4
    ctx.close()


@pytest.mark.parametrize("cls", ["gbmv2", "gbsw_integral"])
def test_function_set_vs_oracle(glob, cls):
    """Every Lepton function in generated code against the oracle."""
    g = glob
    m = model_of(cls, g)
    P = np.stack([g.charge, g.radius], axis=1)
    ctx = CustomContext(m, g.n, FUNCTIONS)
    ctx.set_custom_parameters(P)
    E, F = ctx.execute_host(g.positions)
    ref = CustomOracle(m, FUNCTIONS).energy_forces(g.positions, P)
    print(f"{cls} functions: energy {abs(E / ref['energy'] - 1):.2e} forces {rel_rms(F, ref['forces']):.2e}")
    assert abs(E / ref["energy"] - 1) < E_TOL
    assert rel_rms(F, ref["forces"]) < F_TOL
    assert np.abs(ctx.born_radii() / ref["values"][0] - 1).max() < B_TOL
    ctx.close()
