"""Batched evaluation (gbx_batch): uneven GBSW and GBMV molecules in one call,
first checked, then replayed from a CUDA graph.  Every molecule must match
its own single-molecule context bit for bit (same kernels, same order of
every sum), and the oracle within the usual tolerances; a replay whose table
outgrows its capacity must fall back to a checked run, not return a
truncated result."""
import numpy as np
import pytest

from openmmcustomgbintegralforce_gb300._lib import Batch, Context
from openmmcustomgbintegralforce_gb300.globule import batch_sizes, make_batch
from openmmcustomgbintegralforce_gb300.spec import GBModel, box_for
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def batch_models(gs):
    ms = []
    for k, g in enumerate(gs):
        if k % 2 == 0:
            ms.append(GBModel.charmm_gbsw(n_radial=24, lebedev=50))
        else:
            ms.append(GBModel.gbmv2(box=box_for(g.positions, margin=1.5), n_radial=24, lebedev=50))
    return ms


@pytest.fixture(scope="module")
def setup():
    gs = make_batch(batch_sizes(10, 150, 1500, seed=77), seed=77, workers=1)
    ms = batch_models(gs)
    b = Batch(ms, [g.n for g in gs])
    for c, g in zip(b.molecules, gs):
        c.set_particle_parameters(g.charge, g.radius)
    X = np.concatenate([g.positions for g in gs])
    return gs, ms, b, X


def plain(gs, ms, X=None):
    out = []
    for k, (g, m) in enumerate(zip(gs, ms)):
        c = Context(m, g.n)
        c.set_particle_parameters(g.charge, g.radius)
        out.append(c.execute_host(g.positions if X is None else X[k]))
        c.close()
    return out


def split(b, F):
    return [F[o:o + n] for o, n in zip(b.offsets, b.sizes)]


def test_batch_matches_single_contexts_bitwise(setup):
    gs, ms, b, X = setup
    ref = plain(gs, ms)
    for call in range(3):  # checked, captured, replayed
        E, F = b.execute_host(X)
        for k, (Fk, (Er, Fr)) in enumerate(zip(split(b, F), ref)):
            assert E[k] == Er, (call, k)
            assert np.array_equal(Fk, Fr), (call, k)


def test_batch_against_oracle(setup):
    gs, ms, b, X = setup
    E, F = b.execute_host(X)
    for k in (0, 1, 2, 3):
        r = O.Oracle(ms[k]).energy_forces(gs[k].positions, gs[k].charge, gs[k].radius)
        assert abs(E[k] / r["energy"] - 1) < 2e-5
        assert rel_rms(split(b, F)[k], r["forces"]) < 1e-4


def test_batch_adjoint_matches_single_contexts_and_oracle(setup):
    """gbx_batch_adjoint (every molecule's energy, dE/dx, dE/dq, dE/dR and
    dE/dalpha in one fanned-out call) equals each molecule's own
    gbx_adjoint_host bit for bit, on the first (checked) call and on a
    repeat; GBSW and GBMV-II molecules also against the oracle's adjoint."""
    gs, ms, b, X = setup
    for call in range(2):
        out = b.adjoint_host(X)
        for k, (c, g) in enumerate(zip(b.molecules, gs)):
            o, n = b.offsets[k], b.sizes[k]
            ref = c.adjoint(X[o:o + n])
            assert out["energies"][k] == ref["energy"], (call, k)
            assert np.array_equal(out["forces"][o:o + n], ref["forces"]), (call, k)
            assert np.array_equal(out["dEdq"][o:o + n], ref["dEdq"]), (call, k)
            assert np.array_equal(out["dEdR"][o:o + n], ref["dEdR"]), (call, k)
            assert np.array_equal(out["dEdalpha"][k], ref["dEdalpha"]), (call, k)
    for k in (0, 1):
        o, n = b.offsets[k], b.sizes[k]
        r = O.Oracle(ms[k]).energy_forces(gs[k].positions, gs[k].charge, gs[k].radius, adjoint=True)
        assert abs(out["energies"][k] / r["energy"] - 1) < 2e-5
        assert rel_rms(out["forces"][o:o + n], r["forces"]) < 1e-4
        assert rel_rms(out["dEdq"][o:o + n], r["dEdq"]) < 1e-4
        assert rel_rms(out["dEdR"][o:o + n], r["dEdR"]) < 1e-4
        assert np.abs(out["dEdalpha"][k] / r["dEdalpha"] - 1).max() < 1e-4


def test_replay_that_outgrows_a_table_reruns_checked(setup):
    gs, ms, b, X = setup
    b.execute_host(X)
    X2 = X.copy()
    o, n = b.offsets[0], b.sizes[0]  # a GBSW molecule: its exact table must grow
    ctr = X2[o:o + n].mean(axis=0)
    X2[o:o + n] = ctr + 1.4 * (X2[o:o + n] - ctr)
    E, F = b.execute_host(X2)
    Xs = [X2[o:o + n] for o, n in zip(b.offsets, b.sizes)]
    ref = plain(gs, ms, Xs)
    for k, (Fk, (Er, Fr)) in enumerate(zip(split(b, F), ref)):
        assert E[k] == Er, k
        assert np.array_equal(Fk, Fr), k
    b.execute_host(X)


def test_tune_keeps_results(setup):
    gs, ms, b, X = setup
    E0, F0 = b.execute_host(X)
    t = b.tune()
    assert t["streams"] >= 1 and t["chunk_divisor"] in (1, 2, 4) and t["ms_per_call"] > 0
    E1, F1 = b.execute_host(X)
    assert np.allclose(E1, E0, rtol=1e-6)
    assert rel_rms(F1, F0) < 1e-5


def test_replay_after_a_molecule_parameter_change(setup):
    """Changing one molecule's coefficients or charges through its context
    between calls: the next replay uses them (the graph is captured again)."""
    gs, ms, b, X = setup
    b.execute_host(X)
    b.execute_host(X)  # a replay
    k = 1
    c = b.molecules[k]
    m2 = ms[k].replace(alpha0=ms[k].alpha0 * 1.02)
    c.set_global_parameters(m2.alpha0, m2.alpha1)
    q2 = gs[k].charge * 0.9
    c.set_particle_parameters(q2, gs[k].radius)
    E, F = b.execute_host(X)
    ref = Context(m2, gs[k].n)
    ref.set_particle_parameters(q2, gs[k].radius)
    Er, Fr = ref.execute_host(gs[k].positions)
    ref.close()
    # the earlier tuning may have changed the quadrature chunking (summation
    # order), so the comparison with a fresh context is to rounding level
    assert abs(E[k] / Er - 1) < 1e-6 and rel_rms(split(b, F)[k], Fr) < 1e-5
    c.set_global_parameters(ms[k].alpha0, ms[k].alpha1)  # restore
    c.set_particle_parameters(gs[k].charge, gs[k].radius)
    E0, _ = b.execute_host(X)
    assert abs(E0[k] / E[k] - 1) > 1e-2


def test_non_finite_position_is_rejected_before_upload(setup):
    """A NaN among the batch's host positions is refused on the host (no
    upload, no launch), and the next call with good positions is unaffected."""
    from openmmcustomgbintegralforce_gb300._lib import GBXError

    gs, ms, b, X = setup
    E0, F0 = b.execute_host(X)
    Xbad = X.copy()
    Xbad[len(X) // 2, 1] = np.nan
    with pytest.raises(GBXError):
        b.execute_host(Xbad)
    E1, F1 = b.execute_host(X)
    assert np.array_equal(E0, E1) and np.array_equal(F0, F1)
