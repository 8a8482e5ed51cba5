"""The device entry point as an OpenMM CUDA kernel uses it, through the C ABI:

* OpenMM's precision modes: double4 positions (double precision) and a float
  energy buffer (single precision) give a float4 / double call's results;
* OpenMM's atom reordering: with gbx_set_atom_order, positions and forces in
  a permuted slot order give the unpermuted call's forces, moved to the
  slots, bit for bit (the lists keep ascending atom order);
* unchecked calls that never synchronise and are never silently wrong: atoms
  spread after the buffers were sized make the table outgrow them, and the
  next call reports GBX_ERR_STALE_RESULT with results equal to a fresh
  context's; MD-like drift grows the buffers ahead of need without a report.
"""
import numpy as np
import pytest

from openmmcustomgbintegralforce_gb300._lib import (EXEC_CHECK, EXEC_ENERGY, EXEC_ENERGY_FLOAT, EXEC_FORCES,
                                                     EXEC_POSQ_DOUBLE, Context, GBXError)
from openmmcustomgbintegralforce_gb300.globule import make_globule
from openmmcustomgbintegralforce_gb300.spec import GBModel, box_for

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

BOTH = EXEC_FORCES | EXEC_ENERGY


def device_call(ctx, pos, flags, dtype=torch.float32, edtype=torch.float64, stride=None):
    dev = torch.device("cuda:0")
    n = ctx.n
    stride = stride or n
    posq = torch.zeros((n, 4), dtype=dtype, device=dev)
    posq[:, :3] = torch.from_numpy(np.asarray(pos)).to(dev, dtype)
    force = torch.zeros(3 * stride, dtype=torch.int64, device=dev)
    energy = torch.zeros(1, dtype=edtype, device=dev)
    torch.cuda.synchronize()
    status = 0
    try:
        ctx.execute_device(posq.data_ptr(), force.data_ptr(), stride, energy.data_ptr(), flags, 0)
    except GBXError as e:
        status = e.status
    torch.cuda.synchronize()
    f = force.cpu().numpy().astype(np.float64) / 2.0 ** 32
    F = np.stack([f[:n], f[stride:stride + n], f[2 * stride:2 * stride + n]], axis=1)
    return float(energy.cpu()[0]), F, status


@pytest.fixture(scope="module")
def glob():
    return make_globule(1500, seed=61)


@pytest.mark.parametrize("name", ["gbsw", "gbmv2"])
def test_precision_modes(glob, name):
    g = glob
    m = GBModel.charmm_gbsw() if name == "gbsw" else GBModel.gbmv2(box=box_for(g.positions, margin=1.0))
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    pos32 = g.positions.astype(np.float32).astype(np.float64)
    E0, F0, _ = device_call(ctx, pos32, BOTH | EXEC_CHECK)
    # double4 positions holding the same float values: the same bits
    E1, F1, _ = device_call(ctx, pos32, BOTH | EXEC_CHECK | EXEC_POSQ_DOUBLE, dtype=torch.float64)
    assert E1 == E0 and np.array_equal(F1, F0)
    # a float energy buffer receives the double energy rounded once
    E2, F2, _ = device_call(ctx, pos32, BOTH | EXEC_CHECK | EXEC_ENERGY_FLOAT, edtype=torch.float32)
    assert E2 == float(np.float32(E0)) and np.array_equal(F2, F0)
    # and unchecked (captured) calls in both modes
    for _ in range(2):
        E3, F3, st = device_call(ctx, pos32, BOTH | EXEC_POSQ_DOUBLE | EXEC_ENERGY_FLOAT, dtype=torch.float64,
                                 edtype=torch.float32)
        assert st == 0 and E3 == float(np.float32(E0)) and np.array_equal(F3, F0)
    ctx.close()


@pytest.mark.parametrize("name", ["gbsw", "gbmv1"])
def test_atom_order(glob, name):
    g = glob
    m = GBModel.charmm_gbsw() if name == "gbsw" else GBModel.gbmv1(box=box_for(g.positions, margin=1.0))
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    E0, F0, _ = device_call(ctx, g.positions, BOTH | EXEC_CHECK)
    rng = np.random.default_rng(5)
    for check in (EXEC_CHECK, 0, 0):
        order = rng.permutation(g.n).astype(np.int32)  # slot k holds atom order[k]
        ctx.set_atom_order(order)
        stride = g.n + 7
        E1, F1, st = device_call(ctx, g.positions[order], BOTH | check, stride=stride)
        assert st == 0
        assert E1 == E0
        assert np.array_equal(F1, F0[order])
    ctx.set_atom_order(None)
    E2, F2, _ = device_call(ctx, g.positions, BOTH)
    assert E2 == E0 and np.array_equal(F2, F0)
    with pytest.raises(GBXError):
        ctx.set_atom_order(np.zeros(g.n, np.int32))
    ctx.close()


def test_unchecked_overflow_is_reported_not_silent():
    g = make_globule(2000, seed=13)
    m = GBModel.charmm_gbsw()
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    device_call(ctx, g.positions, BOTH | EXEC_CHECK)
    E0, F0, st = device_call(ctx, g.positions, BOTH)
    assert st == 0
    c = g.positions.mean(axis=0)
    wide = c + 1.6 * (g.positions - c)
    _, _, st = device_call(ctx, wide, BOTH)  # outgrows the table: lacks the volume terms, not known yet
    assert st == 0
    E2, F2, st = device_call(ctx, wide, BOTH)  # reads the published status: checked re-run, reported
    assert st == 10
    fresh = Context(m, g.n)
    fresh.set_particle_parameters(g.charge, g.radius)
    E3, F3, _ = device_call(fresh, wide, BOTH | EXEC_CHECK)
    assert E2 == E3 and np.array_equal(F2, F3)
    E4, F4, st = device_call(ctx, wide, BOTH)  # unchecked again, on the grown buffers
    assert st == 0 and E4 == E3 and np.array_equal(F4, F3)
    ctx.close()
    fresh.close()


def test_drift_grows_buffers_ahead_of_need():
    """Slow expansion (0.2 % per call, as a heating or barostat run might):
    the published table sizes grow the buffers before they are outgrown, so
    no call lacks the volume terms and none reports."""
    g = make_globule(2000, seed=17)
    m = GBModel.charmm_gbsw()
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    device_call(ctx, g.positions, BOTH | EXEC_CHECK)
    c = g.positions.mean(axis=0)
    fresh = Context(m, g.n)
    fresh.set_particle_parameters(g.charge, g.radius)
    for k in range(1, 60):
        x = c + (1.0 + 0.002 * k) * (g.positions - c)
        E, F, st = device_call(ctx, x, BOTH)
        assert st == 0, f"call {k} reported {st}"
    Ef, Ff, _ = device_call(fresh, x, BOTH | EXEC_CHECK)
    assert E == Ef and np.array_equal(F, Ff)
    ctx.close()
    fresh.close()
