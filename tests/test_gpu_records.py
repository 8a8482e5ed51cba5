"""The streamed GBSW chain rule (integral pass writes (point, in-shell atom)
records, the chain rule reads them) against the list-walking chain rule it
replaces and against the FP64 oracle, including a record buffer too small for
the call, where the device must fall back to the list walk."""
import numpy as np
import pytest

from openmmcustomgbintegralforce_gb300._lib import EXEC_ENERGY, EXEC_FORCES, Context
from openmmcustomgbintegralforce_gb300.globule import make_globule
from openmmcustomgbintegralforce_gb300.spec import GBModel
from oracle import oracle as O

pytestmark = pytest.mark.gpu

E_TOL = 2e-5
F_TOL = 1e-4


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.fixture(scope="module")
def glob():
    return make_globule(1500, seed=23)


def run(g, model, per_warp, calls=2):
    ctx = Context(model, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    ctx.set_chain_records(per_warp)
    out = [ctx.execute_host(g.positions) for _ in range(calls)]
    info = ctx.chain_records()
    ctx.close()
    return out, info


def same(a, b):
    return a[0] == b[0] and np.array_equal(a[1], b[1])


# cutoff 1.2 nm: no pair of this globule lies within 1e-6 of it, where the
# FP32 and FP64 cutoff tests can disagree (at 1.0 nm one pair does)
@pytest.mark.parametrize("model", [GBModel.charmm_gbsw(), GBModel.charmm_gbsw(cutoff=1.2),
                                   GBModel.charmm_gbsw(reference_table=True)],
                         ids=["exact_table", "cutoff_quirk", "reference_table"])
def test_records_match_list_walk_and_oracle(glob, model):
    g = glob
    (walk, _), info = run(g, model, 0)
    assert info["written"] == -1
    (auto1, auto2), info = run(g, model, -1)
    assert info["written"] > 0 and info["max_need"] <= info["per_warp"]
    # the reference table's uncapped lists can exceed the 64-entry record
    # mask; those warps walk their lists
    if not model.reference_table:
        assert info["overflowed"] == 0
    # records and list walk round every contribution the same way: same bits
    assert same(auto1, walk) and same(auto2, walk)
    ref = O.Oracle(model).energy_forces(g.positions, g.charge, g.radius)
    assert abs(auto1[0] / ref["energy"] - 1) < E_TOL
    assert rel_rms(auto1[1], ref["forces"]) < F_TOL


def test_overflowing_warps_walk_their_lists(glob):
    g = glob
    m = GBModel.charmm_gbsw()
    (walk, _), _ = run(g, m, 0)
    (small, _), info = run(g, m, 32)
    assert info["per_warp"] == 32 and info["overflowed"] > 0 and info["written"] > 0
    assert same(small, walk)


def test_fixed_size_that_fits(glob):
    g = glob
    m = GBModel.charmm_gbsw()
    (auto, _), info = run(g, m, -1)
    R = (info["max_need"] + 31) // 32 * 32
    (fixed, _), info2 = run(g, m, R)
    assert info2["per_warp"] == R and info2["overflowed"] == 0
    assert info2["written"] == info["written"]
    assert same(fixed, auto)


def test_energy_only_skips_chain(glob):
    import torch
    g = glob
    m = GBModel.charmm_gbsw()
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    E_host, _ = ctx.execute_host(g.positions)
    dev = torch.device("cuda:0")
    posq = torch.zeros((g.n, 4), dtype=torch.float32, device=dev)
    posq[:, :3] = torch.from_numpy(g.positions.astype(np.float32)).to(dev)
    energy = torch.zeros(1, dtype=torch.float64, device=dev)
    force = torch.zeros(3 * g.n, dtype=torch.int64, device=dev)
    ctx.execute_device(posq.data_ptr(), force.data_ptr(), g.n, energy.data_ptr(), EXEC_ENERGY, 0)
    torch.cuda.synchronize()
    assert float(energy.item()) == pytest.approx(E_host, rel=1e-12)
    assert int(force.abs().sum().item()) == 0
    energy.zero_()
    ctx.execute_device(posq.data_ptr(), force.data_ptr(), g.n, energy.data_ptr(), EXEC_ENERGY | EXEC_FORCES, 0)
    torch.cuda.synchronize()
    assert float(energy.item()) == pytest.approx(E_host, rel=1e-12)
    assert int(force.abs().sum().item()) > 0
    ctx.close()
