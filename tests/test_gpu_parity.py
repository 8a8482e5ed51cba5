"""CUDA path vs the FP64 oracle and the reference's golden vectors, through
the C ABI.  Tolerances (FP32 arithmetic, FP64 Born-radius assembly):

* lookup tables: bit-exact (counts and ascending lists)
* Born radii: max relative error <= 1e-4
* energy: relative error <= 2e-5
* forces: relative RMS error <= 1e-4 (the accuracy target of the path)
"""
import numpy as np
import pytest

from openmmcustomgbintegralforce_gb300._lib import Context, GBXError
from openmmcustomgbintegralforce_gb300.globule import make_globule
from openmmcustomgbintegralforce_gb300.spec import GBModel, box_for
from oracle import oracle as O
from tests.conftest import golden

pytestmark = pytest.mark.gpu

E_TOL = 2e-5
F_TOL = 1e-4
B_TOL = 1e-4


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def models_for(g):
    box = box_for(g.positions, margin=1.0)
    return {
        "charmm_gbsw": GBModel.charmm_gbsw(),
        "gbsw_integral": GBModel.gbsw_integral(),
        "gbmv1": GBModel.gbmv1(box=box),
        "gbmv2": GBModel.gbmv2(box=box),
    }


@pytest.fixture(scope="module")
def glob1000():
    return make_globule(1000, seed=11)


@pytest.mark.parametrize("name", ["charmm_gbsw", "gbsw_integral", "gbmv1", "gbmv2"])
def test_table_bit_exact(glob1000, name):
    g = glob1000
    m = models_for(g)[name]
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    ctx.execute_host(g.positions)
    t = ctx.lookup_table()
    ref = O.Oracle(m).table(g.positions, g.radius)
    assert np.array_equal(t["dims"], ref["dims"])
    assert np.array_equal(t["min"], ref["min"])
    assert np.array_equal(t["counts"], ref["counts"])
    assert np.array_equal(t["atoms"], ref["atoms"])


@pytest.mark.parametrize("name", ["charmm_gbsw", "gbsw_integral", "gbmv1", "gbmv2"])
def test_energy_forces_born_vs_oracle(glob1000, name):
    g = glob1000
    m = models_for(g)[name]
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    E, F = ctx.execute_host(g.positions)
    ref = O.Oracle(m).energy_forces(g.positions, g.charge, g.radius)
    B = ctx.born_radii()
    I = ctx.integrals()
    assert np.abs(B / ref["born"] - 1).max() < B_TOL
    assert np.abs(I - ref["integrals"]).max() < 1e-5 * np.abs(ref["integrals"]).max()
    assert abs(E / ref["energy"] - 1) < E_TOL
    assert rel_rms(F, ref["forces"]) < F_TOL


def test_charmm_gbsw_vs_reference_golden():
    """The reference's own CharmmGBSWForce outputs (1,000-atom globule)."""
    gd = golden("gbsw_1000.npz")
    n = len(gd["radius"])
    ctx = Context(GBModel.charmm_gbsw(), n)
    ctx.set_particle_parameters(gd["charge"], gd["radius"])
    E, F = ctx.execute_host(gd["positions"])
    assert abs(E / float(gd["energy"]) - 1) < E_TOL
    assert rel_rms(F, gd["forces"]) < F_TOL
    assert np.abs(ctx.born_radii() / gd["born"] - 1).max() < B_TOL


def test_charmm_gbsw_table_vs_reference_golden():
    gd = golden("gbsw_200.npz")
    n = len(gd["radius"])
    ctx = Context(GBModel.charmm_gbsw(), n)
    ctx.set_particle_parameters(gd["charge"], gd["radius"])
    ctx.execute_host(gd["positions"])
    t = ctx.lookup_table()
    assert np.array_equal(t["dims"], gd["table_dims"])
    assert np.array_equal(t["counts"], gd["table_counts"])
    assert np.array_equal(t["atoms"], gd["table_atoms"])


def test_cutoff_quirk_vs_reference_golden():
    gd = golden("gbsw_200_cutoff1.npz")
    n = len(gd["radius"])
    ctx = Context(GBModel.charmm_gbsw(cutoff=float(gd["cutoff"])), n)
    ctx.set_particle_parameters(gd["charge"], gd["radius"])
    E, F = ctx.execute_host(gd["positions"])
    assert abs(E / float(gd["energy"]) - 1) < E_TOL
    assert rel_rms(F, gd["forces"]) < F_TOL


@pytest.mark.parametrize("tag", ["gbsw", "gbmv1", "gbmv2"])
def test_integral_classes_vs_reference_golden(tag):
    gd = golden("integrals_600.npz")
    box = tuple(gd["box"])
    m = {"gbsw": GBModel.gbsw_integral(), "gbmv1": GBModel.gbmv1(box=box), "gbmv2": GBModel.gbmv2(box=box)}[tag]
    n = len(gd["radius"])
    ctx = Context(m, n)
    ctx.set_particle_parameters(gd["charge"], gd["radius"])
    ctx.execute_host(gd["positions"])
    t = ctx.lookup_table()
    assert np.array_equal(t["counts"], gd[f"{tag}_table_counts"])
    assert np.array_equal(t["atoms"], gd[f"{tag}_table_atoms"])
    I = ctx.integrals()
    ref = gd[f"{tag}_integrals"]
    assert np.abs(I - ref).max() < 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("cutoff", [0.0, 1.0])
def test_exact_table_matches_reference_table(glob1000, cutoff):
    """The exact GBSW table yields the same volumes as the reference's
    standalone table: identical to FP32 rounding of the product order."""
    g = glob1000
    m = GBModel.charmm_gbsw(n_radial=24, lebedev=50, cutoff=cutoff)
    a = Context(m, g.n)
    b = Context(m.replace(reference_table=True), g.n)
    for c in (a, b):
        c.set_particle_parameters(g.charge, g.radius)
    Ea, Fa = a.execute_host(g.positions)
    Eb, Fb = b.execute_host(g.positions)
    assert abs(Ea / Eb - 1) < 1e-6
    assert rel_rms(Fa, Fb) < 1e-5
    assert np.abs(a.born_radii() / b.born_radii() - 1).max() < 1e-5
    # exact-table work is a fraction of the reference's list work
    a.execute_host(g.positions, count_work=True)
    b.execute_host(g.positions, count_work=True)
    assert a.work()["volume_evals"] < 0.5 * b.work()["volume_evals"]
    # the reference table is still available, bit-exact, after an exact-table run
    t = a.lookup_table()
    ref = O.Oracle(m).table(g.positions, g.radius)
    assert np.array_equal(t["counts"], ref["counts"]) and np.array_equal(t["atoms"], ref["atoms"])


def test_bitwise_deterministic(glob1000):
    g = glob1000
    ctx = Context(GBModel.charmm_gbsw(), g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    E1, F1 = ctx.execute_host(g.positions)
    E2, F2 = ctx.execute_host(g.positions)
    assert E1 == E2
    assert np.array_equal(F1, F2)


def test_repeated_calls_do_not_accumulate(glob1000):
    """The reference engine keeps stale accumulators between calls
    (CharmmReferenceGBSW.cpp:235,562); each execute here is independent."""
    g = glob1000
    ctx = Context(GBModel.charmm_gbsw(), g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    rng = np.random.default_rng(0)
    x2 = g.positions + rng.normal(0, 0.001, size=g.positions.shape)
    ctx.execute_host(x2)
    E, F = ctx.execute_host(g.positions)
    ref = O.Oracle(GBModel.charmm_gbsw()).energy_forces(g.positions, g.charge, g.radius)
    assert abs(E / ref["energy"] - 1) < E_TOL
    assert rel_rms(F, ref["forces"]) < F_TOL


@pytest.mark.parametrize("n", [1, 2, 3, 33])
def test_small_systems(n):
    g = make_globule(max(n, 1), seed=2)
    m = GBModel.charmm_gbsw()
    ctx = Context(m, n)
    ctx.set_particle_parameters(g.charge[:n], g.radius[:n])
    E, F = ctx.execute_host(g.positions[:n])
    ref = O.Oracle(m).energy_forces(g.positions[:n], g.charge[:n], g.radius[:n])
    assert abs(E - ref["energy"]) <= E_TOL * abs(ref["energy"]) + 1e-6
    assert np.abs(F - ref["forces"]).max() <= 1e-4 * (np.abs(ref["forces"]).max() + 1e-3)


def test_invalid_inputs_raise():
    g = make_globule(10, seed=1)
    ctx = Context(GBModel.charmm_gbsw(), 10)
    bad = g.radius.copy()
    bad[3] = -1.0
    with pytest.raises(GBXError):
        ctx.set_particle_parameters(g.charge, bad)
    x = g.positions.copy()
    x[0, 0] = np.nan
    ctx.set_particle_parameters(g.charge, g.radius)
    with pytest.raises(GBXError):
        ctx.execute_host(x)
    with pytest.raises(GBXError):
        ctx.set_particle_parameters(g.charge[:5], g.radius[:5])


def test_adjoint_vs_oracle(glob1000):
    g = glob1000
    m = GBModel.charmm_gbsw()
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    out = ctx.adjoint(g.positions)
    ref = O.Oracle(m).energy_forces(g.positions, g.charge, g.radius, adjoint=True)
    assert abs(out["energy"] / ref["energy"] - 1) < E_TOL
    assert rel_rms(out["forces"], ref["forces"]) < F_TOL
    assert rel_rms(out["dEdq"], ref["dEdq"]) < 1e-4
    assert rel_rms(out["dEdR"], ref["dEdR"]) < 1e-4
    assert np.abs(out["dEdalpha"] / ref["dEdalpha"] - 1).max() < 1e-4


def test_api_mirror_kernels(glob1000):
    from openmmcustomgbintegralforce_gb300 import api

    g = glob1000
    f = api.CharmmGBSWForce()
    for i in range(g.n):
        f.addParticle(g.charge[i], g.radius[i], 1.0)
    k = api.CalcCharmmGBSWForceKernel()
    k.initialize(g.n, f)
    E, F = k.execute(g.positions)
    ref = O.Oracle(GBModel.charmm_gbsw()).energy_forces(g.positions, g.charge, g.radius)
    assert abs(E / ref["energy"] - 1) < E_TOL
    # updateParametersInContext
    f.setParticleParameters(0, 0.0, g.radius[0], 1.0)
    f.updateParametersInContext(k)
    q = g.charge.copy()
    q[0] = 0.0
    E2, _ = k.execute(g.positions)
    ref2 = O.Oracle(GBModel.charmm_gbsw()).energy_forces(g.positions, q, g.radius)
    assert abs(E2 / ref2["energy"] - 1) < E_TOL

    gm = api.canonical_gbmv_force(api.GBMVIntegralTypeII)
    for i in range(g.n):
        gm.addParticle([g.charge[i], g.radius[i]])
    box = box_for(g.positions, margin=1.0)
    kk = api.CalcCharmmGBMVForceKernel(box=box)
    kk.initialize(g.n, gm)
    E3, F3 = kk.execute(g.positions)
    ref3 = O.Oracle(GBModel.gbmv2(box=box)).energy_forces(g.positions, g.charge, g.radius)
    assert abs(E3 / ref3["energy"] - 1) < E_TOL
    assert rel_rms(F3, ref3["forces"]) < F_TOL


def test_device_buffers_match_host_path(glob1000):
    torch = pytest.importorskip("torch")
    g = glob1000
    ctx = Context(GBModel.charmm_gbsw(), g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    E, F = ctx.execute_host(g.positions)
    dev = torch.device("cuda:0")
    posq = torch.zeros((g.n, 4), dtype=torch.float32, device=dev)
    posq[:, :3] = torch.from_numpy(g.positions.astype(np.float32)).to(dev)
    stride = ((g.n + 31) // 32) * 32
    force = torch.zeros(3 * stride, dtype=torch.int64, device=dev)
    energy = torch.zeros(1, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    ctx.execute_device(posq.data_ptr(), force.data_ptr(), stride, energy.data_ptr(), 1 | 2 | 4,
                       torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    fx = force.cpu().numpy().astype(np.float64) / 2.0 ** 32
    Fd = np.stack([fx[:g.n], fx[stride:stride + g.n], fx[2 * stride:2 * stride + g.n]], axis=1)
    assert float(energy.cpu()[0]) == E
    assert np.array_equal(Fd, F)


@pytest.mark.parametrize("policy", ["exact_table", "reference_table"])
def test_isolated_atom_known_answer(policy):
    """Analytic pin on the device: isolated atoms' integrals and Born radii
    equal the 1-D Gauss-Legendre sums of the switching polynomial
    (tests/kat_isolated.py), whichever table the context integrates on."""
    from tests.kat_isolated import expected_born, expected_integrals, isolated_system

    m = GBModel.charmm_gbsw(reference_table=(policy == "reference_table"))
    pos, radius = isolated_system([0.12, 0.17, 0.18])
    ctx = Context(m, len(radius))
    ctx.set_particle_parameters(np.full(len(radius), 0.1), radius)
    ctx.execute_host(pos)
    I4, I7 = expected_integrals(m, radius)
    got = ctx.integrals()
    assert np.abs(got[0] / I4 - 1).max() < 1e-6
    assert np.abs(got[1] / I7 - 1).max() < 1e-6
    assert np.abs(ctx.born_radii() / expected_born(m, I4, I7) - 1).max() < 1e-6
    ctx.close()


def test_non_finite_position_is_rejected_and_context_recovers():
    g = make_globule(300, seed=5)
    m = GBModel.charmm_gbsw()
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    E0, F0 = ctx.execute_host(g.positions)
    bad = g.positions.copy()
    bad[17, 1] = np.nan
    with pytest.raises(GBXError):
        ctx.execute_host(bad)
    E1, F1 = ctx.execute_host(g.positions)
    assert E1 == E0 and np.array_equal(F1, F0)
    ctx.close()


def test_host_call_after_the_table_outgrows_its_buffers():
    """A host call sized on one geometry, then given atoms spread 1.6x wider
    (the exact table needs ~4x the cells): the unchecked run never indexes
    the oversized table, the call detects the overflow and re-runs checked,
    and the result equals a fresh context's bit for bit."""
    g = make_globule(2000, seed=13)
    m = GBModel.charmm_gbsw()
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    ctx.execute_host(g.positions)
    ctx.execute_host(g.positions)
    c = g.positions.mean(axis=0)
    wide = c + 1.6 * (g.positions - c)
    E1, F1 = ctx.execute_host(wide)
    fresh = Context(m, g.n)
    fresh.set_particle_parameters(g.charge, g.radius)
    E2, F2 = fresh.execute_host(wide)
    assert E1 == E2 and np.array_equal(F1, F2)
    E3, F3 = ctx.execute_host(g.positions)  # and back
    E4, F4 = fresh.execute_host(g.positions)
    assert E3 == E4 and np.array_equal(F3, F4)
    ctx.close()
    fresh.close()


def test_device_call_graph_replay_matches_checked_calls():
    """Unchecked device calls run as one captured CUDA graph: replays into the
    same buffers, a recapture for new buffers and a recapture after a
    parameter change all give a checked call's bits."""
    torch = pytest.importorskip("torch")
    from openmmcustomgbintegralforce_gb300._lib import EXEC_CHECK, EXEC_ENERGY, EXEC_FORCES

    g = make_globule(1500, seed=21)
    m = GBModel.charmm_gbsw()
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    dev = torch.device("cuda:0")
    posq = torch.zeros((g.n, 4), dtype=torch.float32, device=dev)
    posq[:, :3] = torch.from_numpy(g.positions.astype(np.float32)).to(dev)

    def run(flags, force=None, energy=None):
        force = torch.zeros(3 * g.n, dtype=torch.int64, device=dev) if force is None else force.zero_()
        energy = torch.zeros(1, dtype=torch.float64, device=dev) if energy is None else energy.zero_()
        torch.cuda.synchronize()
        ctx.execute_device(posq.data_ptr(), force.data_ptr(), g.n, energy.data_ptr(), flags, 0)
        torch.cuda.synchronize()
        return float(energy.item()), force.cpu().numpy()

    both = EXEC_FORCES | EXEC_ENERGY
    E0, F0 = run(both | EXEC_CHECK)
    f = torch.zeros(3 * g.n, dtype=torch.int64, device=dev)
    e = torch.zeros(1, dtype=torch.float64, device=dev)
    for _ in range(3):  # capture, then replays
        E1, F1 = run(both, f, e)
        assert E1 == E0 and np.array_equal(F1, F0)
    E2, F2 = run(both)  # new buffers: captured again
    assert E2 == E0 and np.array_equal(F2, F0)
    ctx.set_global_parameters(m.alpha0 * 1.01, m.alpha1)
    E3, F3 = run(both, f, e)
    Ec, Fc = run(both | EXEC_CHECK)
    assert E3 == Ec and np.array_equal(F3, Fc) and E3 != E0
    ctx.close()


def _periodic_force(charge, radius, cutoff):
    from openmmcustomgbintegralforce_gb300 import api

    f = api.CharmmGBSWForce()
    for q, r in zip(charge, radius):
        f.addParticle(float(q), float(r), 1.0)
    f.setNonbondedMethod(api.CutoffPeriodic)
    f.setCutoffDistance(cutoff)
    return f


def test_cutoff_periodic_against_the_reference():
    """CharmmGBSWForce with CutoffPeriodic through the kernel mirror, against
    the reference classes compiled in place (golden fixture): minimum-image
    pair and point distances, the table query wrapped once per axis."""
    from openmmcustomgbintegralforce_gb300 import api

    g = golden("gbsw_200_periodic.npz")
    box, cut = tuple(float(b) for b in g["box"]), float(g["cutoff"])
    k = api.CalcCharmmGBSWForceKernel(box=box)
    k.initialize(len(g["charge"]), _periodic_force(g["charge"], g["radius"], cut))
    E, F = k.execute(g["positions"])
    assert abs(E / float(g["energy"]) - 1) < 2e-5
    assert rel_rms(F, g["forces"]) < 1e-4
    assert np.abs(k.ctx.born_radii() / g["born"] - 1).max() < 1e-4


def test_cutoff_periodic_against_the_oracle_with_adjoint():
    """A 1,000-atom globule in a box of 3.2 nm with a 1.5 nm cutoff: energy,
    forces and the adjoint's dE/dq and dE/dR against the FP64 oracle; the box
    changes the answer on this input."""
    g = make_globule(1000, seed=17)
    pos = g.positions - g.positions.min(axis=0)
    m = GBModel.charmm_gbsw(cutoff=1.5, periodic=True, box=(3.2, 3.2, 3.3))
    ctx = Context(m, g.n)
    ctx.set_particle_parameters(g.charge, g.radius)
    out = ctx.adjoint(pos)
    ref = O.Oracle(m).energy_forces(pos, g.charge, g.radius, adjoint=True)
    assert abs(out["energy"] / ref["energy"] - 1) < 2e-5
    assert rel_rms(out["forces"], ref["forces"]) < 1e-4
    assert rel_rms(out["dEdq"], ref["dEdq"]) < 1e-4
    assert rel_rms(out["dEdR"], ref["dEdR"]) < 1e-4
    E, F = ctx.execute_host(pos)
    assert abs(E / ref["energy"] - 1) < 2e-5 and rel_rms(F, ref["forces"]) < 1e-4
    flat = O.Oracle(m.replace(periodic=False)).energy_forces(pos, g.charge, g.radius)
    assert abs(flat["energy"] / ref["energy"] - 1) > 1e-3
    ctx.close()


def test_cutoff_periodic_exact_table_matches_reference_table():
    """CutoffPeriodic GBSW on the exact table (points off the standalone grid
    moved by a box edge as the reference moves them, then looked up in the
    exact table) against the same system on the reference's standalone
    table: the same volumes, hence energy, forces and Born radii to FP32
    rounding, with a fraction of the list work.  A box too narrow for the
    standalone grid's reach keeps the reference table (identical bits)."""
    g = make_globule(1000, seed=17)
    pos = g.positions - g.positions.min(axis=0)
    m = GBModel.charmm_gbsw(n_radial=24, lebedev=50, cutoff=1.5, periodic=True, box=(3.2, 3.2, 3.3))
    a = Context(m, g.n)
    b = Context(m.replace(reference_table=True), g.n)
    for c in (a, b):
        c.set_particle_parameters(g.charge, g.radius)
    Ea, Fa = a.execute_host(pos)
    Eb, Fb = b.execute_host(pos)
    assert abs(Ea / Eb - 1) < 1e-6
    assert rel_rms(Fa, Fb) < 1e-5
    assert np.abs(a.born_radii() / b.born_radii() - 1).max() < 1e-5
    a.execute_host(pos, count_work=True)
    b.execute_host(pos, count_work=True)
    assert a.work()["volume_evals"] < 0.5 * b.work()["volume_evals"]
    # the oracle (reference semantics) on the same input
    ref = O.Oracle(m).energy_forces(pos, g.charge, g.radius)
    assert abs(Ea / ref["energy"] - 1) < 2e-5 and rel_rms(Fa, ref["forces"]) < 1e-4
    for c in (a, b):
        c.close()

    # half of a 1.6 nm edge is below the standalone grid's reach: the
    # reference table serves the exact-table policy too
    small = make_globule(120, seed=5)
    sp = small.positions - small.positions.min(axis=0)
    ms = GBModel.charmm_gbsw(cutoff=0.8, periodic=True, box=(1.6, 1.6, 1.6))
    a = Context(ms, small.n)
    b = Context(ms.replace(reference_table=True), small.n)
    for c in (a, b):
        c.set_particle_parameters(small.charge, small.radius)
    Ea, Fa = a.execute_host(sp)
    Eb, Fb = b.execute_host(sp)
    assert Ea == Eb and np.array_equal(Fa, Fb)
    ref = O.Oracle(ms).energy_forces(sp, small.charge, small.radius)
    assert abs(Ea / ref["energy"] - 1) < 2e-5 and rel_rms(Fa, ref["forces"]) < 1e-4
    for c in (a, b):
        c.close()


@pytest.mark.parametrize("itype", ["gbsw", "gbmv1", "gbmv2"])
def test_gbmv_force_cutoff_periodic_against_the_oracle(itype):
    """A CharmmGBMVForce with CutoffPeriodic through the kernel mirror: the
    integral classes and the pair terms by minimum image (GBSWIntegral on the
    box-sampled table), against the FP64 oracle in a box barely larger than
    twice the cutoff."""
    from openmmcustomgbintegralforce_gb300 import api
    from openmmcustomgbintegralforce_gb300.spec import TABLE_PERIODIC

    g = make_globule(600, seed=23)
    pos = g.positions - g.positions.min(axis=0)
    box = (2.8, 2.8, 2.9)
    t = {"gbsw": api.GBSWIntegral, "gbmv1": api.GBMVIntegralTypeI, "gbmv2": api.GBMVIntegralTypeII}[itype]
    f = api.canonical_gbmv_force(t)
    for i in range(g.n):
        f.addParticle([g.charge[i], g.radius[i]])
    f.setNonbondedMethod(api.CutoffPeriodic)
    f.setCutoffDistance(1.3)
    k = api.CalcCharmmGBMVForceKernel(box=box)
    k.initialize(g.n, f)
    E, F = k.execute(pos)
    base = {"gbsw": GBModel.gbsw_integral(), "gbmv1": GBModel.gbmv1(), "gbmv2": GBModel.gbmv2()}[itype]
    m = base.replace(cutoff=1.3, periodic=True, box=box, table_mode=TABLE_PERIODIC)
    ref = O.Oracle(m).energy_forces(pos, g.charge, g.radius)
    assert abs(E / ref["energy"] - 1) < 2e-5
    assert rel_rms(F, ref["forces"]) < 1e-4
    flat = O.Oracle(m.replace(periodic=False, cutoff=0.0)).energy_forces(pos, g.charge, g.radius)
    assert abs(flat["energy"] / ref["energy"] - 1) > 1e-3



def test_surface_area_energy_is_stored_and_unused(glob1000):
    """CharmmGBSWForce's surface-area energy (CharmmGBSWForce.h:144-152,
    default 2.25936 from CharmmGBSWForce.cpp:40) is a stored value that no
    reference kernel reads: setting it changes neither energy nor forces."""
    from openmmcustomgbintegralforce_gb300 import api

    g = glob1000
    out = []
    for sa in (None, 0.0, 10.0):
        f = api.CharmmGBSWForce()
        assert f.getSurfaceAreaEnergy() == 2.25936
        if sa is not None:
            f.setSurfaceAreaEnergy(sa)
            assert f.getSurfaceAreaEnergy() == sa
        for i in range(g.n):
            f.addParticle(g.charge[i], g.radius[i], 1.0)
        k = api.CalcCharmmGBSWForceKernel()
        k.initialize(g.n, f)
        out.append(k.execute(g.positions))
    for E, F in out[1:]:
        assert E == out[0][0] and np.array_equal(F, out[0][1])
