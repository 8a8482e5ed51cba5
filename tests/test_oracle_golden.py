"""The FP64 oracle pinned against the reference's own outputs (golden
fixtures written by tests/golden/make_golden.py from the reference classes
compiled in place).  With the reference's quadrature fed in, agreement is at
rounding level; with the quadrature generated here it is within 1e-12."""
import numpy as np
import pytest

from openmmcustomgbintegralforce_gb300.spec import GBModel
from oracle import oracle as O
from tests.conftest import golden


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.mark.parametrize("name", ["gbsw_200.npz", "gbsw_1000.npz"])
def test_charmm_gbsw_energy_forces_born(name):
    g = golden(name)
    quad = (g["qoff"], g["qrad"], g["qw"])
    out = O.Oracle(GBModel.charmm_gbsw(), quadrature=quad).energy_forces(g["positions"], g["charge"], g["radius"])
    assert abs(out["energy"] / float(g["energy"]) - 1) < 1e-13
    assert np.abs(out["born"] / g["born"] - 1).max() < 1e-13
    assert rel_rms(out["forces"], g["forces"]) < 1e-13
    # quadrature generated here (Lebedev solved, not tabulated)
    own = O.Oracle(GBModel.charmm_gbsw()).energy_forces(g["positions"], g["charge"], g["radius"])
    assert abs(own["energy"] / float(g["energy"]) - 1) < 1e-12
    assert np.abs(own["born"] / g["born"] - 1).max() < 1e-12
    assert rel_rms(own["forces"], g["forces"]) < 1e-12


def test_charmm_gbsw_table_bit_exact():
    g = golden("gbsw_200.npz")
    t = O.Oracle(GBModel.charmm_gbsw()).table(g["positions"], g["radius"])
    assert np.array_equal(t["dims"], g["table_dims"])
    assert np.array_equal(t["min"], g["table_min"])
    assert np.array_equal(t["counts"], g["table_counts"])
    assert np.array_equal(t["atoms"], g["table_atoms"])


def test_charmm_gbsw_cutoff_quirk():
    g = golden("gbsw_200_cutoff1.npz")
    m = GBModel.charmm_gbsw(cutoff=float(g["cutoff"]))
    out = O.Oracle(m).energy_forces(g["positions"], g["charge"], g["radius"])
    assert abs(out["energy"] / float(g["energy"]) - 1) < 1e-12
    assert rel_rms(out["forces"], g["forces"]) < 1e-12


def test_charmm_gbsw_cutoff_periodic():
    """CutoffPeriodic: minimum-image distances everywhere and the table query
    wrapped once per axis, against the reference classes in a rectangular box
    barely larger than twice the cutoff."""
    g = golden("gbsw_200_periodic.npz")
    box = tuple(float(b) for b in g["box"])
    m = GBModel.charmm_gbsw(cutoff=float(g["cutoff"]), periodic=True, box=box)
    out = O.Oracle(m, quadrature=(g["qoff"], g["qrad"], g["qw"])).energy_forces(g["positions"], g["charge"],
                                                                              g["radius"])
    assert abs(out["energy"] / float(g["energy"]) - 1) < 1e-13
    assert np.abs(out["born"] / g["born"] - 1).max() < 1e-13
    assert rel_rms(out["forces"], g["forces"]) < 1e-13
    # the box matters on this input
    flat = O.Oracle(m.replace(periodic=False), quadrature=(g["qoff"], g["qrad"], g["qw"])).energy_forces(
        g["positions"], g["charge"], g["radius"])
    assert abs(flat["energy"] / float(g["energy"]) - 1) > 1e-2


@pytest.mark.parametrize("n", [200, 600])
@pytest.mark.parametrize("tag", ["gbsw", "gbmv1", "gbmv2"])
def test_integral_classes(n, tag):
    g = golden(f"integrals_{n}.npz")
    box = tuple(g["box"])
    model = {"gbsw": GBModel.gbsw_integral(), "gbmv1": GBModel.gbmv1(box=box), "gbmv2": GBModel.gbmv2(box=box)}[tag]
    orc = O.Oracle(model, quadrature=(g["qoff"], g["qrad"], g["qw"]))
    t = orc.table(g["positions"], g["radius"])
    assert np.array_equal(t["dims"], g[f"{tag}_table_dims"])
    assert np.array_equal(t["counts"], g[f"{tag}_table_counts"])
    assert np.array_equal(t["atoms"], g[f"{tag}_table_atoms"])
    I, _ = orc.integrals(g["positions"], g["radius"])
    assert np.abs(I - g[f"{tag}_integrals"]).max() <= 1e-12 * np.abs(g[f"{tag}_integrals"]).max()
    F, _ = orc.integral_chain(g["positions"], g["radius"], g["dEdI"])
    assert rel_rms(F, g[f"{tag}_chain"]) < 1e-12


def test_isolated_atom_known_answer():
    """Analytic pin: isolated atoms, where the integrals are 1-D sums of the
    switching polynomial over the radial nodes (tests/kat_isolated.py)."""
    from tests.kat_isolated import continuous_integrals, expected_born, expected_integrals, isolated_system

    m = GBModel.charmm_gbsw()
    pos, radius = isolated_system([0.12, 0.17, 0.18])
    out = O.Oracle(m).energy_forces(pos, np.zeros(len(radius)), radius)
    I4, I7 = expected_integrals(m, radius)
    assert np.abs(out["integrals"][0] / I4 - 1).max() < 1e-13
    assert np.abs(out["integrals"][1] / I7 - 1).max() < 1e-13
    assert np.abs(out["born"] / expected_born(m, I4, I7) - 1).max() < 1e-13
    # the 24-node radial rule against the integral it approximates (the
    # switching shell's kinks limit Gauss-Legendre to a few parts in 1e3)
    for k, R in enumerate(radius):
        c4, c7 = continuous_integrals(m, R)
        assert abs(I4[k] / c4 - 1) < 2e-2 and abs(I7[k] / c7 - 1) < 2e-2


@pytest.mark.parametrize("tag", ["gbsw", "gbmv1", "gbmv2"])
def test_integral_classes_cutoff_periodic(tag):
    """A CharmmGBMVForce with CutoffPeriodic: the integral classes measure
    point-to-atom distances by minimum image (GBSWIntegral on the box-sampled
    table), bit for bit against the classes compiled in place."""
    from openmmcustomgbintegralforce_gb300.spec import TABLE_PERIODIC

    g = golden("integrals_200_periodic.npz")
    box = tuple(float(b) for b in g["box"])
    base = {"gbsw": GBModel.gbsw_integral(table_mode=TABLE_PERIODIC, box=box), "gbmv1": GBModel.gbmv1(box=box),
            "gbmv2": GBModel.gbmv2(box=box)}[tag]
    m = base.replace(periodic=True, cutoff=1.2)
    I, _ = O.Oracle(m, quadrature=(g["qoff"], g["qrad"], g["qw"])).integrals(g["positions"], g["radius"])
    assert np.array_equal(I, g[f"{tag}_integrals"])

