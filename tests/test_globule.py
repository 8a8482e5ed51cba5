"""The seeded globule workload generator."""
import numpy as np

from openmmcustomgbintegralforce_gb300.globule import make_globule


def test_globule_is_deterministic_and_dense():
    a = make_globule(500, seed=4, cache=False)
    b = make_globule(500, seed=4, cache=False)
    assert np.array_equal(a.positions, b.positions)
    assert np.array_equal(a.charge, b.charge)
    assert abs(a.meta["density_A3"] - 0.1) < 0.01
    assert abs(a.charge.sum()) < 1e-5
    # float32-representable inputs
    assert np.array_equal(a.positions, a.positions.astype(np.float32).astype(np.float64))
    # exclusion honoured except for the walk's own predecessor
    from scipy.spatial import cKDTree

    d, _ = cKDTree(a.positions).query(a.positions, k=2)
    assert d[:, 1].min() > 0.1499  # closest approach is a 1.5 A chain step
    # within the relaxed minimum distance only chain neighbours occur: the
    # close-contact graph has fewer edges than a chain with branch points
    pairs = cKDTree(a.positions).query_pairs(a.meta["final_dmin_A"] * 0.1 - 1e-6)
    assert len(pairs) < 2 * a.n
    # element mix
    counts = np.bincount(a.element, minlength=5) / 500.0
    assert abs(counts[0] - 0.5) < 0.08


def test_globule_differs_by_seed():
    a = make_globule(100, seed=1, cache=False)
    b = make_globule(100, seed=2, cache=False)
    assert not np.array_equal(a.positions, b.positions)
