"""Writes the golden fixtures in this directory by running the reference's own
CPU classes, compiled in place from the reference tree (oracle/Makefile.ref).

    python tests/golden/make_golden.py

Needs the reference tree (GBX_REFERENCE_ROOT, default: a sibling of the repository); the
fixtures it writes are committed so that the CPU tests can pin the oracle
where the reference is absent.  Inputs are seeded globules rounded to
float32, so the FP32 device path sees the same numbers.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import refbind as R  # noqa: E402
from openmmcustomgbintegralforce_gb300.globule import make_globule  # noqa: E402
from openmmcustomgbintegralforce_gb300.spec import box_for  # noqa: E402


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print("wrote", path, os.path.getsize(path), "bytes")


def main():
    R.build()
    # quadrature rules as the reference builds them
    gl24 = R.gauss_legendre(0.05, 2.0, 24)
    gl32 = R.gauss_legendre(0.05, 2.0, 32)
    save("quadrature.npz", gl24_x=gl24[0], gl24_w=gl24[1], gl32_x=gl32[0], gl32_w=gl32[1],
         leb26=R.lebedev(3), leb38=R.lebedev(4), leb50=R.lebedev(5), leb110=R.lebedev(8))

    # CharmmGBSWForce on the Reference platform (its built-in 24x38 quadrature and constants)
    qoff, qrad, qw = R.gbsw_quadrature()
    for n, seed, with_table in ((200, 3, True), (1000, 7, False)):
        g = make_globule(n, seed=seed, cache=False)
        ref = R.gbsw_energy_forces(g.positions, g.charge, g.radius)
        extra = {}
        if with_table:
            t = R.gbsw_table(g.positions, g.radius)
            extra = dict(table_dims=t["dims"], table_min=t["min"], table_counts=t["counts"], table_atoms=t["atoms"])
        save(f"gbsw_{n}.npz", positions=g.positions, charge=g.charge, radius=g.radius, qoff=qoff, qrad=qrad, qw=qw,
             energy=np.array(ref["energy"]), forces=ref["forces"], born=ref["born"], **extra)
    # cutoff variant (the chain rule also drops atoms beyond the cutoff)
    g = make_globule(200, seed=3, cache=False)
    ref = R.gbsw_energy_forces(g.positions, g.charge, g.radius, cutoff=1.0)
    save("gbsw_200_cutoff1.npz", positions=g.positions, charge=g.charge, radius=g.radius, cutoff=np.array(1.0),
         energy=np.array(ref["energy"]), forces=ref["forces"])
    # CutoffPeriodic in a rectangular box barely larger than twice the cutoff: far pairs and far
    # quadrature points take their minimum image, points beyond the table wrap back into it
    pos = g.positions - g.positions.min(axis=0)
    box = np.array([2.5, 2.5, 2.6])
    ref = R.gbsw_energy_forces_periodic(pos, g.charge, g.radius, 1.2, box)
    save("gbsw_200_periodic.npz", positions=pos, charge=g.charge, radius=g.radius, cutoff=np.array(1.2), box=box,
         qoff=qoff, qrad=qrad, qw=qw, energy=np.array(ref["energy"]), forces=ref["forces"], born=ref["born"])

    # integral classes: GBSWIntegral (grid table), GBMV-I and GBMV-II (box table)
    qoff, qrad, qw = R.integral_quadrature(24, 3)
    for n, seed in ((200, 5), (600, 11)):
        g = make_globule(n, seed=seed, cache=False)
        box = np.array(box_for(g.positions, margin=1.0))
        rng = np.random.default_rng(seed)
        dEdI = rng.normal(size=(2, n))
        arrays = dict(positions=g.positions, charge=g.charge, radius=g.radius, box=box, qoff=qoff, qrad=qrad, qw=qw,
                      dEdI=dEdI)
        for itype, tag in ((0, "gbsw"), (1, "gbmv1"), (2, "gbmv2")):
            ev = R.integral_evaluate(itype, g.positions, g.radius, box=box)
            t = R.integral_table(itype, g.positions, g.radius, box=box)
            arrays[f"{tag}_integrals"] = ev["integrals"]
            arrays[f"{tag}_chain"] = -np.einsum("ki,kijc->jc", dEdI, ev["grads"])
            arrays[f"{tag}_table_dims"] = t["dims"]
            arrays[f"{tag}_table_min"] = t["min"]
            arrays[f"{tag}_table_step"] = t["step"]
            arrays[f"{tag}_table_counts"] = t["counts"]
            arrays[f"{tag}_table_atoms"] = t["atoms"]
        save(f"integrals_{n}.npz", **arrays)

    # the integral classes of a CharmmGBMVForce with CutoffPeriodic: minimum-image point-to-atom distances
    # (GBSWIntegral also switches to the box-sampled table) in a box barely larger than the molecule
    g = make_globule(200, seed=5, cache=False)
    pos = g.positions - g.positions.min(axis=0)
    box = np.array([2.5, 2.5, 2.6])
    arrays = dict(positions=pos, radius=g.radius, box=box, qoff=qoff, qrad=qrad, qw=qw)
    for itype, tag in ((0, "gbsw"), (1, "gbmv1"), (2, "gbmv2")):
        arrays[f"{tag}_integrals"] = R.integral_evaluate_periodic(itype, pos, g.radius, box)["integrals"]
    save("integrals_200_periodic.npz", **arrays)


if __name__ == "__main__":
    main()
