"""Model specification shared by the device API and the test oracle.

``GBModel`` carries every constant the reference hard-codes in its classes,
so that the same description can drive the CUDA library (through
``gbx_config``) and the FP64 oracle.  The presets reproduce the reference's
native settings:

* ``charmm_gbsw``   -- ``CharmmGBSWForce`` on the Reference platform
  (``CharmmReferenceGBSW.cpp:20-52``): 24 Gauss-Legendre x 38 Lebedev points
  on [0.05, 2.0] nm, uniform-pad uncapped grid-point table
  (``:440-514``), switching half-width 0.03 nm, alpha0 = -0.180,
  alpha1 = 1.817 (``:559-561``), prefactor -ONE_4PI_EPS0 (1 - 1/80)
  (``:177-178``).
* ``gbsw_integral`` -- ``CharmmGBMVForce`` with ``GBSWIntegral``
  (``GBSWIntegral.cpp:24-61``): 24 x 26 points, per-atom-pad grid table with
  buffer 0.04 nm and cap 64 (``CustomGBIntegral.cpp:12-16,162-228``).
* ``gbmv1`` / ``gbmv2`` -- ``GBMVIntegralTypeI`` / ``TypeII``
  (``GBMVIntegralTypeI.cpp:18-57``, ``GBMVIntegralTypeII.cpp:19-62``): 24 x 26
  points, box-sampled periodic-branch table (always taken, because
  ``BeforeComputation`` sets the box unconditionally) with buffer 0.21 nm and
  cap 64.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field

ONE_4PI_EPS0 = 138.935456  # kJ nm / (mol e^2), OpenMM 7.x
GBSW, GBMV1, GBMV2 = 0, 1, 2
TABLE_STANDALONE, TABLE_GRID, TABLE_PERIODIC = 0, 1, 2
MODEL_NAMES = {GBSW: "gbsw", GBMV1: "gbmv1", GBMV2: "gbmv2"}


@dataclass
class GBModel:
    model: int = GBSW
    n_radial: int = 24
    lebedev: int = 38
    r0: float = 0.05
    r1: float = 2.0
    orders: tuple = (4, 7)
    table_mode: int = TABLE_STANDALONE
    h: float = 0.15
    buffer: float = 0.20
    cap: int = 0                      # <= 0: uncapped
    box: tuple = (0.0, 0.0, 0.0)      # periodic-sampled table; with periodic, the rectangular box
    periodic: bool = False            # CutoffPeriodic: minimum-image distances in box
    sw: float = 0.03
    gamma0: float = 0.44
    beta: float = -100.0
    lam: float = 0.1
    p1: float = 0.45
    p2: float = 1.25
    s0: float = 0.7
    alpha0: float = -0.180
    alpha1: float = 1.817
    pref: float = -ONE_4PI_EPS0 * (1.0 - 1.0 / 80.0)
    cutoff: float = 0.0               # <= 0: no cutoff (full N^2 pair term)
    cutoff_chain_quirk: bool = True   # CharmmReferenceGBSW.cpp:291-292
    skip_empty: bool = True
    standalone_sums: bool = True
    reference_table: bool = False     # device: always integrate on the reference table
    tight_h: float = 0.1              # device: cell edge of the exact GBSW table (nm)

    def replace(self, **kw) -> "GBModel":
        return dataclasses.replace(self, **kw)

    @property
    def n_quad(self) -> int:
        return self.n_radial * self.lebedev

    @staticmethod
    def charmm_gbsw(**kw) -> "GBModel":
        return GBModel(**kw)

    @staticmethod
    def gbsw_integral(**kw) -> "GBModel":
        base = dict(model=GBSW, lebedev=26, table_mode=TABLE_GRID, buffer=0.04, cap=64,
                    skip_empty=True, standalone_sums=False, cutoff_chain_quirk=False)
        base.update(kw)
        return GBModel(**base)

    @staticmethod
    def gbmv1(box=(10.0, 10.0, 10.0), **kw) -> "GBModel":
        base = dict(model=GBMV1, lebedev=26, table_mode=TABLE_PERIODIC, buffer=0.21, cap=64, box=tuple(box),
                    gamma0=0.44, beta=-100.0, lam=0.1, skip_empty=False, standalone_sums=False,
                    cutoff_chain_quirk=False)
        base.update(kw)
        return GBModel(**base)

    @staticmethod
    def gbmv2(box=(10.0, 10.0, 10.0), **kw) -> "GBModel":
        base = dict(model=GBMV2, lebedev=26, table_mode=TABLE_PERIODIC, buffer=0.21, cap=64, box=tuple(box),
                    gamma0=0.44, beta=-20.0, lam=0.5, p1=0.45, p2=1.25, s0=0.7, skip_empty=False,
                    standalone_sums=False, cutoff_chain_quirk=False)
        base.update(kw)
        return GBModel(**base)


def box_for(positions, margin: float = 1.0, h: float = 0.15):
    """A cubic periodic box that holds the molecule plus ``margin`` nm on each
    side (the reference GBMV path always bins atoms into a box-sized grid)."""
    import numpy as np

    span = float((np.max(positions, axis=0) - np.min(positions, axis=0)).max())
    side = span + 2.0 * margin
    side = h * float(int(side / h) + 1)
    return (side, side, side)
