"""Seeded synthetic globules: the workload generator for tests and benchmarks.

A globule is a compact random-walk chain of N atoms inside a sphere sized for
0.1 atoms/A^3, with the element mix H 50 / C 30 / N 8 / O 10 / S 2 % and radii
1.2 / 1.7 / 1.55 / 1.52 / 1.8 A, partial charges from N(0, 0.35 e) shifted to a
net charge of zero.  Units on output are nm and e.

The literal rule "every 1.5 A step is rejected within 2.5 A of an earlier
atom" can never be satisfied (the step always lands 1.5 A from the atom it
left), and 2.5 A exclusion at 0.1 atoms/A^3 is a packing fraction above close
packing.  The walk therefore uses this interpretation:

1. the exclusion test ignores the atom the step leaves from;
2. after 100 failed directions the walk restarts from a random placed atom;
3. when placement stalls (``stall`` consecutive failed restarts) the minimum
   distance relaxes by 0.1 A, down to 2.0 A, and after that the sphere radius
   grows by 1 % at a time.

The achieved density, final minimum distance and sphere radius are returned
in ``meta``.  Coordinates, radii and charges are rounded to float32 so the
FP64 oracle and the FP32 device path see bit-identical inputs.
"""
from __future__ import annotations

import hashlib
import math
import os
from dataclasses import dataclass, field

import numpy as np

ELEMENTS = ("H", "C", "N", "O", "S")
FRACTIONS = (0.50, 0.30, 0.08, 0.10, 0.02)
RADII_A = (1.2, 1.7, 1.55, 1.52, 1.8)


@dataclass
class Globule:
    positions: np.ndarray  # [N,3] nm (float32-representable float64)
    radius: np.ndarray     # [N] nm
    charge: np.ndarray     # [N] e
    element: np.ndarray    # [N] index into ELEMENTS
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.positions.shape[0])


_LIB = None


def _lib():
    """The compiled walk (``csrc/globule_walk.c``), built by ``build.py``."""
    global _LIB
    if _LIB is None:
        import ctypes
        from . import build as _build
        path = _build.globule_library()
        lib = ctypes.CDLL(path)
        lib.gbx_globule_walk.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_void_p]
        lib.gbx_globule_walk.restype = ctypes.c_int
        _LIB = lib
    return _LIB


def _walk(n: int, seed: int, density_A3: float, step_A: float, dmin_A: float, dmin_floor_A: float, stall: int):
    pos = np.zeros((n, 3), dtype=np.float64)
    meta = np.zeros(2, dtype=np.float64)
    rc = _lib().gbx_globule_walk(n, seed, density_A3, step_A, dmin_A, dmin_floor_A, stall, 100,
                                 pos.ctypes.data, meta.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"globule walk failed (status {rc})")
    return pos, float(meta[0]), float(meta[1])


def make_globule(n: int, seed: int = 0, density_A3: float = 0.1, step_A: float = 1.5, dmin_A: float = 2.5,
                 dmin_floor_A: float = 2.0, stall: int = 200, charge_sigma: float = 0.35,
                 cache: bool = True) -> Globule:
    """Deterministic globule for (n, seed)."""
    if n < 1:
        raise ValueError("n must be >= 1")
    tag = f"v2-{n}-{seed}-{density_A3}-{step_A}-{dmin_A}-{dmin_floor_A}-{stall}-{charge_sigma}"
    path = None
    if cache:
        d = os.environ.get("GBX_GLOBULE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "gbx_globules"))
        try:
            os.makedirs(d, exist_ok=True)
            path = os.path.join(d, hashlib.sha1(tag.encode()).hexdigest()[:16] + ".npz")
            if os.path.exists(path):
                z = np.load(path, allow_pickle=False)
                meta = dict(zip(z["meta_k"].tolist(), z["meta_v"].tolist()))
                return Globule(z["positions"], z["radius"], z["charge"], z["element"], meta)
        except OSError:
            path = None
    pos_A, R, dmin = _walk(n, seed, density_A3, step_A, dmin_A, dmin_floor_A, stall)
    rng = np.random.default_rng(seed)
    elem = rng.choice(len(ELEMENTS), size=n, p=np.array(FRACTIONS))
    radius = np.array(RADII_A)[elem] * 0.1
    q = rng.normal(0.0, charge_sigma, size=n)
    q -= q.mean()
    positions = (pos_A * 0.1).astype(np.float32).astype(np.float64)
    radius = radius.astype(np.float32).astype(np.float64)
    q = q.astype(np.float32).astype(np.float64)
    meta = {
        "seed": float(seed),
        "n": float(n),
        "sphere_radius_A": float(R),
        "final_dmin_A": float(dmin),
        "density_A3": float(n / (4.0 / 3.0 * math.pi * R ** 3)),
    }
    g = Globule(positions, radius, q, elem.astype(np.int32), meta)
    if path:
        try:
            np.savez(path, positions=positions, radius=radius, charge=q, element=g.element,
                     meta_k=np.array(list(meta.keys())), meta_v=np.array(list(meta.values())))
        except OSError:
            pass
    return g


def jitter(positions: np.ndarray, sigma_nm: float, rng: np.random.Generator) -> np.ndarray:
    """MD-like perturbation (N(0, sigma) per coordinate), rounded to float32."""
    return (positions + rng.normal(0.0, sigma_nm, size=positions.shape)).astype(np.float32).astype(np.float64)


def _globule_job(args):
    n, seed = args
    return make_globule(n, seed=seed)


def batch_sizes(count: int = 256, lo: int = 500, hi: int = 8000, seed: int = 4242):
    """Atom counts drawn log-uniformly from [lo, hi] (seeded)."""
    rng = np.random.default_rng(seed)
    return [int(round(np.exp(x))) for x in rng.uniform(np.log(lo), np.log(hi), count)]


def make_batch(sizes, seed: int = 4242, workers: int = 0):
    """One globule per size (seed + index), generated in a spawn-started
    process pool so that it is safe before or after CUDA initialisation."""
    import multiprocessing as mp
    import os

    jobs = [(int(n), seed + k) for k, n in enumerate(sizes)]
    workers = workers or min(len(jobs), os.cpu_count() or 1)
    if workers <= 1:
        return [_globule_job(j) for j in jobs]
    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.map(_globule_job, jobs, chunksize=1)
