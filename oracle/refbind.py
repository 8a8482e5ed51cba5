"""ctypes binding of the reference CPU classes compiled in place
(``Makefile.ref`` -> ``_ref/libgbref.so``) -- TEST INFRASTRUCTURE.

Available only where the reference tree exists (it does not on the GPU
host); callers skip when ``available()`` is false.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libgbref.so")
# the reference tree: GBX_REFERENCE_ROOT, else a sibling of this repository
REF_ROOT = os.environ.get("GBX_REFERENCE_ROOT",
                          os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                                       "reference"))

_LIB = None


def available() -> bool:
    return os.path.exists(LIB_PATH) or os.path.isdir(os.path.join(REF_ROOT, "platforms", "reference", "src"))


def build() -> str:
    if os.path.isdir(os.path.join(REF_ROOT, "platforms")):
        subprocess.run(["make", "-C", HERE, "-s", "-f", "Makefile.ref", f"REF={REF_ROOT}"], check=True)
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("compiled reference unavailable")
    return LIB_PATH


def lib():
    global _LIB
    if _LIB is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, ci, cd, cl = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_long
        L.ref_gauss_legendre.argtypes = [cd, cd, ci, vp, vp]
        L.ref_lebedev.argtypes = [ci, vp, ci]
        L.ref_gbsw_quadrature.argtypes = [vp, ci]
        L.ref_gbsw_energy_forces.argtypes = [ci, vp, vp, vp, cd, vp, vp]
        L.ref_gbsw_energy_forces.restype = cd
        L.ref_gbsw_energy_forces_periodic.argtypes = [ci, vp, vp, vp, cd, vp, vp, vp]
        L.ref_gbsw_energy_forces_periodic.restype = cd
        L.ref_gbsw_table.argtypes = [ci, vp, vp, vp, vp, vp, cl, vp, cl]
        L.ref_gbsw_table.restype = cl
        L.ref_integral_evaluate.argtypes = [ci, ci, vp, vp, ci, vp, vp, vp, vp]
        L.ref_integral_evaluate_periodic.argtypes = [ci, ci, vp, vp, ci, vp, vp, vp]
        L.ref_integral_table.argtypes = [ci, ci, vp, vp, vp, vp, vp, vp, vp, cl, vp, cl]
        L.ref_integral_table.restype = cl
        _LIB = L
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def gauss_legendre(x0, x1, n):
    x, w = np.zeros(n), np.zeros(n)
    lib().ref_gauss_legendre(x0, x1, n, _p(x), _p(w))
    return x, w


def lebedev(rule):
    buf = np.zeros(4 * 6000)
    n = lib().ref_lebedev(rule, _p(buf), 6000)
    return buf[: 4 * n].reshape(n, 4)


def gbsw_quadrature():
    """The 24 x 38 quadrature CharmmReferenceGBSW builds: (offsets, r, w)."""
    buf = np.zeros(5 * 4000)
    n = lib().ref_gbsw_quadrature(_p(buf), 4000)
    q = buf[: 5 * n].reshape(n, 5)
    return q[:, :3].copy(), q[:, 3].copy(), q[:, 4].copy()


def integral_quadrature(n_radial=24, rule=3, r0=0.05, r1=2.0):
    """The tensor quadrature the integral classes build (GBSWIntegral.cpp:41-56)."""
    x, w = gauss_legendre(r0, r1, n_radial)
    s = lebedev(rule)
    nS = len(s)
    Q = n_radial * nS
    off, rad, wt = np.zeros((Q, 3)), np.zeros(Q), np.zeros(Q)
    for i in range(n_radial):
        for j in range(nS):
            idx = i * nS + j
            off[idx] = x[i] * s[j, :3]
            rad[idx] = x[i]
            wt[idx] = w[i] * s[j, 3]
    return off, rad, wt


def gbsw_energy_forces(pos, charge, radius, cutoff=-1.0):
    pos = np.ascontiguousarray(pos, np.float64)
    q = np.ascontiguousarray(charge, np.float64)
    R = np.ascontiguousarray(radius, np.float64)
    n = len(R)
    F = np.zeros(3 * n)
    B = np.zeros(n)
    E = lib().ref_gbsw_energy_forces(n, _p(pos), _p(q), _p(R), cutoff, _p(F), _p(B))
    return {"energy": E, "forces": F.reshape(n, 3), "born": B}


def gbsw_energy_forces_periodic(pos, charge, radius, cutoff, box):
    pos = np.ascontiguousarray(pos, np.float64)
    q = np.ascontiguousarray(charge, np.float64)
    R = np.ascontiguousarray(radius, np.float64)
    bx = np.ascontiguousarray(box, np.float64)
    n = len(R)
    F = np.zeros(3 * n)
    B = np.zeros(n)
    E = lib().ref_gbsw_energy_forces_periodic(n, _p(pos), _p(q), _p(R), cutoff, _p(bx), _p(F), _p(B))
    return {"energy": E, "forces": F.reshape(n, 3), "born": B}


def gbsw_table(pos, radius):
    pos = np.ascontiguousarray(pos, np.float64)
    R = np.ascontiguousarray(radius, np.float64)
    n = len(R)
    dims = np.zeros(3, np.int32)
    mn = np.zeros(3)
    ccap, acap = 4_000_000, 40_000_000
    counts = np.zeros(ccap, np.int32)
    atoms = np.zeros(acap, np.int32)
    tot = lib().ref_gbsw_table(n, _p(pos), _p(R), _p(dims), _p(mn), _p(counts), ccap, _p(atoms), acap)
    if tot < 0:
        raise RuntimeError("reference table too large for the buffers")
    ncell = int(np.prod(dims))
    return {"dims": dims, "min": mn, "counts": counts[:ncell].copy(), "atoms": atoms[:tot].copy()}


def integral_evaluate(itype, pos, radius, orders=(4, 7), box=None, grads=True):
    pos = np.ascontiguousarray(pos, np.float64)
    R = np.ascontiguousarray(radius, np.float64)
    n = len(R)
    o = np.array(orders, np.int32)
    I = np.zeros(len(orders) * n)
    G = np.zeros(len(orders) * n * n * 3) if grads else None
    b = np.ascontiguousarray(box, np.float64) if box is not None else None
    rc = lib().ref_integral_evaluate(itype, n, _p(pos), _p(R), len(orders), _p(o), _p(b), _p(I), _p(G))
    if rc:
        raise RuntimeError("reference integral evaluation failed")
    out = {"integrals": I.reshape(len(orders), n)}
    if grads:
        out["grads"] = G.reshape(len(orders), n, n, 3)
    return out


def integral_evaluate_periodic(itype, pos, radius, box, orders=(4, 7)):
    """Integrals of a CharmmGBMVForce with CutoffPeriodic (minimum-image distances)."""
    pos = np.ascontiguousarray(pos, np.float64)
    R = np.ascontiguousarray(radius, np.float64)
    n = len(R)
    o = np.array(orders, np.int32)
    I = np.zeros(len(orders) * n)
    b = np.ascontiguousarray(box, np.float64)
    if lib().ref_integral_evaluate_periodic(itype, n, _p(pos), _p(R), len(orders), _p(o), _p(b), _p(I)):
        raise RuntimeError("reference integral evaluation failed")
    return {"integrals": I.reshape(len(orders), n)}


def integral_table(itype, pos, radius, box=None):
    pos = np.ascontiguousarray(pos, np.float64)
    R = np.ascontiguousarray(radius, np.float64)
    n = len(R)
    dims = np.zeros(3, np.int32)
    mn = np.zeros(3)
    step = np.zeros(3)
    ccap, acap = 8_000_000, 80_000_000
    counts = np.zeros(ccap, np.int32)
    atoms = np.zeros(acap, np.int32)
    b = np.ascontiguousarray(box, np.float64) if box is not None else None
    tot = lib().ref_integral_table(itype, n, _p(pos), _p(R), _p(b), _p(dims), _p(mn), _p(step), _p(counts), ccap,
                                   _p(atoms), acap)
    if tot < 0:
        raise RuntimeError("reference table too large for the buffers")
    ncell = int(np.prod(dims))
    return {"dims": dims, "min": mn, "step": step, "counts": counts[:ncell].copy(), "atoms": atoms[:tot].copy()}
