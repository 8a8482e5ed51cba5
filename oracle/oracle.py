"""ctypes binding of the FP64 oracle (``gbx_oracle.c``) -- TEST INFRASTRUCTURE.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module.  It is what results are compared against, never the thing
measured or shipped.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")

_c_double_p = ctypes.POINTER(ctypes.c_double)


class OrcConfig(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int),
        ("nq", ctypes.c_int),
        ("qoff", _c_double_p),
        ("qrad", _c_double_p),
        ("qw", _c_double_p),
        ("n_int", ctypes.c_int),
        ("orders", ctypes.c_int * 4),
        ("table_mode", ctypes.c_int),
        ("h", ctypes.c_double),
        ("buffer", ctypes.c_double),
        ("cap", ctypes.c_int),
        ("box", ctypes.c_double * 3),
        ("sw", ctypes.c_double),
        ("gamma0", ctypes.c_double),
        ("beta", ctypes.c_double),
        ("lam", ctypes.c_double),
        ("p1", ctypes.c_double),
        ("p2", ctypes.c_double),
        ("s0", ctypes.c_double),
        ("r0", ctypes.c_double),
        ("alpha0", ctypes.c_double),
        ("alpha1", ctypes.c_double),
        ("pref", ctypes.c_double),
        ("use_cutoff", ctypes.c_int),
        ("cutoff", ctypes.c_double),
        ("cutoff_chain_quirk", ctypes.c_int),
        ("skip_empty", ctypes.c_int),
        ("standalone_sums", ctypes.c_int),
        ("nthreads", ctypes.c_int),
        ("atom_stride", ctypes.c_int),
        ("periodic", ctypes.c_int),
    ]


class OrcTable(ctypes.Structure):
    _fields_ = [
        ("mode", ctypes.c_int),
        ("dims", ctypes.c_int * 3),
        ("min", ctypes.c_double * 3),
        ("max", ctypes.c_double * 3),
        ("step", ctypes.c_double * 3),
        ("box", ctypes.c_double * 3),
        ("pad", ctypes.c_double),
        ("ncell", ctypes.c_int64),
        ("count", ctypes.POINTER(ctypes.c_int32)),
        ("start", ctypes.POINTER(ctypes.c_int64)),
        ("atoms", ctypes.POINTER(ctypes.c_int32)),
        ("dropped", ctypes.c_int64),
        ("oob", ctypes.c_int64),
        ("wrap", ctypes.c_int),
    ]


class OrcWork(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in
                ("volume_evals", "shell_evals", "points", "active_points", "chain_pairs", "pairs")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_LIB = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or any(
            os.path.getmtime(os.path.join(HERE, f)) > os.path.getmtime(LIB_PATH)
            for f in ("gbx_oracle.c", "gbx_oracle.h")):
        subprocess.run(["make", "-C", HERE, "-s"], check=True)
    return LIB_PATH


def lib():
    global _LIB
    if _LIB is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        L.orc_table_build.argtypes = [vp, ctypes.c_int, vp, vp, vp]
        L.orc_table_free.argtypes = [vp]
        L.orc_integrals.argtypes = [vp, vp, ctypes.c_int, vp, vp, vp, vp]
        L.orc_integral_chain.argtypes = [vp, vp, ctypes.c_int, vp, vp, vp, vp, vp]
        L.orc_energy_forces.argtypes = [vp, ctypes.c_int, vp, vp, vp] + [vp] * 9
        L.orc_pair_terms.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp, vp, vp, vp]
        L.orc_table_query.argtypes = [vp, vp]
        L.orc_table_query.restype = ctypes.c_int64
        _LIB = L
    return _LIB


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Oracle:
    """FP64 evaluation of one model on host arrays."""

    def __init__(self, model, quadrature=None, nthreads: int = 0, atom_stride: int = 1):
        from openmmcustomgbintegralforce_gb300.quadrature import tensor_quadrature

        self.model = model
        if quadrature is None:
            quadrature = tensor_quadrature(model.n_radial, model.lebedev, model.r0, model.r1)
        off, rad, w = quadrature
        self.qoff = np.ascontiguousarray(off, dtype=np.float64)
        self.qrad = np.ascontiguousarray(rad, dtype=np.float64)
        self.qw = np.ascontiguousarray(w, dtype=np.float64)
        c = OrcConfig()
        c.model = model.model
        c.nq = len(self.qrad)
        c.qoff = self.qoff.ctypes.data_as(_c_double_p)
        c.qrad = self.qrad.ctypes.data_as(_c_double_p)
        c.qw = self.qw.ctypes.data_as(_c_double_p)
        c.n_int = len(model.orders)
        for k, o in enumerate(model.orders):
            c.orders[k] = o
        c.table_mode = model.table_mode
        c.h = model.h
        c.buffer = model.buffer
        c.cap = model.cap
        for k in range(3):
            c.box[k] = model.box[k]
        c.sw = model.sw
        c.gamma0, c.beta, c.lam = model.gamma0, model.beta, model.lam
        c.p1, c.p2, c.s0 = model.p1, model.p2, model.s0
        c.r0 = model.r0
        c.alpha0, c.alpha1 = model.alpha0, model.alpha1
        c.pref = model.pref
        c.use_cutoff = 1 if model.cutoff > 0 else 0
        c.cutoff = model.cutoff
        c.cutoff_chain_quirk = 1 if model.cutoff_chain_quirk else 0
        c.skip_empty = 1 if model.skip_empty else 0
        c.standalone_sums = 1 if model.standalone_sums else 0
        c.nthreads = nthreads
        c.atom_stride = atom_stride
        c.periodic = 1 if model.periodic else 0
        self.cfg = c

    def table(self, pos, radius):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        radius = np.ascontiguousarray(radius, dtype=np.float64)
        t = OrcTable()
        rc = lib().orc_table_build(ctypes.byref(self.cfg), len(radius), _ptr(pos), _ptr(radius), ctypes.byref(t))
        if rc:
            raise RuntimeError(f"oracle table build failed ({rc})")
        ncell = t.ncell
        total = t.start[ncell]
        out = {
            "dims": np.array(t.dims[:]),
            "min": np.array(t.min[:]),
            "max": np.array(t.max[:]),
            "step": np.array(t.step[:]),
            "pad": t.pad,
            "counts": np.ctypeslib.as_array(t.count, shape=(ncell,)).copy(),
            "start": np.ctypeslib.as_array(t.start, shape=(ncell + 1,)).copy(),
            "atoms": np.ctypeslib.as_array(t.atoms, shape=(max(total, 1),))[:total].copy(),
            "dropped": t.dropped,
            "oob": t.oob,
        }
        lib().orc_table_free(ctypes.byref(t))
        return out

    def integrals(self, pos, radius):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        radius = np.ascontiguousarray(radius, dtype=np.float64)
        n = len(radius)
        t = OrcTable()
        if lib().orc_table_build(ctypes.byref(self.cfg), n, _ptr(pos), _ptr(radius), ctypes.byref(t)):
            raise RuntimeError("oracle table build failed")
        I = np.zeros(len(self.model.orders) * n)
        w = OrcWork()
        lib().orc_integrals(ctypes.byref(self.cfg), ctypes.byref(t), n, _ptr(pos), _ptr(radius), _ptr(I),
                            ctypes.byref(w))
        lib().orc_table_free(ctypes.byref(t))
        return I.reshape(len(self.model.orders), n), w.as_dict()

    def integral_chain(self, pos, radius, dEdI):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        radius = np.ascontiguousarray(radius, dtype=np.float64)
        dEdI = np.ascontiguousarray(dEdI, dtype=np.float64)
        n = len(radius)
        t = OrcTable()
        if lib().orc_table_build(ctypes.byref(self.cfg), n, _ptr(pos), _ptr(radius), ctypes.byref(t)):
            raise RuntimeError("oracle table build failed")
        F = np.zeros(3 * n)
        w = OrcWork()
        lib().orc_integral_chain(ctypes.byref(self.cfg), ctypes.byref(t), n, _ptr(pos), _ptr(radius), _ptr(dEdI),
                                 _ptr(F), ctypes.byref(w))
        lib().orc_table_free(ctypes.byref(t))
        return F.reshape(n, 3), w.as_dict()

    def energy_forces(self, pos, charge, radius, adjoint: bool = False):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        q = np.ascontiguousarray(charge, dtype=np.float64)
        radius = np.ascontiguousarray(radius, dtype=np.float64)
        n = len(radius)
        E = np.zeros(1)
        F = np.zeros(3 * n)
        B = np.zeros(n)
        I = np.zeros(2 * n)
        dB = np.zeros(n)
        dq = np.zeros(n) if adjoint else None
        dR = np.zeros(n) if adjoint else None
        da = np.zeros(2) if adjoint else None
        w = OrcWork()
        rc = lib().orc_energy_forces(ctypes.byref(self.cfg), n, _ptr(pos), _ptr(q), _ptr(radius), _ptr(E), _ptr(F),
                                     _ptr(B), _ptr(I), _ptr(dB), _ptr(dq), _ptr(dR), _ptr(da), ctypes.byref(w))
        if rc:
            raise RuntimeError(f"oracle energy_forces failed ({rc})")
        out = {"energy": float(E[0]), "forces": F.reshape(n, 3), "born": B, "integrals": I.reshape(2, n),
               "dEdB": dB, "work": w.as_dict()}
        if adjoint:
            out.update({"dEdq": dq, "dEdR": dR, "dEdalpha": da})
        return out

    def pair_terms(self, pos, charge, born):
        """The pair term alone for given Born radii (CharmmReferenceGBSW.cpp:237-283):
        energy (self terms included), pair forces, dE/dB and dE/dq."""
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        q = np.ascontiguousarray(charge, dtype=np.float64)
        B = np.ascontiguousarray(born, dtype=np.float64)
        n = len(B)
        E = np.zeros(1)
        F = np.zeros(3 * n)
        dB = np.zeros(n)
        dq = np.zeros(n)
        rc = lib().orc_pair_terms(ctypes.byref(self.cfg), n, _ptr(pos), _ptr(q), _ptr(B), _ptr(E), _ptr(F), _ptr(dB),
                                  _ptr(dq), None)
        if rc:
            raise RuntimeError(f"oracle pair_terms failed ({rc})")
        return {"energy": float(E[0]), "forces": F.reshape(n, 3), "dEdB": dB, "dEdq": dq}
