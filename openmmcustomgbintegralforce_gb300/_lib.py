"""ctypes binding of the gbx C ABI (``include/gbx.h``, ``lib/libgbx.so``).

There is no fallback: if the CUDA library is missing or no GPU is present,
calls raise.  The library is built in-tree by ``build.py``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build
from .spec import GBModel

GBX_OK = 0
STATUS_NAMES = {
    0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory", 4: "unsupported",
    5: "non-finite result", 6: "lookup table too large", 7: "no result yet", 8: "device wait timed out",
    9: "more atoms than the static scratch of gbx_pair_noalloc holds",
    10: "an earlier unchecked call lacked the volume terms (its lookup table outgrew its buffers)",
}
EXEC_FORCES, EXEC_ENERGY, EXEC_CHECK, EXEC_COUNT_WORK = 1, 2, 4, 8
EXEC_POSQ_DOUBLE, EXEC_ENERGY_FLOAT = 16, 32

# every symbol include/gbx.h declares
EXPORTED = (
    "gbx_status_string", "gbx_version", "gbx_config_preset", "gbx_create", "gbx_destroy", "gbx_last_error",
    "gbx_set_particle_parameters", "gbx_set_global_parameters", "gbx_set_box", "gbx_execute", "gbx_set_atom_order",
    "gbx_execute_host",
    "gbx_get_born_radii", "gbx_get_integrals", "gbx_get_dEdB", "gbx_build_lookup_table", "gbx_get_lookup_table",
    "gbx_adjoint_host", "gbx_adjoint", "gbx_get_work", "gbx_get_chain_work", "gbx_set_chain_records",
    "gbx_get_chain_records", "gbx_get_launches", "gbx_set_timing", "gbx_get_stage_times", "gbx_pair_noalloc",
    "gbx_create_custom", "gbx_get_custom_param_derivs", "gbx_set_custom_parameters", "gbx_set_custom_global", "gbx_custom_check",
    "gbx_batch_create", "gbx_batch_destroy", "gbx_batch_molecule", "gbx_batch_buffers", "gbx_batch_execute",
    "gbx_batch_execute_host", "gbx_batch_adjoint", "gbx_batch_adjoint_host", "gbx_batch_tune",
    "gbx_batch_last_error",
)
STAGES = ("stage_positions", "lookup_table", "point_binning", "integrals", "born_radii", "pair", "chain_prep", "chain_rule",
          "energy_reduce")


class GBXError(RuntimeError):
    def __init__(self, status: int, message: str = ""):
        self.status = status
        super().__init__(f"gbx: {STATUS_NAMES.get(status, status)}" + (f": {message}" if message else ""))


class GbxConfig(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int),
        ("n_radial", ctypes.c_int),
        ("lebedev_order", ctypes.c_int),
        ("r0", ctypes.c_double),
        ("r1", ctypes.c_double),
        ("table_mode", ctypes.c_int),
        ("table_cap", ctypes.c_int),
        ("grid_length", ctypes.c_double),
        ("table_buffer", ctypes.c_double),
        ("box", ctypes.c_double * 3),
        ("switch_width", ctypes.c_double),
        ("gamma0", ctypes.c_double),
        ("beta", ctypes.c_double),
        ("lam", ctypes.c_double),
        ("p1", ctypes.c_double),
        ("p2", ctypes.c_double),
        ("s0", ctypes.c_double),
        ("alpha0", ctypes.c_double),
        ("alpha1", ctypes.c_double),
        ("prefactor", ctypes.c_double),
        ("cutoff", ctypes.c_double),
        ("cutoff_chain_quirk", ctypes.c_int),
        ("skip_empty", ctypes.c_int),
        ("table_policy", ctypes.c_int),
        ("periodic", ctypes.c_int),
        ("tight_grid_length", ctypes.c_double),
        ("integral_orders", ctypes.c_int * 2),
        ("reserved", ctypes.c_int * 2),
    ]

    @staticmethod
    def from_model(m: GBModel) -> "GbxConfig":
        c = GbxConfig()
        c.model = m.model
        c.n_radial = m.n_radial
        c.lebedev_order = m.lebedev
        c.r0, c.r1 = m.r0, m.r1
        c.table_mode = m.table_mode
        c.table_cap = m.cap
        c.grid_length = m.h
        c.table_buffer = m.buffer
        for k in range(3):
            c.box[k] = m.box[k] if m.box[k] > 0 else 10.0
        c.switch_width = m.sw
        c.gamma0, c.beta, c.lam = m.gamma0, m.beta, m.lam
        c.p1, c.p2, c.s0 = m.p1, m.p2, m.s0
        c.alpha0, c.alpha1 = m.alpha0, m.alpha1
        c.prefactor = m.pref
        c.cutoff = m.cutoff
        c.cutoff_chain_quirk = 1 if m.cutoff_chain_quirk else 0
        c.skip_empty = 1 if m.skip_empty else 0
        c.table_policy = 1 if m.reference_table else 0
        c.tight_grid_length = m.tight_h
        c.periodic = 1 if m.periodic else 0
        c.integral_orders[0] = int(m.orders[0])
        c.integral_orders[1] = int(m.orders[1] if len(m.orders) > 1 else m.orders[0])
        return c


_LIB = None


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load lib/libgbx.so (building it first if absent and nvcc is available)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise GBXError(4, f"CUDA library not built: {path}")
        _build.build_cuda()
    L = ctypes.CDLL(path)
    vp, ci, cd, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_size_t
    L.gbx_status_string.restype = ctypes.c_char_p
    L.gbx_status_string.argtypes = [ci]
    L.gbx_version.restype = ci
    L.gbx_config_preset.argtypes = [ci, vp]
    L.gbx_create.argtypes = [vp, ci, ctypes.POINTER(vp)]
    L.gbx_destroy.argtypes = [vp]
    L.gbx_last_error.argtypes = [vp, ctypes.c_char_p, sz]
    L.gbx_set_particle_parameters.argtypes = [vp, vp, vp]
    L.gbx_set_global_parameters.argtypes = [vp, cd, cd]
    L.gbx_set_box.argtypes = [vp, vp]
    L.gbx_set_atom_order.argtypes = [vp, vp]
    L.gbx_create_custom.argtypes = [vp, ci, vp, vp]
    L.gbx_get_custom_param_derivs.argtypes = [vp, vp, ci]
    L.gbx_set_custom_parameters.argtypes = [vp, vp]
    L.gbx_set_custom_global.argtypes = [vp, ctypes.c_char_p, cd]
    L.gbx_custom_check.argtypes = [vp, ctypes.c_char_p, sz]
    L.gbx_execute.argtypes = [vp, vp, vp, ci, vp, ci, vp]
    L.gbx_execute_host.argtypes = [vp, vp, vp, vp, ci]
    L.gbx_get_born_radii.argtypes = [vp, vp]
    L.gbx_get_integrals.argtypes = [vp, vp]
    L.gbx_get_dEdB.argtypes = [vp, vp]
    L.gbx_build_lookup_table.argtypes = [vp, vp, vp]
    L.gbx_get_lookup_table.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
    L.gbx_adjoint_host.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.gbx_get_work.argtypes = [vp, vp, vp, vp]
    L.gbx_adjoint.argtypes = [vp, vp, vp, vp, vp, vp, vp, ci, vp]
    L.gbx_get_chain_work.argtypes = [vp, vp, vp]
    L.gbx_set_chain_records.argtypes = [vp, ci]
    L.gbx_get_chain_records.argtypes = [vp, vp, vp, vp, vp]
    L.gbx_get_launches.argtypes = [vp, vp]
    L.gbx_batch_create.argtypes = [vp, vp, ci, ctypes.POINTER(vp)]
    L.gbx_batch_destroy.argtypes = [vp]
    L.gbx_batch_molecule.argtypes = [vp, ci, ctypes.POINTER(vp), vp]
    L.gbx_batch_buffers.argtypes = [vp, vp, vp, vp, vp]
    L.gbx_batch_execute.argtypes = [vp, ci, vp]
    L.gbx_batch_execute_host.argtypes = [vp, vp, vp, vp]
    L.gbx_batch_adjoint.argtypes = [vp, vp, vp, vp, vp, vp, ci, vp]
    L.gbx_batch_adjoint_host.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.gbx_batch_tune.argtypes = [vp, vp, vp, vp]
    L.gbx_batch_last_error.argtypes = [vp, ctypes.c_char_p, sz]
    L.gbx_set_timing.argtypes = [vp, ci]
    L.gbx_get_stage_times.argtypes = [vp, vp, ci, vp]
    L.gbx_pair_noalloc.argtypes = [vp, vp, vp, ci, cd, cd, vp, ci, vp, vp, vp]
    for name in EXPORTED:
        if name not in ("gbx_status_string", "gbx_version"):
            getattr(L, name).restype = ci
    _LIB = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Context:
    """One gbx_context: the device state behind one force instance."""

    def __init__(self, model: GBModel, num_atoms: int):
        self.lib = load()
        self.model = model
        self.n = int(num_atoms)
        self.cfg = GbxConfig.from_model(model)
        h = ctypes.c_void_p()
        self._check(self.lib.gbx_create(ctypes.byref(self.cfg), self.n, ctypes.byref(h)), ctx=False)
        self.h = h

    def _check(self, status: int, ctx: bool = True):
        if status != GBX_OK:
            msg = ""
            if ctx and getattr(self, "h", None):
                buf = ctypes.create_string_buffer(512)
                self.lib.gbx_last_error(self.h, buf, 512)
                msg = buf.value.decode()
            raise GBXError(status, msg)

    @classmethod
    def _borrowed(cls, lib, handle, model: GBModel, num_atoms: int) -> "Context":
        """A view of a context owned by something else (a batch molecule)."""
        c = cls.__new__(cls)
        c.lib, c.model, c.n, c.cfg, c.h, c._owner = lib, model, int(num_atoms), GbxConfig.from_model(model), handle, False
        return c

    def close(self):
        if getattr(self, "h", None):
            if getattr(self, "_owner", True):
                self.lib.gbx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_particle_parameters(self, charge, radius):
        q = np.ascontiguousarray(charge, dtype=np.float64)
        r = np.ascontiguousarray(radius, dtype=np.float64)
        if q.shape != (self.n,) or r.shape != (self.n,):
            raise GBXError(1, "charge/radius must have one entry per particle")
        self._check(self.lib.gbx_set_particle_parameters(self.h, _p(q), _p(r)))

    def set_global_parameters(self, alpha0: float, alpha1: float):
        self._check(self.lib.gbx_set_global_parameters(self.h, float(alpha0), float(alpha1)))

    def set_atom_order(self, atom_index):
        """Slot k of the device positions / forces holds atom atom_index[k] (None: identity)."""
        if atom_index is None:
            self._check(self.lib.gbx_set_atom_order(self.h, None))
            return
        a = np.ascontiguousarray(atom_index, dtype=np.int32)
        if a.shape != (self.n,):
            raise GBXError(1, "atom_index must have one entry per particle")
        self._check(self.lib.gbx_set_atom_order(self.h, a.ctypes.data_as(ctypes.c_void_p)))

    def set_box(self, box):
        b = np.ascontiguousarray(box, dtype=np.float64)
        self._check(self.lib.gbx_set_box(self.h, _p(b)))

    def execute_host(self, positions, forces: bool = True, energy: bool = True, count_work: bool = False,
                     check: bool = False):
        """Energy and forces from host positions [n, 3] (nm).  The first call
        sizes the lookup table (checked); later ones synchronise once and
        re-run checked only if the table outgrew its buffers.  check=True
        forces a checked run."""
        x = np.ascontiguousarray(positions, dtype=np.float64)
        if x.shape != (self.n, 3):
            raise GBXError(1, "positions must be [n, 3]")
        F = np.zeros((self.n, 3))
        E = np.zeros(1)
        flags = (EXEC_FORCES if forces else 0) | (EXEC_ENERGY if energy else 0) | (EXEC_CHECK if check else 0)
        if count_work:
            flags |= EXEC_COUNT_WORK
        self._check(self.lib.gbx_execute_host(self.h, _p(x), _p(F), _p(E), flags))
        return float(E[0]), F

    def execute_device(self, posq_ptr: int, force_ptr: int, force_stride: int, energy_ptr: int, flags: int,
                       stream: int = 0):
        self._check(self.lib.gbx_execute(self.h, ctypes.c_void_p(posq_ptr), ctypes.c_void_p(force_ptr),
                                         int(force_stride), ctypes.c_void_p(energy_ptr), int(flags),
                                         ctypes.c_void_p(stream)))

    def adjoint(self, positions):
        x = np.ascontiguousarray(positions, dtype=np.float64)
        E = np.zeros(1)
        F = np.zeros((self.n, 3))
        dq = np.zeros(self.n)
        dR = np.zeros(self.n)
        da = np.zeros(2)
        self._check(self.lib.gbx_adjoint_host(self.h, _p(x), _p(E), _p(F), _p(dq), _p(dR), _p(da)))
        return {"energy": float(E[0]), "forces": F, "dEdq": dq, "dEdR": dR, "dEdalpha": da}

    def adjoint_device(self, posq_ptr: int, energy_ptr: int, forces_ptr: int, dEdq_ptr: int, dEdR_ptr: int,
                       dEdalpha_ptr: int, flags: int = 0, stream: int = 0):
        """Device adjoint: every pointer a device address (0 = not wanted)."""
        self._check(self.lib.gbx_adjoint(self.h, ctypes.c_void_p(posq_ptr), ctypes.c_void_p(energy_ptr or None),
                                         ctypes.c_void_p(forces_ptr or None), ctypes.c_void_p(dEdq_ptr or None),
                                         ctypes.c_void_p(dEdR_ptr or None), ctypes.c_void_p(dEdalpha_ptr or None),
                                         int(flags), ctypes.c_void_p(stream or None)))

    def born_radii(self):
        out = np.zeros(self.n)
        self._check(self.lib.gbx_get_born_radii(self.h, _p(out)))
        return out

    def integrals(self):
        out = np.zeros(2 * self.n)
        self._check(self.lib.gbx_get_integrals(self.h, _p(out)))
        return out.reshape(2, self.n)

    def dEdB(self):
        out = np.zeros(self.n)
        self._check(self.lib.gbx_get_dEdB(self.h, _p(out)))
        return out

    def work(self):
        v, s, p = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.gbx_get_work(self.h, ctypes.byref(v), ctypes.byref(s), ctypes.byref(p)))
        fe, fs = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.gbx_get_chain_work(self.h, ctypes.byref(fe), ctypes.byref(fs)))
        return {"volume_evals": v.value, "shell_evals": s.value, "pairs": p.value,
                "chain_list_evals": fe.value, "chain_derivative_evals": fs.value}

    def set_chain_records(self, per_warp: int):
        """-1: automatic, 0: no chain records, > 0: records per (atom, quadrature chunk) warp."""
        self._check(self.lib.gbx_set_chain_records(self.h, int(per_warp)))

    def chain_records(self):
        w, mx, R, over = ctypes.c_longlong(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.gbx_get_chain_records(self.h, ctypes.byref(w), ctypes.byref(mx), ctypes.byref(R),
                                                   ctypes.byref(over)))
        return {"written": w.value, "max_need": mx.value, "per_warp": R.value, "overflowed": over.value}

    def launches(self) -> int:
        v = ctypes.c_longlong()
        self._check(self.lib.gbx_get_launches(self.h, ctypes.byref(v)))
        return v.value

    def set_timing(self, enable: bool = True):
        self._check(self.lib.gbx_set_timing(self.h, 1 if enable else 0))

    def stage_times(self):
        ms = np.zeros(len(STAGES))
        k = ctypes.c_int()
        self._check(self.lib.gbx_get_stage_times(self.h, _p(ms), len(STAGES), ctypes.byref(k)))
        return dict(zip(STAGES, ms.tolist()))

    def lookup_table(self):
        dims = np.zeros(3, np.int32)
        mn = np.zeros(3)
        step = np.zeros(3)
        ncell = ctypes.c_int64()
        total = ctypes.c_int64()
        self._check(self.lib.gbx_get_lookup_table(self.h, _p(dims), _p(mn), _p(step), ctypes.byref(ncell), None,
                                                  ctypes.byref(total), None))
        counts = np.zeros(ncell.value, np.int32)
        atoms = np.zeros(max(total.value, 1), np.int32)
        self._check(self.lib.gbx_get_lookup_table(self.h, _p(dims), _p(mn), _p(step), ctypes.byref(ncell),
                                                  _p(counts), ctypes.byref(total), _p(atoms)))
        return {"dims": dims, "min": mn, "step": step, "counts": counts, "atoms": atoms[: total.value]}


class GbxCustom(ctypes.Structure):
    _fields_ = [
        ("num_params", ctypes.c_int), ("param_names", ctypes.POINTER(ctypes.c_char_p)),
        ("num_globals", ctypes.c_int), ("global_names", ctypes.POINTER(ctypes.c_char_p)),
        ("global_values", ctypes.POINTER(ctypes.c_double)),
        ("num_integrals", ctypes.c_int), ("integral_names", ctypes.POINTER(ctypes.c_char_p)),
        ("integral_orders", ctypes.POINTER(ctypes.c_int)),
        ("num_values", ctypes.c_int), ("value_names", ctypes.POINTER(ctypes.c_char_p)),
        ("value_expressions", ctypes.POINTER(ctypes.c_char_p)),
        ("num_terms", ctypes.c_int), ("term_expressions", ctypes.POINTER(ctypes.c_char_p)),
        ("term_types", ctypes.POINTER(ctypes.c_int)),
        ("num_exclusions", ctypes.c_int), ("exclusions", ctypes.POINTER(ctypes.c_int)),
        ("num_param_derivs", ctypes.c_int), ("param_deriv_names", ctypes.POINTER(ctypes.c_char_p)),
        ("num_functions", ctypes.c_int), ("function_names", ctypes.POINTER(ctypes.c_char_p)),
        ("function_sizes", ctypes.POINTER(ctypes.c_int)), ("function_values", ctypes.POINTER(ctypes.c_double)),
        ("function_ranges", ctypes.POINTER(ctypes.c_double)),
    ]


TERM_SINGLE, TERM_PAIR, TERM_PAIR_NO_EXCLUSIONS = 0, 1, 2


def custom_struct(custom: dict):
    """A GbxCustom for ``custom`` (see CustomContext) and the buffers it points into."""
    keep = []

    def strs(xs):
        arr = (ctypes.c_char_p * max(1, len(xs)))(*[x.encode() for x in xs])
        keep.append(arr)
        return arr

    gl = list(custom.get("globals", {}).items())
    integ = list(custom["integrals"])
    vals = list(custom.get("values", []))
    terms = list(custom["terms"])
    c = GbxCustom()
    c.num_params = len(custom["params"])
    c.param_names = strs(custom["params"])
    c.num_globals = len(gl)
    c.global_names = strs([k for k, _ in gl])
    gv = (ctypes.c_double * max(1, len(gl)))(*[float(v) for _, v in gl])
    c.global_values = gv
    c.num_integrals = len(integ)
    c.integral_names = strs([k for k, _ in integ])
    io = (ctypes.c_int * max(1, len(integ)))(*[int(o) for _, o in integ])
    c.integral_orders = io
    c.num_values = len(vals)
    c.value_names = strs([k for k, _ in vals])
    c.value_expressions = strs([e for _, e in vals])
    c.num_terms = len(terms)
    c.term_expressions = strs([e for e, _ in terms])
    tt = (ctypes.c_int * max(1, len(terms)))(*[int(t) for _, t in terms])
    c.term_types = tt
    ex = [int(v) for pair in custom.get("exclusions", []) for v in pair]
    ea = (ctypes.c_int * max(1, len(ex)))(*ex)
    c.num_exclusions = len(ex) // 2
    c.exclusions = ea
    pd = list(custom.get("param_derivs", []))
    c.num_param_derivs = len(pd)
    c.param_deriv_names = strs(pd)
    fns = list(custom.get("functions", {}).items())  # name -> (values, min, max)
    fv = [float(v) for _, (vals_, _, _) in fns for v in vals_]
    fs = (ctypes.c_int * max(1, len(fns)))(*[len(vals_) for _, (vals_, _, _) in fns])
    fva = (ctypes.c_double * max(1, len(fv)))(*fv)
    fr = (ctypes.c_double * max(1, 2 * len(fns)))(*[float(x) for _, (_, lo, hi) in fns for x in (lo, hi)])
    c.num_functions = len(fns)
    c.function_names = strs([k for k, _ in fns])
    c.function_sizes = fs
    c.function_values = fva
    c.function_ranges = fr
    keep += [gv, io, tt, ea, fs, fva, fr]
    return c, keep


def check_custom(custom: dict):
    """Parses and compiles an expression set without a device (gbx_custom_check):
    (status, message)."""
    lib = load()
    c, _keep = custom_struct(custom)
    buf = ctypes.create_string_buffer(4096)
    st = lib.gbx_custom_check(ctypes.byref(c), buf, 4096)
    return st, buf.value.decode(errors="replace")


class CustomContext(Context):
    """A context for CharmmGBMVForce expressions outside the canonical set
    (gbx_create_custom): ``custom`` is a dict with ``params`` (names, one of
    them "radius"), ``globals`` ({name: value}), ``integrals`` ([(name,
    order)]), ``values`` ([(name, expression)]) and ``terms`` ([(expression,
    TERM_SINGLE | TERM_PAIR | TERM_PAIR_NO_EXCLUSIONS)]), and optionally
    ``exclusions`` ([(i, j)], skipped by TERM_PAIR terms),
    ``param_derivs`` ([global names] whose energy derivative
    ``param_derivs()`` returns) and ``functions`` ({name: (values, min,
    max)}: Continuous1DFunction tables, called by name in any expression).
    The integral class, quadrature and table come from ``model``."""

    def __init__(self, model: GBModel, num_atoms: int, custom: dict):
        self.lib = load()
        self.model = model
        self.n = int(num_atoms)
        self.custom = custom
        self.cfg = GbxConfig.from_model(model)
        c, keep = custom_struct(custom)
        h = ctypes.c_void_p()
        self._check(self.lib.gbx_create_custom(ctypes.byref(self.cfg), self.n, ctypes.byref(c), ctypes.byref(h)),
                    ctx=False)
        self.h = h

    def set_custom_parameters(self, params):
        p = np.ascontiguousarray(params, dtype=np.float64)
        if p.shape != (self.n, len(self.custom["params"])):
            raise GBXError(1, "params must be [n, num_params]")
        self._check(self.lib.gbx_set_custom_parameters(self.h, _p(p)))

    def set_custom_global(self, name: str, value: float):
        self._check(self.lib.gbx_set_custom_global(self.h, name.encode(), float(value)))

    def param_derivs(self):
        """dE/dg of the last call for each global in ``custom["param_derivs"]``."""
        k = len(self.custom.get("param_derivs", []))
        out = np.zeros(max(1, k))
        self._check(self.lib.gbx_get_custom_param_derivs(self.h, _p(out), k))
        return out[:k]


class Batch:
    """gbx_batch: many molecules per call (one CUDA graph after the first)."""

    def __init__(self, models, sizes):
        self.lib = load()
        self.models = list(models)
        self.sizes = [int(n) for n in sizes]
        if len(self.models) != len(self.sizes) or not self.sizes:
            raise GBXError(1, "one model per molecule")
        cfgs = (GbxConfig * len(self.sizes))(*[GbxConfig.from_model(m) for m in self.models])
        ns = (ctypes.c_int * len(self.sizes))(*self.sizes)
        h = ctypes.c_void_p()
        st = self.lib.gbx_batch_create(cfgs, ns, len(self.sizes), ctypes.byref(h))
        if st != GBX_OK:
            raise GBXError(st, "gbx_batch_create")
        self.h = h
        self.offsets = []
        self.molecules = []
        for m, (model, n) in enumerate(zip(self.models, self.sizes)):
            ch, off = ctypes.c_void_p(), ctypes.c_longlong()
            self._check(self.lib.gbx_batch_molecule(self.h, m, ctypes.byref(ch), ctypes.byref(off)))
            self.offsets.append(off.value)
            self.molecules.append(Context._borrowed(self.lib, ch, model, n))
        self.total = sum(self.sizes)

    def _check(self, status: int):
        if status != GBX_OK:
            buf = ctypes.create_string_buffer(512)
            self.lib.gbx_batch_last_error(self.h, buf, 512)
            raise GBXError(status, buf.value.decode())

    def close(self):
        if getattr(self, "h", None):
            for c in self.molecules:
                c.h = None
            self.lib.gbx_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def buffers(self):
        """Device addresses: (posq float4 [total], forces u64 [3 total], energies f64 [molecules])."""
        p, f, e, t = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_longlong()
        self._check(self.lib.gbx_batch_buffers(self.h, ctypes.byref(p), ctypes.byref(f), ctypes.byref(e),
                                               ctypes.byref(t)))
        return p.value, f.value, e.value

    def execute_device(self, flags: int = 0, stream: int = 0):
        self._check(self.lib.gbx_batch_execute(self.h, int(flags), ctypes.c_void_p(stream or None)))

    def adjoint_device(self, energies: int, forces: int, dEdq: int, dEdR: int, dEdalpha: int, flags: int = 0,
                       stream: int = 0):
        """gbx_batch_adjoint on device FP64 arrays (addresses; 0 for none)."""
        v = lambda a: ctypes.c_void_p(a or None)  # noqa: E731
        self._check(self.lib.gbx_batch_adjoint(self.h, v(energies), v(forces), v(dEdq), v(dEdR), v(dEdalpha),
                                               int(flags), ctypes.c_void_p(stream or None)))

    def adjoint_host(self, positions):
        """Energies [molecules], forces [total, 3], dEdq [total], dEdR [total], dEdalpha [molecules, 2]."""
        x = np.ascontiguousarray(positions, dtype=np.float64)
        if x.shape != (self.total, 3):
            raise GBXError(1, "positions must be [total atoms, 3]")
        M = len(self.sizes)
        out = {"energies": np.zeros(M), "forces": np.zeros((self.total, 3)), "dEdq": np.zeros(self.total),
               "dEdR": np.zeros(self.total), "dEdalpha": np.zeros((M, 2))}
        self._check(self.lib.gbx_batch_adjoint_host(self.h, _p(x), _p(out["energies"]), _p(out["forces"]),
                                                    _p(out["dEdq"]), _p(out["dEdR"]), _p(out["dEdalpha"])))
        return out

    def execute_host(self, positions):
        x = np.ascontiguousarray(positions, dtype=np.float64)
        if x.shape != (self.total, 3):
            raise GBXError(1, "positions must be [total atoms, 3]")
        F = np.zeros((self.total, 3))
        E = np.zeros(len(self.sizes))
        self._check(self.lib.gbx_batch_execute_host(self.h, _p(x), _p(F), _p(E)))
        return E, F

    def tune(self):
        s, d, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        self._check(self.lib.gbx_batch_tune(self.h, ctypes.byref(s), ctypes.byref(d), ctypes.byref(ms)))
        return {"streams": s.value, "chunk_divisor": d.value, "ms_per_call": ms.value}
