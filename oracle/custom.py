"""FP64 oracle for CharmmGBMVForce expressions outside the canonical CHARMM
set -- TEST INFRASTRUCTURE (only tests/ may use it; the product never does).

It restates the reference's generic CharmmGBMVForce evaluation
(CharmmReferenceGBMV.cpp:151-444): the GB integrals (from the C oracle,
``orc_integrals``), the computed values in order
(``calculateSingleParticleValue``, :207-230), the single-particle and
pair energy terms over every pair i < j with atom 1 the lower index
(``calculateParticlePairEnergyTerm`` / ``calculateOnePairEnergyTerm``,
:268-347), and the chain rule through the values into the integrals and
through every quadrature point to the atoms (``calculateChainRuleForces``,
:349-384; the point-by-point chain of the C oracle, ``orc_integral_chain``).
Expressions are parsed and differentiated with sympy, independently of the
library's own expression compiler, and evaluated in FP64 with numpy.
"""
from __future__ import annotations

import numpy as np
import sympy as sp

from oracle import oracle as O

_FUNCS = {
    "sqrt": sp.sqrt, "exp": sp.exp, "log": sp.log, "sin": sp.sin, "cos": sp.cos, "tan": sp.tan,
    "asin": sp.asin, "acos": sp.acos, "atan": sp.atan, "sinh": sp.sinh, "cosh": sp.cosh, "tanh": sp.tanh,
    "erf": sp.erf, "erfc": sp.erfc, "abs": sp.Abs, "min": sp.Min, "max": sp.Max,
    "step": lambda x: sp.Heaviside(x, 1), "square": lambda x: x ** 2, "cube": lambda x: x ** 3,
    "recip": lambda x: 1 / x, "floor": sp.floor, "ceil": sp.ceiling,
    "select": lambda c, a, b: sp.Piecewise((a, sp.Ne(c, 0)), (b, True)),
}


def tabulated(functions: dict) -> dict:
    """sympy functions for a force's Continuous1DFunction tables ({name:
    (values, min, max)}): the natural cubic spline through the evenly spaced
    values (scipy's CubicSpline with bc_type="natural", an implementation
    independent of the library's), zero outside [min, max]; differentiating
    gives the spline's first and second derivatives."""
    from scipy.interpolate import CubicSpline

    out = {}
    for name, (vals, lo, hi) in functions.items():
        cs = CubicSpline(np.linspace(lo, hi, len(vals)), np.asarray(vals, float), bc_type="natural")
        classes = []
        for d in range(3):
            f = cs if d == 0 else cs.derivative(d)

            def impl(t, f=f, lo=lo, hi=hi):
                t = np.asarray(t, float)
                return np.where((t >= lo) & (t <= hi), f(np.clip(t, lo, hi)), 0.0)

            classes.append(type(f"{name}_d{d}", (sp.Function,), {"nargs": 1, "_imp_": staticmethod(impl)}))
        for d in range(2):
            classes[d].fdiff = (lambda nxt: lambda self, argindex=1: nxt(self.args[0]))(classes[d + 1])
        out[name] = classes[0]
    return out


def parse(text: str, names, functions=None) -> sp.Expr:
    """Lepton syntax ("expr; a = ...; b = ...") -> sympy, over the given
    variable names and tabulated functions (``tabulated``)."""
    parts = [p.strip() for p in text.split(";")]
    local = dict(_FUNCS)
    local.update(functions or {})
    for n in names:
        local[n] = sp.Symbol(n)

    def conv(s):
        return sp.sympify(s.replace("^", "**"), locals=local)

    main = conv(parts[0])
    defs = {}
    for d in parts[1:]:
        if not d:
            continue
        k, v = d.split("=", 1)
        defs[k.strip()] = conv(v.strip())
    for _ in range(len(defs) + 1):  # definitions may use later ones
        main = main.subs({sp.Symbol(k): v for k, v in defs.items()})
        defs = {k: v.subs({sp.Symbol(kk): vv for kk, vv in defs.items() if kk != k}) for k, v in defs.items()}
    return main


def _lam(e, syms):
    # scipy supplies the array forms of erf and erfc
    return sp.lambdify(syms, e, modules=[{"Heaviside": lambda x, h=1: np.heaviside(x, h)}, "numpy", "scipy"])


def _ev(e, env, count):
    syms = sorted(e.free_symbols, key=str)
    return np.broadcast_to(np.asarray(_lam(e, syms)(*[env[str(s)] for s in syms]), float), (count,))


class CustomOracle:
    """``custom`` as for ``_lib.CustomContext``; ``model`` gives the integral
    class, quadrature and table (its ``orders`` are replaced by the
    integrals').  Term types: 0 single particle, 1 particle pair (excluded
    pairs skipped, CharmmReferenceGBMV.cpp:272-284), 2 particle pair without
    exclusions.  Computed values and single-particle terms may read the
    atom's coordinates x, y, z (their gradients are forces,
    CharmmReferenceGBMV.cpp:232-262,409-435); ``param_derivs`` names globals
    whose energy derivative is returned (:225-229,263-264,438-443);
    ``functions`` holds Continuous1DFunction tables ({name: (values, min,
    max)}, CharmmReferenceKernels.cpp:187-191 hands them to Lepton as custom
    functions)."""

    def __init__(self, model, custom):
        self.custom = custom
        orders = tuple(int(o) for _, o in custom["integrals"])
        self.model = model.replace(orders=orders)
        self.params = list(custom["params"])
        self.globals = dict(custom.get("globals", {}))
        self.integrals = [k for k, _ in custom["integrals"]]
        self.values = list(custom.get("values", []))
        self.terms = list(custom["terms"])
        self.exclusions = [tuple(sorted(e)) for e in custom.get("exclusions", [])]
        self.param_derivs = list(custom.get("param_derivs", []))
        vnames = [v for v, _ in self.values]
        single_names = self.params + list(self.globals) + self.integrals + vnames + ["x", "y", "z"]
        pair_names = ["r"] + list(self.globals) + [f"{x}{s}" for x in self.params + self.integrals + vnames
                                                   for s in "12"]
        fns = tabulated(custom.get("functions", {}))
        self.vexpr = [parse(e, single_names, fns) for _, e in self.values]
        self.texpr = [(parse(e, single_names if t == 0 else pair_names, fns), t) for e, t in self.terms]

    def energy_forces(self, pos, params):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        params = np.asarray(params, dtype=np.float64)
        n = len(pos)
        radius = params[:, self.params.index("radius")]
        orc = O.Oracle(self.model)
        I, _ = orc.integrals(pos, radius)  # [ni][n]
        ni, nv = len(self.integrals), len(self.values)
        vnames = [v for v, _ in self.values]
        env = {p: params[:, k] for k, p in enumerate(self.params)}
        env.update({g: np.full(n, v) for g, v in self.globals.items()})
        env.update({name: I[k] for k, name in enumerate(self.integrals)})
        env.update({"x": pos[:, 0], "y": pos[:, 1], "z": pos[:, 2]})
        coords = ("x", "y", "z")
        V, dVdI, dVdX, dVdG = [], [], [], []
        for m, (name, _) in enumerate(self.values):
            e = self.vexpr[m]
            V.append(_ev(e, env, n).copy())

            def total(var, earlier):  # the partial plus the chain through earlier values
                t = _ev(sp.diff(e, sp.Symbol(var)), env, n).copy()
                for l in range(m):
                    t += _ev(sp.diff(e, sp.Symbol(vnames[l])), env, n) * earlier[l]
                return t

            dVdI.append([total(self.integrals[k], [d[k] for d in dVdI]) for k in range(ni)])
            dVdX.append([total(c, [d[a] for d in dVdX]) for a, c in enumerate(coords)])
            dVdG.append([total(g, [d[k] for d in dVdG]) for k, g in enumerate(self.param_derivs)])
            env[name] = V[-1]
        E = 0.0
        F = np.zeros((n, 3))
        dEdV = np.zeros((nv, n))
        dEdI = np.zeros((ni, n))
        dEdG = np.zeros(len(self.param_derivs))
        for e, t in self.texpr:
            if t != 0:
                continue
            E += float(_ev(e, env, n).sum())
            for m, v in enumerate(vnames):
                dEdV[m] += _ev(sp.diff(e, sp.Symbol(v)), env, n)
            for k, name in enumerate(self.integrals):
                dEdI[k] += _ev(sp.diff(e, sp.Symbol(name)), env, n)
            for a, c in enumerate(coords):
                F[:, a] -= _ev(sp.diff(e, sp.Symbol(c)), env, n)
            for k, g in enumerate(self.param_derivs):
                dEdG[k] += float(_ev(sp.diff(e, sp.Symbol(g)), env, n).sum())
        pair_terms = [(e, t) for e, t in self.texpr if t != 0]
        if pair_terms:
            a, b = np.triu_indices(n, k=1)  # atom 1 = a < atom 2 = b
            d = pos[a] - pos[b]
            if self.model.periodic:
                L = np.asarray(self.model.box, float)
                d -= L * np.floor(d / L + 0.5)
            r = np.sqrt((d ** 2).sum(axis=1))
            keep = r < self.model.cutoff if self.model.cutoff > 0 else np.ones(len(r), bool)
            excluded = np.zeros(len(r), bool)
            if self.exclusions:
                ex = {i * n + j for i, j in self.exclusions}
                excluded = np.fromiter((int(i) * n + int(j) in ex for i, j in zip(a, b)), bool, count=len(a))
            for e, t in pair_terms:
                sel = keep & ~excluded if t == 1 else keep
                aa, bb, dd, rr = a[sel], b[sel], d[sel], r[sel]
                m_ = len(rr)
                penv = {"r": rr}
                penv.update({g: np.full(m_, v) for g, v in self.globals.items()})
                for x in self.params + self.integrals + vnames:
                    arr = env[x]
                    penv[x + "1"] = arr[aa]
                    penv[x + "2"] = arr[bb]
                E += float(_ev(e, penv, m_).sum())
                g = _ev(sp.diff(e, sp.Symbol("r")), penv, m_) / rr
                fpair = -g[:, None] * dd  # force on atom 1 (d = x1 - x2)
                np.add.at(F, aa, fpair)
                np.add.at(F, bb, -fpair)
                for mm, v in enumerate(vnames):
                    np.add.at(dEdV[mm], aa, _ev(sp.diff(e, sp.Symbol(v + "1")), penv, m_))
                    np.add.at(dEdV[mm], bb, _ev(sp.diff(e, sp.Symbol(v + "2")), penv, m_))
                for k, name in enumerate(self.integrals):
                    np.add.at(dEdI[k], aa, _ev(sp.diff(e, sp.Symbol(name + "1")), penv, m_))
                    np.add.at(dEdI[k], bb, _ev(sp.diff(e, sp.Symbol(name + "2")), penv, m_))
                for k, gname in enumerate(self.param_derivs):
                    dEdG[k] += float(_ev(sp.diff(e, sp.Symbol(gname)), penv, m_).sum())
        tot = dEdI.copy()
        for m in range(nv):
            for k in range(ni):
                tot[k] += dEdV[m] * dVdI[m][k]
            for a_ in range(3):
                F[:, a_] -= dEdV[m] * dVdX[m][a_]
            for k in range(len(self.param_derivs)):
                dEdG[k] += float((dEdV[m] * dVdG[m][k]).sum())
        Fc, _ = orc.integral_chain(pos, radius, tot.reshape(-1))
        F += Fc
        return {"energy": E, "forces": F, "values": np.array(V), "integrals": I, "dEdV": dEdV,
                "param_derivs": dEdG}
