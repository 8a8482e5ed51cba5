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


def parse(text: str, names) -> sp.Expr:
    """Lepton syntax ("expr; a = ...; b = ...") -> sympy, over the given variable names."""
    parts = [p.strip() for p in text.split(";")]
    local = dict(_FUNCS)
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
    return sp.lambdify(syms, e, modules=[{"Heaviside": lambda x, h=1: np.heaviside(x, h)}, "numpy"])


def _ev(e, env, count):
    syms = sorted(e.free_symbols, key=str)
    return np.broadcast_to(np.asarray(_lam(e, syms)(*[env[str(s)] for s in syms]), float), (count,))


class CustomOracle:
    """``custom`` as for ``_lib.CustomContext``; ``model`` gives the integral
    class, quadrature and table (its ``orders`` are replaced by the
    integrals')."""

    def __init__(self, model, custom):
        self.custom = custom
        orders = tuple(int(o) for _, o in custom["integrals"])
        self.model = model.replace(orders=orders)
        self.params = list(custom["params"])
        self.globals = dict(custom.get("globals", {}))
        self.integrals = [k for k, _ in custom["integrals"]]
        self.values = list(custom.get("values", []))
        self.terms = list(custom["terms"])
        vnames = [v for v, _ in self.values]
        single_names = self.params + list(self.globals) + self.integrals + vnames
        pair_names = ["r"] + list(self.globals) + [f"{x}{s}" for x in self.params + self.integrals + vnames
                                                   for s in "12"]
        self.vexpr = [parse(e, single_names) for _, e in self.values]
        self.texpr = [(parse(e, single_names if t == 0 else pair_names), t) for e, t in self.terms]

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
        V, dVdI = [], []
        for m, (name, _) in enumerate(self.values):
            e = self.vexpr[m]
            V.append(_ev(e, env, n).copy())
            d = []
            for k in range(ni):  # total derivative: the partial plus the chain through earlier values
                tot = _ev(sp.diff(e, sp.Symbol(self.integrals[k])), env, n).copy()
                for l in range(m):
                    tot += _ev(sp.diff(e, sp.Symbol(vnames[l])), env, n) * dVdI[l][k]
                d.append(tot)
            dVdI.append(d)
            env[name] = V[-1]
        E = 0.0
        F = np.zeros((n, 3))
        dEdV = np.zeros((nv, n))
        dEdI = np.zeros((ni, n))
        for e, t in self.texpr:
            if t != 0:
                continue
            E += float(_ev(e, env, n).sum())
            for m, v in enumerate(vnames):
                dEdV[m] += _ev(sp.diff(e, sp.Symbol(v)), env, n)
            for k, name in enumerate(self.integrals):
                dEdI[k] += _ev(sp.diff(e, sp.Symbol(name)), env, n)
        pair_terms = [e for e, t in self.texpr if t == 1]
        if pair_terms:
            a, b = np.triu_indices(n, k=1)  # atom 1 = a < atom 2 = b
            d = pos[a] - pos[b]
            if self.model.periodic:
                L = np.asarray(self.model.box, float)
                d -= L * np.floor(d / L + 0.5)
            r = np.sqrt((d ** 2).sum(axis=1))
            keep = r < self.model.cutoff if self.model.cutoff > 0 else np.ones(len(r), bool)
            a, b, d, r = a[keep], b[keep], d[keep], r[keep]
            m_ = len(r)
            penv = {"r": r}
            penv.update({g: np.full(m_, v) for g, v in self.globals.items()})
            for x in self.params + self.integrals + vnames:
                arr = env[x]
                penv[x + "1"] = arr[a]
                penv[x + "2"] = arr[b]
            for e in pair_terms:
                E += float(_ev(e, penv, m_).sum())
                g = _ev(sp.diff(e, sp.Symbol("r")), penv, m_) / r
                fpair = -g[:, None] * d  # force on atom 1 (d = x1 - x2)
                np.add.at(F, a, fpair)
                np.add.at(F, b, -fpair)
                for m, v in enumerate(vnames):
                    np.add.at(dEdV[m], a, _ev(sp.diff(e, sp.Symbol(v + "1")), penv, m_))
                    np.add.at(dEdV[m], b, _ev(sp.diff(e, sp.Symbol(v + "2")), penv, m_))
                for k, name in enumerate(self.integrals):
                    np.add.at(dEdI[k], a, _ev(sp.diff(e, sp.Symbol(name + "1")), penv, m_))
                    np.add.at(dEdI[k], b, _ev(sp.diff(e, sp.Symbol(name + "2")), penv, m_))
        tot = dEdI.copy()
        for m in range(nv):
            for k in range(ni):
                tot[k] += dEdV[m] * dVdI[m][k]
        Fc, _ = orc.integral_chain(pos, radius, tot.reshape(-1))
        F += Fc
        return {"energy": E, "forces": F, "values": np.array(V), "integrals": I, "dEdV": dEdV}
