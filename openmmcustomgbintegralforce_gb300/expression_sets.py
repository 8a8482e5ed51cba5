"""Example expression sets for the compiled CharmmGBMVForce path (used by the
tests and the benchmark).

CANONICAL is the canonical CHARMM set written as user expressions.  MODIFIED
is outside it: a per-atom scale of the Born radius through a second computed
value, the solvent dielectric as a global parameter, an ACE-style nonpolar
single-particle term and a Lepton definition in the pair term.  EXTENDED
adds coordinates, exclusions and energy parameter derivatives; TABULATED
calls tabulated functions; FUNCTIONS uses the Lepton function set.
"""
from openmmcustomgbintegralforce_gb300.spec import ONE_4PI_EPS0

K = repr(ONE_4PI_EPS0)

CANONICAL = {
    "params": ["q", "radius"],
    "globals": {"alpha0": -0.180, "alpha1": 1.817},
    "integrals": [("I4", 4), ("I7", 7)],
    "values": [("B", "1/(alpha0*(1/0.05-I4)+alpha1*(1/(4*0.05^4)-I7)^(1/4))")],
    "terms": [(f"-0.5*{K}*(1-1/80)*q^2/B", 0),
              (f"-{K}*(1-1/80)*q1*q2/sqrt(r^2+B1*B2*exp(-r^2/(4*B1*B2)))", 1)],
}

MODIFIED = {
    "params": ["q", "radius", "s"],
    "globals": {"alpha0": -0.180, "alpha1": 1.817, "eps": 78.5, "gamma": 0.54},
    "integrals": [("I4", 4), ("I7", 7)],
    "values": [("B", "1/(alpha0*(1/0.05-I4)+alpha1*(1/(4*0.05^4)-I7)^(1/4))"),
               ("Bs", "s*B")],
    "terms": [(f"-0.5*{K}*(1-1/eps)*q^2/Bs", 0),
              ("gamma*4*3.14159265*(radius+0.14)^2*(radius/Bs)^6", 0),
              (f"-{K}*(1-1/eps)*q1*q2/f; f=sqrt(r^2+Bs1*Bs2*exp(-D)); D=r^2/(4*Bs1*Bs2)", 1)],
}


def modified_params(g, seed=0):
    import numpy as np

    rng = np.random.default_rng(seed)
    s = 0.9 + 0.2 * rng.random(g.n)
    return np.stack([g.charge, g.radius, s], axis=1)


# Outside the canonical set in the ways the compiled path supports beyond
# MODIFIED: a computed value and a single-particle term that read the atom's
# coordinates (a slab-like dielectric scaling along z and a harmonic
# restraint), a ParticlePair term (excluded pairs skipped) beside a
# ParticlePairNoExclusions term, and energy derivatives by two globals.
EXTENDED = {
    "params": ["q", "radius"],
    "globals": {"alpha0": -0.180, "alpha1": 1.817, "eps": 78.5, "kr": 2.0},
    "integrals": [("I4", 4), ("I7", 7)],
    "values": [("B", "1/(alpha0*(1/0.05-I4)+alpha1*(1/(4*0.05^4)-I7)^(1/4))"),
               ("Bz", "B*(1+0.1*tanh(z-zc)); zc=1.3")],
    "terms": [(f"-0.5*{K}*(1-1/eps)*q^2/Bz", 0),
              ("kr*((x-1.2)^2+(y-1.3)^2)", 0),
              (f"-{K}*(1-1/eps)*q1*q2/f; f=sqrt(r^2+Bz1*Bz2*exp(-r^2/(4*Bz1*Bz2)))", 1),
              ("0.01*q1*q2/(r+0.3)", 2)],
    "param_derivs": ["eps", "kr"],
}


def extended_exclusions(n, seed=0):
    """Pairs of near neighbours in index order, as bonded exclusions would be."""
    import numpy as np

    rng = np.random.default_rng(seed)
    out = set()
    for i in range(n - 1):
        out.add((i, i + 1))
        if i + 2 < n and rng.random() < 0.5:
            out.add((i, i + 2))
    return sorted(out)


def tabulated_functions():
    """Two Continuous1DFunction tables: a smooth scaling of a radius over
    [0.05, 3] nm, and a pair correction over [0, 2] nm that goes to zero
    with zero slope at its upper end (beyond it the function is zero, so
    the farther pairs of a 1,000-atom globule fall outside the table)."""
    import numpy as np

    x = np.linspace(0.05, 3.0, 40)
    scale = 1.0 + 0.2 * np.sin(3.0 * x) * np.exp(-x)
    r = np.linspace(0.0, 2.0, 61)
    tail = 0.5 * np.exp(-r) * np.cos(3.0 * r) * (1.0 - (r / 2.0) ** 2) ** 2
    return {"scale": (scale.tolist(), 0.05, 3.0), "tail": (tail.tolist(), 0.0, 2.0)}


# Tabulated functions (addTabulatedFunction with Continuous1DFunction) in a
# computed value, a single-particle term and a pair term.
TABULATED = {
    "params": ["q", "radius"],
    "globals": {"alpha0": -0.180, "alpha1": 1.817},
    "integrals": [("I4", 4), ("I7", 7)],
    "values": [("B", "1/(alpha0*(1/0.05-I4)+alpha1*(1/(4*0.05^4)-I7)^(1/4))"),
               ("Bt", "B*scale(B)")],
    "terms": [(f"-0.5*{K}*(1-1/80)*q^2/Bt", 0),
              ("0.01*scale(10*radius)", 0),
              (f"-{K}*(1-1/80)*q1*q2/sqrt(r^2+Bt1*Bt2*exp(-r^2/(4*Bt1*Bt2)))", 2),
              ("q1*q2*tail(r)", 2)],
    "functions": tabulated_functions(),
}


# The Lepton function set in a computed value, a single-particle term and a
# pair term (smooth where the globule's values fall, so central differences
# and FP32 both apply).
FUNCTIONS = {
    "params": ["q", "radius"],
    "globals": {"alpha0": -0.180, "alpha1": 1.817},
    "integrals": [("I4", 4), ("I7", 7)],
    "values": [("B", "1/(alpha0*(1/0.05-I4)+alpha1*(1/(4*0.05^4)-I7)^(1/4))"),
               ("Bf", "B*(1+0.05*erf(q))*(1+0.02*tanh(B-0.3))")],
    "terms": [(f"-0.5*{K}*(1-1/80)*q^2/Bf", 0),
              ("0.01*(abs(q) + step(q)*square(q) + select(step(radius-0.15), 1, 2)*sqrt(radius)"
               " + min(radius, 0.16) + max(radius, 0.14) + log(radius) + exp(-radius) + sin(radius)"
               " + cos(radius) + atan(radius) + cosh(radius)/sinh(radius+1) + recip(radius+1)"
               " + cube(radius) + erfc(radius) + tan(radius) + asin(radius) + acos(radius))", 0),
              (f"-{K}*(1-1/80)*q1*q2/sqrt(r^2+Bf1*Bf2*exp(-r^2/(4*Bf1*Bf2)))", 2),
              ("0.01*q1*q2*exp(-r)*(1+0.1*cos(3*r))*atan(Bf1+Bf2) + 0.001*erfc(r)*min(Bf1, Bf2)", 2)],
}
