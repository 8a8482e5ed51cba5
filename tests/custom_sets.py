"""Expression sets for the custom CharmmGBMVForce path (shared by tests).

CANONICAL is the canonical CHARMM set written as user expressions.  MODIFIED
is outside it: a per-atom scale of the Born radius through a second computed
value, the solvent dielectric as a global parameter, an ACE-style nonpolar
single-particle term and a Lepton definition in the pair term.
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
