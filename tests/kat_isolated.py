"""Known answer for isolated atoms (no test functions here).

For an atom whose quadrature points no other atom reaches, the GBSW
solvent fraction of a point depends only on its distance r from the atom:
V(r) = u(r - R') with R' = (R + 0.03) 0.952 (CharmmReferenceGBSW.cpp:616-639),
u = 0 inside R' - w, 1 outside R' + w and 1/2 + 3/(4w) dr - dr^3/(4w^3) in
the switching shell.  The Lebedev weights sum to 1, so the integrals
I_n = sum_q w_q (1 - V)/r^(n-2) reduce to one-dimensional Gauss-Legendre sums
over the radial nodes, and the Born radius follows from
CharmmReferenceGBSW.cpp:591-593.  The continuous integral of the same
integrand is given for a looser check of the quadrature itself.
"""
import numpy as np

from openmmcustomgbintegralforce_gb300.quadrature import gauss_legendre


def radius_prime(R):
    return (np.asarray(R, dtype=np.float64) + 0.03) * 0.952


def solute_fraction(r, Rp, w):
    """1 - V(r) for an isolated atom of switching radius Rp."""
    dr = r - Rp
    u = 0.5 + 3.0 / (4.0 * w) * dr - dr ** 3 / (4.0 * w ** 3)
    return np.where(r <= Rp - w, 1.0, np.where(r >= Rp + w, 0.0, 1.0 - u))


def expected_integrals(model, radius):
    """(I4, I7) per atom from the radial Gauss-Legendre nodes of the model."""
    xr, wr = gauss_legendre(model.r0, model.r1, model.n_radial)
    xr, wr = np.asarray(xr), np.asarray(wr)
    I4, I7 = [], []
    for R in np.atleast_1d(radius):
        f = solute_fraction(xr, radius_prime(R), model.sw)
        I4.append(float(np.sum(wr * f / xr ** 2)))
        I7.append(float(np.sum(wr * f / xr ** 5)))
    return np.array(I4), np.array(I7)


def expected_born(model, I4, I7):
    r0 = model.r0
    inv = model.alpha0 * (1.0 / r0 - I4) + model.alpha1 * (1.0 / (4.0 * r0 ** 4) - I7) ** 0.25
    return 1.0 / inv


def continuous_integrals(model, R):
    """The integrals the quadrature approximates, by adaptive integration."""
    from scipy.integrate import quad

    Rp, w = float(radius_prime(R)), model.sw
    pts = [Rp - w, Rp + w]

    def I(n):
        return quad(lambda r: float(solute_fraction(np.array(r), Rp, w)) / r ** (n - 2), model.r0, model.r1,
                    points=pts, limit=200)[0]

    return I(4), I(7)


def isolated_system(radii, spacing=8.0):
    """Atoms on the x axis, `spacing` nm apart (farther than any point reaches)."""
    radii = np.asarray(radii, dtype=np.float64)
    pos = np.zeros((len(radii), 3))
    pos[:, 0] = spacing * np.arange(len(radii))
    return pos, radii
