"""Radial x angular quadrature used by the Born-radius integrals.

The reference builds every integral's quadrature as a tensor product of a
Gauss-Legendre rule on [r0, r1] and a Lebedev rule on the unit sphere
(``CharmmReferenceGBSW.cpp:29-46``, ``GBSWIntegral.cpp:37-56``,
``platforms/cuda/src/CustomGBIntegral.cpp:173-206``).  Point ``idx = ir*nS + is``
sits at ``r_ir * u_is`` with weight ``w_ir * w_is``; Lebedev weights sum to 1.

Both rules are generated here from their mathematics, not read from a table:

* Gauss-Legendre: Newton iteration on the Legendre recurrence, the published
  ``gauleg`` procedure (Press et al., Numerical Recipes, 2nd ed., sec. 4.5),
  which is the procedure ``CharmmQuadrature.h:47-75`` follows.  The iteration
  below performs the same floating-point operations in the same order, so the
  abscissae and weights come out bit-identical to the reference's.
* Lebedev: the octahedrally symmetric rules of Lebedev & Laikov (Doklady Math.
  59 (1999) 477).  Each rule is a fixed set of orbits (a1, a2, a3, b_k, c_k);
  the orbit weights and free coordinates are solved here from the requirement
  that every even monomial x^2a y^2b z^2c up to the rule's degree is
  integrated exactly over the sphere (Levenberg-Marquardt on the moment
  equations, then Newton polish in extended precision).  The solved rules are
  frozen into ``csrc/lebedev_rules.h`` by ``python -m
  openmmcustomgbintegralforce_gb300.quadrature --emit-header``.
"""
from __future__ import annotations

import itertools
import math
import sys
from functools import lru_cache

import numpy as np

# order -> (degree, orbit list).  Orbit codes: 'a1' 6 pts (1,0,0); 'a2' 12 pts
# (0,s,s) s=1/sqrt2; 'a3' 8 pts (c,c,c) c=1/sqrt3; 'b' 24 pts (l,l,m);
# 'c' 24 pts (p,q,0).  Rule numbering follows the 65-rule Lebedev-Laikov
# sequence used by CharmmQuadrature::Lebedev(rule) (rule 3 -> 26 points,
# 4 -> 38, 5 -> 50, 8 -> 110; CharmmQuadrature.h:6833-6840).
LEBEDEV_ORBITS = {
    6: (3, ["a1"]),
    14: (5, ["a1", "a3"]),
    26: (7, ["a1", "a2", "a3"]),
    38: (9, ["a1", "a3", "c"]),
    50: (11, ["a1", "a2", "a3", "b"]),
    74: (13, ["a1", "a2", "a3", "b", "c"]),
    86: (15, ["a1", "a3", "b", "b", "c"]),
    110: (17, ["a1", "a3", "b", "b", "b", "c"]),
}
LEBEDEV_RULE_TO_ORDER = {1: 6, 2: 14, 3: 26, 4: 38, 5: 50, 6: 74, 7: 86, 8: 110}


def gauss_legendre(x0: float, x1: float, n: int):
    """Gauss-Legendre abscissae (ascending) and weights on [x0, x1].

    Restates the Numerical Recipes ``gauleg`` Newton iteration that
    ``CharmmQuadrature.h:47-75`` uses: initial guess cos(pi (i-1/4)/(n+1/2)),
    three-term Legendre recurrence, stop once |z - z_prev| <= 3e-14.  The
    weight uses the derivative from the last Newton step, as the reference
    does.  (The reference reads ``z1`` before assigning it; the loop below
    always runs at least one Newton step, which is what the reference does in
    practice.)
    """
    eps = 3.0e-14
    pi = 3.14159265358979323846264338327950
    x = [0.0] * n
    w = [0.0] * n
    m = (n + 1) // 2
    xm = 0.5 * (x1 + x0)
    xl = 0.5 * (x1 - x0)
    for i in range(1, m + 1):
        z = math.cos(pi * (i - 0.25) / (n + 0.5))
        first = True
        z1 = 0.0
        pp = 0.0
        while first or abs(z - z1) > eps:
            first = False
            p1 = 1.0
            p2 = 0.0
            for j in range(1, n + 1):
                p3 = p2
                p2 = p1
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j
            pp = n * (z * p1 - p2) / (z * z - 1.0)
            z1 = z
            z = z1 - p1 / pp
        x[i - 1] = xm - xl * z
        x[n - i] = xm + xl * z
        w[i - 1] = 2.0 * xl / ((1.0 - z * z) * pp * pp)
        w[n - i] = w[i - 1]
    return np.array(x), np.array(w)


def _orbit_points(code: str, param: float | None = None) -> np.ndarray:
    pts = []
    if code == "a1":
        for ax in range(3):
            for s in (1.0, -1.0):
                v = [0.0, 0.0, 0.0]
                v[ax] = s
                pts.append(v)
    elif code == "a2":
        a = math.sqrt(0.5)
        for zero in range(3):
            others = [k for k in range(3) if k != zero]
            for s1 in (1.0, -1.0):
                for s2 in (1.0, -1.0):
                    v = [0.0, 0.0, 0.0]
                    v[others[0]] = s1 * a
                    v[others[1]] = s2 * a
                    pts.append(v)
    elif code == "a3":
        a = math.sqrt(1.0 / 3.0)
        for s1 in (1.0, -1.0):
            for s2 in (1.0, -1.0):
                for s3 in (1.0, -1.0):
                    pts.append([s1 * a, s2 * a, s3 * a])
    elif code == "b":
        l = param
        m = math.sqrt(max(0.0, 1.0 - 2.0 * l * l))
        for odd in range(3):  # axis holding m
            for s1 in (1.0, -1.0):
                for s2 in (1.0, -1.0):
                    for s3 in (1.0, -1.0):
                        v = [s1 * l, s2 * l, s3 * l]
                        v[odd] = [s1, s2, s3][odd] * m
                        pts.append(v)
    elif code == "c":
        p = param
        q = math.sqrt(max(0.0, 1.0 - p * p))
        for zero in range(3):
            others = [k for k in range(3) if k != zero]
            for (u, v_) in ((p, q), (q, p)):
                for s1 in (1.0, -1.0):
                    for s2 in (1.0, -1.0):
                        v = [0.0, 0.0, 0.0]
                        v[others[0]] = s1 * u
                        v[others[1]] = s2 * v_
                        pts.append(v)
    else:
        raise ValueError(code)
    return np.array(pts, dtype=np.float64)


def _dfact(k: int) -> int:
    r = 1
    while k > 1:
        r *= k
        k -= 2
    return r


def _moments(degree: int):
    """Sorted even exponent triples (a>=b>=c) with 2(a+b+c) <= degree and the
    exact sphere averages (2a-1)!!(2b-1)!!(2c-1)!!/(2n+1)!!."""
    out = []
    nmax = degree // 2
    for n in range(nmax + 1):
        for a in range(n, -1, -1):
            for b in range(min(a, n - a), -1, -1):
                c = n - a - b
                if c < 0 or c > b:
                    continue
                exact = _dfact(2 * a - 1) * _dfact(2 * b - 1) * _dfact(2 * c - 1) / _dfact(2 * n + 1)
                out.append((a, b, c, exact))
    return out


def _residual(theta, orbits, moments):
    nw = len(orbits)
    weights = theta[:nw]
    params = theta[nw:]
    res = np.zeros(len(moments))
    pi = 0
    for o, code in enumerate(orbits):
        if code in ("b", "c"):
            pts = _orbit_points(code, params[pi])
            pi += 1
        else:
            pts = _orbit_points(code)
        x2, y2, z2 = pts[:, 0] ** 2, pts[:, 1] ** 2, pts[:, 2] ** 2
        for k, (a, b, c, _) in enumerate(moments):
            res[k] += weights[o] * np.sum(x2 ** a * y2 ** b * z2 ** c)
    for k, m in enumerate(moments):
        res[k] -= m[3]
    return res


def _polish_mp(theta, orbits, moments, digits: int = 40):
    """Gauss-Newton polish of the moment equations in ``digits``-digit
    arithmetic (mpmath), then round once to double."""
    import mpmath as mp

    mp.mp.dps = digits
    nw = len(orbits)

    def orbit_sums(code, param):
        # Sum over one orbit of x^2a y^2b z^2c for every moment.  An orbit is
        # the distinct permutations of a squared-coordinate triple, each with
        # 2^(nonzero coordinates) sign patterns.
        if code == "a1":
            sq = (mp.mpf(1), mp.mpf(0), mp.mpf(0))
        elif code == "a2":
            sq = (mp.mpf(0), mp.mpf(1) / 2, mp.mpf(1) / 2)
        elif code == "a3":
            sq = (mp.mpf(1) / 3,) * 3
        elif code == "b":
            l2 = param * param
            sq = (l2, l2, 1 - 2 * l2)
        else:
            p2 = param * param
            sq = (p2, 1 - p2, mp.mpf(0))
        triples = []
        for perm in itertools.permutations(range(3)):
            t = tuple(sq[k] for k in perm)
            if t not in triples:
                triples.append(t)
        out = []
        for (a, b, c, _) in moments:
            acc = mp.mpf(0)
            for t in triples:
                nz = sum(1 for v in t if v != 0)
                acc += (2 ** nz) * (t[0] ** a if a else 1) * (t[1] ** b if b else 1) * (t[2] ** c if c else 1)
            out.append(acc)
        return out

    th = [mp.mpf(float(v)) for v in theta]
    exact = [mp.mpf(_dfact(2 * a - 1) * _dfact(2 * b - 1) * _dfact(2 * c - 1)) / _dfact(2 * (a + b + c) + 1)
             for (a, b, c, _) in moments]

    def resid(t):
        r = [-e for e in exact]
        pi = 0
        for o, code in enumerate(orbits):
            param = None
            if code in ("b", "c"):
                param = t[nw + pi]
                pi += 1
            s = orbit_sums(code, param)
            for k in range(len(r)):
                r[k] += t[o] * s[k]
        return r

    for _ in range(6):
        r = resid(th)
        J = mp.matrix(len(r), len(th))
        for k in range(len(th)):
            h = mp.mpf(10) ** (-digits // 2)
            tp = list(th); tp[k] += h
            tm = list(th); tm[k] -= h
            rp, rm = resid(tp), resid(tm)
            for i in range(len(r)):
                J[i, k] = (rp[i] - rm[i]) / (2 * h)
        # normal equations
        JT = J.T
        step = mp.lu_solve(JT * J, -(JT * mp.matrix(r)))
        th = [th[k] + step[k] for k in range(len(th))]
    return np.array([float(v) for v in th])


# Seeds for the free orbit coordinates (b: l in (0, 1/sqrt2); c: p in (0, 1/sqrt2)).
# Any seed in the right basin converges to the same rule; these are coarse
# starting guesses, the digits come from the solve.
_SEEDS = {
    38: [0.46],
    50: [0.30],
    74: [0.48, 0.32],
    86: [0.37, 0.69, 0.43],
    110: [0.19, 0.69, 0.40, 0.48],
}


@lru_cache(maxsize=None)
def lebedev(order: int):
    """Lebedev rule with ``order`` points: returns (xyz [n,3], w [n]), sum(w) = 1."""
    from scipy.optimize import least_squares

    if order not in LEBEDEV_ORBITS:
        raise ValueError(f"unsupported Lebedev order {order}; have {sorted(LEBEDEV_ORBITS)}")
    degree, orbits = LEBEDEV_ORBITS[order]
    moments = _moments(degree)
    nparam = sum(1 for o in orbits if o in ("b", "c"))
    seeds = _SEEDS.get(order, [])
    assert len(seeds) == nparam
    w0 = np.full(len(orbits), 1.0 / order)
    theta0 = np.concatenate([w0, np.array(seeds, dtype=np.float64)])
    lo = np.concatenate([np.full(len(orbits), -1.0), np.full(nparam, 1e-3)])
    hi = np.concatenate([np.full(len(orbits), 1.0), np.full(nparam, 0.7070)])
    sol = least_squares(_residual, theta0, args=(orbits, moments), bounds=(lo, hi),
                        xtol=1e-15, ftol=1e-15, gtol=1e-15, max_nfev=20000)
    theta = _polish_mp(sol.x, orbits, moments)
    r = _residual(theta, orbits, moments)
    if np.max(np.abs(r)) > 1e-15:
        raise RuntimeError(f"Lebedev {order}: moment residual {np.max(np.abs(r)):.3e}")
    nw = len(orbits)
    pts, wts = [], []
    pi = 0
    for o, code in enumerate(orbits):
        if code in ("b", "c"):
            p = _orbit_points(code, theta[nw + pi])
            pi += 1
        else:
            p = _orbit_points(code)
        pts.append(p)
        wts.append(np.full(len(p), theta[o]))
    xyz = np.concatenate(pts)
    w = np.concatenate(wts)
    assert xyz.shape[0] == order
    return xyz, w


def tensor_quadrature(n_radial: int, lebedev_order: int, r0: float, r1: float):
    """Tensor-product points as the reference lays them out
    (``CharmmReferenceGBSW.cpp:34-46``): index = ir*nS + is; returns
    offsets [Q,3], radii [Q], weights [Q] (= w_r * w_s)."""
    xr, wr = gauss_legendre(r0, r1, n_radial)
    u, ws = lebedev(lebedev_order)
    Q = n_radial * len(ws)
    off = np.empty((Q, 3))
    rad = np.empty(Q)
    wt = np.empty(Q)
    for i in range(n_radial):
        for j in range(len(ws)):
            idx = i * len(ws) + j
            off[idx] = xr[i] * u[j]
            rad[idx] = xr[i]
            wt[idx] = wr[i] * ws[j]
    return off, rad, wt


def emit_header(path: str) -> None:
    lines = [
        "// Generated by `python -m openmmcustomgbintegralforce_gb300.quadrature --emit-header`.",
        "// Lebedev-Laikov octahedral rules solved from the sphere moment equations",
        "// (see quadrature.py).  Weights sum to 1.  Do not edit by hand.",
        "#pragma once",
        "namespace gbx_lebedev {",
        "struct Rule { int order; const double* xyzw; };",
    ]
    for order in sorted(LEBEDEV_ORBITS):
        xyz, w = lebedev(order)
        lines.append(f"static const double kRule{order}[{order * 4}] = {{")
        for k in range(order):
            lines.append("  " + ", ".join(f"{v:.17e}" for v in (*xyz[k], w[k])) + ",")
        lines.append("};")
    lines.append("static const Rule kRules[] = {")
    for order in sorted(LEBEDEV_ORBITS):
        lines.append(f"  {{{order}, kRule{order}}},")
    lines.append("};")
    lines.append(f"static const int kNumRules = {len(LEBEDEV_ORBITS)};")
    lines.append("}  // namespace gbx_lebedev")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    if len(sys.argv) >= 2 and sys.argv[1] == "--emit-header":
        import os
        out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(os.path.dirname(__file__), "csrc", "lebedev_rules.h")
        emit_header(out)
        print("wrote", out)
