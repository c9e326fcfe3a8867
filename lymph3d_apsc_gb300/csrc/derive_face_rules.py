"""Derives the fully symmetric triangle rules of mf.cu (kFaceRule).

For each degree p = 1..4 the rule must integrate every polynomial of total
degree <= 2p exactly on the reference triangle (0,0), (1,0), (0,1):
    sum_q w_q xi_q^i eta_q^j = i! j! / (i + j + 2)!   for i + j <= 2p.
The nodes come in orbits of the triangle's symmetry group, one weight per
orbit: the centroid (S3), (a, a, 1 - 2a) in barycentric coordinates (S21, 3
nodes) and (a, b, 1 - a - b) (S111, 6 nodes).  The orbit structures used
(S21 for degree 2; 2 x S21 for 4; 2 x S21 + S111 for 6; S3 + 3 x S21 + S111
for 8) are the classical ones with 3, 6, 12 and 16 nodes.  The script finds a
solution with interior nodes and positive weights by least squares from
seeded random starts (double precision), refines it by Gauss-Newton at 40
digits (mpmath) and prints the table.  The degree-6 structure admits more
than one such rule; the seeded search finds the one in mf.cu, and any of them
would give the same integrals.  Run: python derive_face_rules.py
"""
from math import factorial

import mpmath as mp
import numpy as np
from scipy.optimize import least_squares

STRUCT = {1: ["S21"], 2: ["S21", "S21"], 3: ["S21", "S21", "S111"], 4: ["S3", "S21", "S21", "S21", "S111"]}
NPAR = {"S3": 0, "S21": 1, "S111": 2}


def orbit(kind, par, one):
    if kind == "S3":
        return [(one / 3, one / 3)]
    if kind == "S21":
        a = par[0]
        return [(a, a), (a, one - 2 * a), (one - 2 * a, a)]
    a, b = par
    c = one - a - b
    return [(a, b), (b, a), (a, c), (c, a), (b, c), (c, b)]


def nodes(struct, x, one=1.0):
    pts, ws, k = [], [], 0
    for kind in struct:
        par = x[k:k + NPAR[kind]]
        k += NPAR[kind]
        o = orbit(kind, par, one)
        pts += o
        ws += [x[k]] * len(o)
        k += 1
    return pts, ws


def residual(struct, deg, x, one=1.0, fact=factorial):
    pts, ws = nodes(struct, x, one)
    return [sum(w * p[0] ** i * p[1] ** j for p, w in zip(pts, ws)) - one * fact(i) * fact(j) / fact(i + j + 2)
            for i in range(deg + 1) for j in range(deg + 1 - i)]


def first_guess(struct, deg, seed=0):
    rng = np.random.default_rng(seed)
    while True:
        x0 = []
        for kind in struct:
            x0 += list(rng.uniform(0.01, 0.49, NPAR[kind])) + [rng.uniform(0.01, 0.2)]
        r = least_squares(lambda x: residual(struct, deg, x), np.array(x0), xtol=1e-15, ftol=1e-15, gtol=1e-15)
        pts, ws = nodes(struct, r.x)
        inside = all(min(a, b, 1 - a - b) > 1e-6 for a, b in pts)
        if inside and min(ws) > 0 and np.abs(residual(struct, deg, r.x)).max() < 1e-14:
            return r.x


def refine(struct, deg, x, iters=30):
    mp.mp.dps = 40
    one = mp.mpf(1)
    x = [mp.mpf(float(v)) for v in x]
    h = mp.mpf(10) ** -25
    for _ in range(iters):
        r = residual(struct, deg, x, one, mp.factorial)
        J = mp.matrix(len(r), len(x))
        for c in range(len(x)):
            xp = list(x)
            xp[c] += h
            rp = residual(struct, deg, xp, one, mp.factorial)
            for q in range(len(r)):
                J[q, c] = (rp[q] - r[q]) / h
        dx = mp.lu_solve(J.T * J, -(J.T * mp.matrix(r)))
        x = [x[c] + dx[c] for c in range(len(x))]
    return x, max(abs(v) for v in residual(struct, deg, x, one, mp.factorial))


if __name__ == "__main__":
    for p, struct in STRUCT.items():
        deg = 2 * p
        x, res = refine(struct, deg, first_guess(struct, deg))
        pts, ws = nodes(struct, x, mp.mpf(1))
        print(f"    // p = {p}, exact to degree {deg} ({len(ws)} nodes; largest moment residual {float(res):.1e})")
        for (a, b), w in zip(pts, ws):
            print(f"    {mp.nstr(a, 20)}, {mp.nstr(b, 20)}, {mp.nstr(w, 20)},")
