"""Generate tetrahedron_rules.h: symmetric Gauss rules for tetrahedra and their triangular faces.

The reference obtains its rules from gmsh ("Gauss{order}", src/Mesh/Quadrature.cpp:28-34) with the
orders of src/Solver/SimulationControl.cpp:268-283: volume 2P, face 2P+1.  For P = 1..3 the point
counts are
  tetrahedron volume, orders 2/4/6 : 4 / 11 / 24 points (kTetrahedronQuadratureNumber), the counts of
      P. Keast, "Moderate-degree tetrahedral quadrature formulas", CMAME 55 (1986);
  triangle face, orders 3/5/7      : 4 / 7 / 13 points (kTriangleQuadratureNumber), the counts of
      D.A. Dunavant, "High degree efficient symmetrical Gaussian quadrature rules for the triangle",
      IJNME 21 (1985).
For P = 4 the face rule is Dunavant's degree-9 rule (19 points, the reference's count); the volume rule of
order 8 is the Grundmann-Moeller rule s = 4 (70 points, exact to degree 9) in place of gmsh's 43-point rule,
whose values are not in the reference tree.
This script takes the published orbit structure and starting values, polishes them with Newton's method
on the moment equations so every monomial up to the rule's degree is integrated to round-off, and writes
the rules on the reference elements (0,0,0),(1,0,0),(0,1,0),(0,0,1) (weights summing to 1/6) and
(0,0),(1,0),(0,1) (weights summing to 1/2).

The face rules list their points in the orbit order that the reference's face-point permutations
(src/Solver/SimulationControl.cpp:405-434, the Triangle cases for P = 1..3) imply: the centroid, then each
3-point orbit as (a,a), (a,1-2a), (1-2a,a), then the 6-point orbit with barycentric values (x,y,z) as
(x,y), (y,z), (z,x), (x,z), (y,x), (z,y).  The point values themselves are unpinned against gmsh, which
is not vendored with the reference.

Run:  python gen_tetrahedron_rules.py > tetrahedron_rules.h
"""
import math

import numpy as np


def tri_exact(a, b):
    return math.factorial(a) * math.factorial(b) / math.factorial(a + b + 2)


def tet_exact(a, b, c):
    return math.factorial(a) * math.factorial(b) * math.factorial(c) / math.factorial(a + b + c + 3)


def tri_build(params, orbits, alt=False):
    """Points and weights of a symmetric triangle rule.  The orbits are listed in the order the reference's
    Triangle permutation tables imply: for P1..P4 (a,a), (a,1-2a), (1-2a,a) and (x,y), (y,z), (z,x), (x,z),
    (y,x), (z,y); for P5 (`alt`: its table swaps rotations 1 and 2 against that order) (a,a), (1-2a,a),
    (a,1-2a) and (x,y), (z,x), (y,z), (z,y), (y,x), (x,z)."""
    pts, w, k = [], [], 0
    for o in orbits:
        if o == "c":
            pts.append((1 / 3, 1 / 3)); w.append(params[k]); k += 1
        elif o == "s21":
            a, wt = params[k], params[k + 1]; k += 2
            orbit = [(a, a), (a, 1 - 2 * a), (1 - 2 * a, a)]
            for p in ([orbit[i] for i in (0, 2, 1)] if alt else orbit):
                pts.append(p); w.append(wt)
        else:
            x, y, wt = params[k], params[k + 1], params[k + 2]; k += 3
            z = 1 - x - y
            orbit = [(x, y), (y, z), (z, x), (x, z), (y, x), (z, y)]
            for p in ([orbit[i] for i in (0, 2, 1, 5, 4, 3)] if alt else orbit):
                pts.append(p); w.append(wt)
    return np.array(pts), np.array(w)


def tet_build(params, orbits):
    bary, w, k = [], [], 0
    for o in orbits:
        if o == "c":
            bary.append((0.25, 0.25, 0.25, 0.25)); w.append(params[k]); k += 1
        elif o == "s31":
            a, wt = params[k], params[k + 1]; k += 2
            b = 1 - 3 * a
            for i in range(4):
                l = [a] * 4; l[i] = b
                bary.append(tuple(l)); w.append(wt)
        elif o == "s22":
            a, wt = params[k], params[k + 1]; k += 2
            b = 0.5 - a
            for i in range(4):
                for j in range(i + 1, 4):
                    l = [b] * 4; l[i] = a; l[j] = a
                    bary.append(tuple(l)); w.append(wt)
        else:  # s211: (a, a, b, c)
            a, b, wt = params[k], params[k + 1], params[k + 2]; k += 3
            c = 1 - 2 * a - b
            for i in range(4):
                for j in range(i + 1, 4):
                    rest = [m for m in range(4) if m not in (i, j)]
                    for r0, r1 in ((rest[0], rest[1]), (rest[1], rest[0])):
                        l = [0.0] * 4; l[i] = a; l[j] = a; l[r0] = b; l[r1] = c
                        bary.append(tuple(l)); w.append(wt)
    bary = np.array(bary)
    return bary[:, 1:], np.array(w)


def tri_resid(params, orbits, deg):
    p, w = tri_build(params, orbits)
    return np.array([(w * p[:, 0] ** a * p[:, 1] ** b).sum() - tri_exact(a, b)
                     for a in range(deg + 1) for b in range(deg + 1 - a)])


def tet_resid(params, orbits, deg):
    p, w = tet_build(params, orbits)
    return np.array([(w * p[:, 0] ** a * p[:, 1] ** b * p[:, 2] ** c).sum() - tet_exact(a, b, c)
                     for a in range(deg + 1) for b in range(deg + 1 - a) for c in range(deg + 1 - a - b)])


# Dunavant's odd-degree rules: orbit structure and published values (weights normalised to area 1).
FACE_RULES = {
    3: (["c", "s21"], [-27 / 48, 0.2, 25 / 48]),
    5: (["c", "s21", "s21"], [0.225000000000000, 0.470142064105115, 0.132394152788506,
                              0.101286507323456, 0.125939180544827]),
    7: (["c", "s21", "s21", "s111"], [-0.149570044467682, 0.260345966079040, 0.175615257433208,
                                      0.065130102902216, 0.053347235608838,
                                      0.048690315425316, 0.312865496004874, 0.077113760890257]),
    9: (["c", "s21", "s21", "s21", "s21", "s111"], [0.097135796282799,
                                                     0.489682519198738, 0.031334700227139,
                                                     0.437089591492937, 0.077827541004774,
                                                     0.188203535619033, 0.079647738927210,
                                                     0.044729513394453, 0.025577675658698,
                                                     0.036838412054736, 0.221962989160766, 0.043283539377289]),
    # degree 11: 27 points, one orbit outside the triangle (Dunavant's rule as published)
    11: (["s21"] * 5 + ["s111"] * 2, [0.534611048270758, 0.000927006328961,
                                       0.398969302965855, 0.077149534914813,
                                       0.203309900431282, 0.059322977380774,
                                       0.119350912282581, 0.036184540503418,
                                       0.032364948111276, 0.013659731002678,
                                       0.050178138310495, 0.356620648261293, 0.052337111962204,
                                       0.021022016536166, 0.171488980304042, 0.020707659639141]),
}
# Keast's rules of degree 2, 4 and 6: orbit structure and published values (weights for volume 1/6).
VOLUME_RULES = {
    2: (["s31"], [(5 - math.sqrt(5)) / 20, 1 / 24]),
    4: (["c", "s31", "s22"], [-0.013155555555556, 0.071428571428571, 0.007622222222222,
                              0.399403576166799, 0.024888888888889]),
    6: (["s31", "s31", "s31", "s211"], [0.214602871259152, 0.006653791709695,
                                        0.040673958534611, 0.001679535175887,
                                        0.322337890142276, 0.009226196923942,
                                        0.063661001875018, 0.269672331458316, 0.008035714285714]),
}


def compositions(total, parts):
    """All tuples of `parts` non-negative integers summing to `total`, in lexicographic order."""
    if parts == 1:
        yield (total,)
        return
    for first in range(total, -1, -1):
        for rest in compositions(total - first, parts - 1):
            yield (first,) + rest


def grundmann_moeller(s, n=3):
    """The Grundmann-Moeller rule of degree 2s+1 on the n-simplex of volume 1/n! (A. Grundmann, H.M. Moeller,
    "Invariant integration formulas for the n-simplex by combinatorial methods", SIAM J. Numer. Anal. 15 (1978)):
    Q[f] = sum_{i=0..s} (-1)^i 2^{-2s} (d+n-2i)^d / (i! (d+n-i)!) sum_{|b| = s-i} f((2 b_j + 1)/(d+n-2i)),
    d = 2s+1, the points in barycentric coordinates; coinciding points of different levels are merged."""
    d = 2 * s + 1
    pts, ws = [], []
    for i in range(s + 1):
        den = d + n - 2 * i
        wt = (-1) ** i * 2.0 ** (-2 * s) * den ** d / (math.factorial(i) * math.factorial(d + n - i))
        for beta in compositions(s - i, n + 1):
            x = tuple((2 * b + 1) / den for b in beta[1:])
            for k, q in enumerate(pts):
                if max(abs(a - c) for a, c in zip(q, x)) < 1e-15:
                    ws[k] += wt
                    break
            else:
                pts.append(x)
                ws.append(wt)
    return np.array(pts), np.array(ws)


def polish(resid, orbits, x0, deg):
    x = np.array(x0, dtype=float)
    for _ in range(10):
        r = resid(x, orbits, deg)
        jac = np.zeros((len(r), len(x)))
        for i in range(len(x)):
            h = 1e-7
            xp = x.copy(); xp[i] += h
            xm = x.copy(); xm[i] -= h
            jac[:, i] = (resid(xp, orbits, deg) - resid(xm, orbits, deg)) / (2 * h)
        step = np.linalg.lstsq(jac, -r, rcond=None)[0]
        # a step that does not reduce the residual ends the iteration (closed-form values stay as they are)
        if np.linalg.norm(resid(x + step, orbits, deg)) >= np.linalg.norm(r):
            break
        x = x + step
    return x


def weight_positions(orbits):
    k, out = 0, []
    for o in orbits:
        step = {"c": 1, "s21": 2, "s111": 3, "s31": 2, "s22": 2, "s211": 3}[o]
        out.append(k + step - 1)
        k += step
    return out


def main():
    fmt = lambda v: ", ".join("%.17g" % t for t in v)
    print("// Generated by gen_tetrahedron_rules.py -- do not edit.")
    print("// Tetrahedron volume rules (Keast 1986 orbit structure) and triangle face rules (Dunavant 1985,")
    print("// odd degrees, in the reference's face-point orbit order), Newton-polished.")
    print("// Reference tetrahedron (0,0,0),(1,0,0),(0,1,0),(0,0,1): weights sum to 1/6.")
    print("// Reference triangle (0,0),(1,0),(0,1): weights sum to 1/2.")
    print("#pragma once")
    print("namespace sdg_tables {")
    print("struct FaceTriangleRule { int degree; int count; const double* xi; const double* eta; const double* weight; };")
    print("struct TetrahedronRule { int degree; int count; const double* xi; const double* eta; const double* zeta;")
    print("                         const double* weight; };")
    faces = []
    for deg, (orb, p0) in FACE_RULES.items():
        x0 = np.array(p0)
        for k in weight_positions(orb):
            x0[k] *= 0.5
        x = polish(tri_resid, orb, x0, deg)
        err = np.abs(tri_resid(x, orb, deg)).max()
        assert err < 1e-15, (deg, err)
        # the published 15 digits move by up to 4e-11 on the degree-11 rule (an orbit outside the triangle
        # makes its moment system ill-conditioned)
        assert np.abs(x - x0).max() < (1e-10 if deg == 11 else 1e-11), (deg, np.abs(x - x0).max())
        p, w = tri_build(x, orb, alt=deg == 11)
        n = len(w)
        print(f"// face degree {deg}: {n} points, max moment error {err:.1e}")
        print(f"inline constexpr double kFaceTri{deg}Xi[{n}] = {{{fmt(p[:, 0])}}};")
        print(f"inline constexpr double kFaceTri{deg}Eta[{n}] = {{{fmt(p[:, 1])}}};")
        print(f"inline constexpr double kFaceTri{deg}W[{n}] = {{{fmt(w)}}};")
        faces.append((deg, n))
    vols = []
    for deg, (orb, p0) in VOLUME_RULES.items():
        x = polish(tet_resid, orb, p0, deg)
        err = np.abs(tet_resid(x, orb, deg)).max()
        assert err < 1e-15, (deg, err)
        assert np.abs(x - np.array(p0)).max() < 1e-11, (deg, np.abs(x - np.array(p0)).max())
        p, w = tet_build(x, orb)
        n = len(w)
        print(f"// volume degree {deg}: {n} points, max moment error {err:.1e}")
        print(f"inline constexpr double kTet{deg}Xi[{n}] = {{{fmt(p[:, 0])}}};")
        print(f"inline constexpr double kTet{deg}Eta[{n}] = {{{fmt(p[:, 1])}}};")
        print(f"inline constexpr double kTet{deg}Zeta[{n}] = {{{fmt(p[:, 2])}}};")
        print(f"inline constexpr double kTet{deg}W[{n}] = {{{fmt(w)}}};")
        vols.append((deg, n))
    # orders 8 and 10 (P4, P5): Grundmann-Moeller s = 4 (degree 9) and s = 5 (degree 11; 126 points, the
    # reference's count, 125 once the doubled centroid is merged); the reference's order-8 gmsh rule has 43
    # points and is not restated here (gmsh is not vendored)
    for order, gm in ((8, 4), (10, 5)):
        p, w = grundmann_moeller(gm)
        top = 2 * gm + 1
        # the alternating-sign weights of the closed form lose ~1e-16 to cancellation: refine them on the
        # rounded points by least squares on the exact moments, residuals summed exactly (math.fsum)
        mom = [(a, b, c) for a in range(top + 1) for b in range(top + 1 - a) for c in range(top + 1 - a - b)]
        V = np.array([p[:, 0] ** a * p[:, 1] ** b * p[:, 2] ** c for a, b, c in mom])
        for _ in range(3):
            r = np.array([tet_exact(a, b, c) - math.fsum(V[k] * w) for k, (a, b, c) in enumerate(mom)])
            w = w + np.linalg.lstsq(V, r, rcond=None)[0]
        err = max(abs((w * p[:, 0] ** a * p[:, 1] ** b * p[:, 2] ** c).sum() - tet_exact(a, b, c))
                  for a, b, c in mom)
        assert err < 1e-15, err
        n = len(w)
        print(f"// volume order {order}: Grundmann-Moeller s = {gm} (exact to degree {top}), {n} points, "
              f"max moment error {err:.1e}")
        print(f"inline constexpr double kTet{order}Xi[{n}] = {{{fmt(p[:, 0])}}};")
        print(f"inline constexpr double kTet{order}Eta[{n}] = {{{fmt(p[:, 1])}}};")
        print(f"inline constexpr double kTet{order}Zeta[{n}] = {{{fmt(p[:, 2])}}};")
        print(f"inline constexpr double kTet{order}W[{n}] = {{{fmt(w)}}};")
        vols.append((order, n))
    print("inline constexpr FaceTriangleRule kFaceTriangleRules[] = {")
    for deg, n in faces:
        print(f"    {{{deg}, {n}, kFaceTri{deg}Xi, kFaceTri{deg}Eta, kFaceTri{deg}W}},")
    print("};")
    print("inline constexpr TetrahedronRule kTetrahedronRules[] = {")
    for deg, n in vols:
        print(f"    {{{deg}, {n}, kTet{deg}Xi, kTet{deg}Eta, kTet{deg}Zeta, kTet{deg}W}},")
    print("};")
    print("}  // namespace sdg_tables")


if __name__ == "__main__":
    main()
