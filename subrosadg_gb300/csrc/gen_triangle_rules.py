"""Generate triangle_rules.h: symmetric Gauss rules on the reference triangle.

The reference obtains its triangle rules from gmsh ("Gauss{order}", called at
src/Mesh/Quadrature.cpp:28-34); gmsh's point counts for orders 2,4,6,8,10 are
3,6,12,16,25 (src/Solver/SimulationControl.cpp:269), which are the point counts
of D.A. Dunavant, "High degree efficient symmetrical Gaussian quadrature rules
for the triangle", IJNME 21 (1985).  This script takes Dunavant's published
orbit structure and starting values (15 digits), polishes them with Newton's
method on the moment equations so every monomial up to the rule's degree is
integrated to round-off, and writes the rules with weights summing to 1/2 (the
area of the reference triangle (0,0),(1,0),(0,1)).

Run:  python gen_triangle_rules.py > triangle_rules.h
"""
import math
import numpy as np


def exact(a, b):
    return math.factorial(a) * math.factorial(b) / math.factorial(a + b + 2)


def build(params, orbits):
    pts, w, k = [], [], 0
    for o in orbits:
        if o == "c":
            pts.append((1 / 3, 1 / 3)); w.append(params[k]); k += 1
        elif o == "s21":
            a, wt = params[k], params[k + 1]; k += 2
            for p in [(a, a), (1 - 2 * a, a), (a, 1 - 2 * a)]:
                pts.append(p); w.append(wt)
        else:
            a, b, wt = params[k], params[k + 1], params[k + 2]; k += 3
            c = 1 - a - b
            for p in [(a, b), (b, a), (a, c), (c, a), (b, c), (c, b)]:
                pts.append(p); w.append(wt)
    return np.array(pts), np.array(w)


def resid(params, orbits, deg):
    p, w = build(params, orbits)
    return np.array([(w * p[:, 0] ** a * p[:, 1] ** b).sum() - exact(a, b)
                     for a in range(deg + 1) for b in range(deg + 1 - a)])


# Dunavant's orbit structure and published values (weights normalised to area 1).
RULES = {
    2: (["s21"], [1 / 6, 1 / 3]),
    4: (["s21", "s21"], [0.445948490915965, 0.223381589678011, 0.091576213509771, 0.109951743655322]),
    6: (["s21", "s21", "s111"], [0.249286745170910, 0.116786275726379, 0.063089014491502, 0.050844906370207,
                                  0.310352451033785, 0.053145049844816, 0.082851075618374]),
    8: (["c", "s21", "s21", "s21", "s111"], [0.144315607677787, 0.459292588292723, 0.095091634267285,
                                            0.170569307751760, 0.103217370534718, 0.050547228317031,
                                            0.032458497623198, 0.263112829634638, 0.008394777409958,
                                            0.027230314174435]),
    10: (["c", "s21", "s21", "s111", "s111", "s111"], [0.090817990382754, 0.485577633383657, 0.036725957756467,
                                                       0.109481575485037, 0.045321059435528, 0.141707219414880,
                                                       0.307939838764121, 0.072757916845420, 0.025003534762686,
                                                       0.246672560639903, 0.028327242531057, 0.009540815400299,
                                                       0.066803251012200, 0.009421666963733]),
}


def polish(orbits, p0, deg):
    x = np.array(p0, dtype=float)
    # weights -> area-1/2 normalisation
    k = 0
    for o in orbits:
        step = {"c": 1, "s21": 2, "s111": 3}[o]
        x[k + step - 1] *= 0.5
        k += step
    for _ in range(8):
        r = resid(x, orbits, deg)
        jac = np.zeros((len(r), len(x)))
        for i in range(len(x)):
            h = 1e-7
            xp = x.copy(); xp[i] += h
            xm = x.copy(); xm[i] -= h
            jac[:, i] = (resid(xp, orbits, deg) - resid(xm, orbits, deg)) / (2 * h)
        x = x + np.linalg.lstsq(jac, -r, rcond=None)[0]
    return x


def main():
    print("// Generated by gen_triangle_rules.py -- do not edit.")
    print("// Symmetric triangle rules (Dunavant 1985 orbit structure, Newton-polished).")
    print("// Reference triangle (0,0),(1,0),(0,1); weights sum to 1/2.")
    print("#pragma once")
    print("namespace sdg_tables {")
    print("struct TriangleRule { int degree; int count; const double* xi; const double* eta; const double* weight; };")
    names = []
    for deg, (orb, p0) in RULES.items():
        x = polish(orb, p0, deg)
        err = np.abs(resid(x, orb, deg)).max()
        assert err < 1e-15, (deg, err)
        p, w = build(x, orb)
        n = len(w)
        fmt = lambda v: ", ".join("%.17g" % t for t in v)
        print(f"// degree {deg}: {n} points, max moment error {err:.1e}")
        print(f"inline constexpr double kTri{deg}Xi[{n}] = {{{fmt(p[:, 0])}}};")
        print(f"inline constexpr double kTri{deg}Eta[{n}] = {{{fmt(p[:, 1])}}};")
        print(f"inline constexpr double kTri{deg}W[{n}] = {{{fmt(w)}}};")
        names.append((deg, n))
    print("inline constexpr TriangleRule kTriangleRules[] = {")
    for deg, n in names:
        print(f"    {{{deg}, {n}, kTri{deg}Xi, kTri{deg}Eta, kTri{deg}W}},")
    print("};")
    print("}  // namespace sdg_tables")


if __name__ == "__main__":
    main()
