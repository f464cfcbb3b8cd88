"""Generate the golden fixtures of the test suite.

Part 1 -- known answers read as text from the reference source tree, whose root is passed
with --reference:
  * face quadrature permutations by rotation   src/Solver/SimulationControl.cpp:381-523
  * quadrature point counts by order           src/Solver/SimulationControl.cpp:268-273
  * face vertex lists                          src/Solver/SimulationControl.cpp:170-216
  * point-face normals of lines                src/Mesh/Geometry.cpp:102-112
  * SSP-RK / Heun / Euler coefficient tables   src/Solver/TimeIntegration.cpp:45-65
  * gamma, Prandtl, Sutherland constants       src/Solver/PhysicalModel.cpp:45,91,109
Part 2 -- oracle reference vectors on small seeded meshes (the oracle is the CPU restatement
of the reference algorithm; these pin it across machines and edits).

    python tests/golden/make_golden.py --reference <root of the SubrosaDG source tree>
"""
from __future__ import annotations

import argparse
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def _func_body(text, name):
    i = text.index(name)
    j = text.index("{", i)
    depth = 0
    for k in range(j, len(text)):
        if text[k] == "{":
            depth += 1
        elif text[k] == "}":
            depth -= 1
            if depth == 0:
                return text[j:k + 1]
    raise ValueError(name)


def reference_tables(ref):
    sc = open(os.path.join(ref, "src/Solver/SimulationControl.cpp")).read()
    out = {}
    body = _func_body(sc, "getAdjacencyElementQuadratureSequence([[maybe_unused]] int rotation)")
    perms = {}
    for elem in ("Line", "Triangle", "Quadrangle"):
        m = re.search(r"ElementType == ElementEnum::%s\) \{(.*?)\n  \}\n" % elem, body, re.S)
        seg = m.group(1)
        for pm in re.finditer(r"PolynomialOrder == (\d)\) \{(.*?)\n    \}", seg, re.S):
            p = int(pm.group(1))
            blk = pm.group(2)
            if "switch" in blk:
                rots = {}
                for cm in re.finditer(r"case (\d):\s*return \{([^}]*)\};", blk):
                    rots[int(cm.group(1))] = [int(x) for x in cm.group(2).replace("\n", " ").split(",")]
                perms[f"{elem}/P{p}"] = rots
            else:
                vals = re.search(r"return \{([^}]*)\};", blk).group(1)
                perms[f"{elem}/P{p}"] = {0: [int(x) for x in vals.split(",")]}
    out["face_permutation"] = perms
    counts = {}
    for name in ("Line", "Triangle", "Quadrangle", "Tetrahedron", "Pyramid", "Hexahedron"):
        m = re.search(r"k%sQuadratureNumber\{([^}]*)\}" % name, sc)
        counts[name] = [int(x) for x in m.group(1).split(",")]
    out["quadrature_count"] = counts
    body = _func_body(sc, "getElementPerAdjacencyNodeIndex()")
    faces = {}
    for name in ("Line", "Triangle", "Quadrangle", "Tetrahedron", "Hexahedron"):
        m = re.search(r"ElementType == ElementEnum::%s\) \{\s*return \{([^}]*)\};" % name, body, re.S)
        faces[name] = [int(x) for x in m.group(1).replace("\n", " ").split(",")]
    out["face_vertices"] = faces
    # outward normals of a line's point faces by their sequence in the parent (Geometry.cpp:102-112)
    geo = open(os.path.join(ref, "src/Mesh/Geometry.cpp")).read()
    body = _func_body(geo, "calculateNormalVector(const Isize adjacency_sequence_in_parent")
    out["point_normals"] = {int(m.group(1)): float(m.group(2)) for m in re.finditer(
        r"adjacency_sequence_in_parent == (\d)\) \{\s*normal_vector\(0, 0\) = ([-0-9.]+)_r;", body)}
    ti = open(os.path.join(ref, "src/Solver/TimeIntegration.cpp")).read()
    rk = {}
    for name in ("ForwardEuler", "HeunRK2", "SSPRK3"):
        m = re.search(r"TimeIntegrationEnum::%s> : TimeIntegrationBase \{.*?kStepCoefficients\{(.*?)\};" % name, ti, re.S)
        txt = m.group(1).replace("_r", "")
        rows = re.findall(r"\{([^{}]*)\}", txt)
        rk[name] = [[eval(x) for x in r.split(",")] for r in rows]
    out["rk_coefficients"] = rk
    pm = open(os.path.join(ref, "src/Solver/PhysicalModel.cpp")).read()
    out["specific_heat_ratio"] = float(re.search(r"kSpecificHeatRatio = ([0-9.]+)_r", pm).group(1))
    out["prandtl_number"] = float(re.search(r"kPrandtlNumber = ([0-9.]+)_r", pm).group(1))
    st = re.search(r"kSutherlandTemperature = ([0-9.]+)_r / ([0-9.]+)_r", pm)
    out["sutherland_temperature"] = float(st.group(1)) / float(st.group(2))
    cf = open(os.path.join(ref, "src/Solver/ConvectiveFlux.cpp")).read()
    out["harten_divisor"] = float(re.search(r"harten_delta = roe_sound_speed / ([0-9.]+)_r", cf).group(1))
    # weakly compressible pressure addition factor (p = c0^2 (rho - rho0) + f rho0 c0^2) and Boussinesq gravity
    out["weak_pressure_addition"] = float(
        re.search(r"reference_pressure_addition =\s*([0-9.]+) \* this->reference_density", pm).group(1))
    stf = open(os.path.join(ref, "src/Solver/SourceTerm.cpp")).read()
    out["boussinesq_gravity"] = float(re.search(r"kGravity = ([0-9.]+)_r", stf).group(1))
    # artificial-viscosity sensor thresholds s0(P) (the uncommented table)
    m = re.search(r"^inline constexpr std::array<Real, 5> kArtificialViscosityTolerance\{([^}]*)\}", sc, re.M)
    out["artificial_viscosity_tolerance"] = [float(x) for x in m.group(1).replace("\n", " ").split(",")]
    return out


def oracle_vectors():
    sys.path.insert(0, ROOT)
    import subrosadg_gb300 as sdg  # mesh generators only (host code)
    from oracle.orc import Oracle
    from tests import cases

    vectors = {}
    for name, case in cases.golden_cases().items():
        mesh, cfg, prim, bprim, dt, steps = case()
        o = Oracle(mesh, cfg, faithful=False)
        o.initialize_primitive(prim(o.volume_points()))
        if o.boundary:
            bpts, phys = o.boundary_points()
            o.set_boundary_primitive(bprim(bpts, np.repeat(phys, o.nfq)))
        r0 = o.residual_point()
        o.step(dt, steps)
        vectors[name] = {
            "steps": steps, "dt": dt,
            "residual_checksum": float(np.abs(r0).sum()),
            "residual_sample": r0[:: max(1, len(r0) // 16)].tolist(),
            "state_sample": o.state_point()[:: max(1, o.volume_points_count // 16)].tolist(),
            "relative_error": o.relative_error().tolist(),
            "delta_time_cfl_0.2": o.delta_time(0.2),
        }
    return vectors


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of the SubrosaDG source tree (read only)")
    args = ap.parse_args()
    tables = reference_tables(args.reference)
    with open(os.path.join(HERE, "reference_tables.json"), "w") as f:
        json.dump(tables, f, indent=1)
    with open(os.path.join(HERE, "oracle_vectors.json"), "w") as f:
        json.dump(oracle_vectors(), f, indent=1)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
