"""Known-answer vectors from the reference's shape unit tests (tests/golden/unit_*.json,
made by tests/golden/extract_unit_vectors.py): loading, shape construction through either
geometry API (the oracle's or the product's, which share method names), and the tests'
own comparison rules."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FILES = ["Box", "Tube", "Cons", "Polycone", "Torus2", "Trd", "Polyhedra", "Trap", "Sphere", "GenTrap", "Hype"]
QUERY_ID = {"Inside": 0, "Contains": 1, "DistanceToIn": 2, "DistanceToOut": 3, "SafetyToIn": 4, "SafetyToOut": 5}
APPROX_TOL = 1e-6   # kApproxEqualTolerance of test/unit_tests/ApproxEqual.h
RANGE_DELTA = 1e-4  # DELTA of OutRange in test/unit_tests/TestCons.cpp


# Soft checks the reference itself does not meet, found by reading its code path:
# (file, line) -> reason.
SOFT_EXCEPTIONS = {
    ("Cons", 591): "point 2.5e-7 mm outside -dz: ConeImplementation::DistanceToOut returns -1 when "
                   "|z| - dz > kConeTolerance (1e-7), VecGeom/volumes/kernel/ConeImplementation.h:274-284",
}


# Hard asserts that the reference's scalar CPU path meets and its generic kernels (the ones
# its CUDA build runs, which the oracle and the product restate) miss by FP64 rounding only:
# (file, line) -> reason. Such a check must still hold within ROUNDING_SLACK relative.
ROUNDING_EXCEPTIONS = {
    ("GenTrap", line): "SafetyToIn 0.15 along the outward normal of a planar face: the generic "
                       "SecondOrderSurfaceShell::SafetyToIn returns (p - a).n = 0.15 + 3 ulp, the "
                       "asserted bound is exact; the unit test runs the scalar CPU path, which routes "
                       "planar GenTraps through TessellatedSection (GenTrapImplementation.h "
                       "SafetyToIn specialisation), a helper the CUDA build does not have"
    for line in (146, 155, 165, 174)
}
ROUNDING_SLACK = 1e-15


def excepted(name, case):
    return case.get("soft", False) and (name, case["line"]) in SOFT_EXCEPTIONS


def case_passes(name, case, actual):
    """The case's own comparison, with the documented exceptions above."""
    if passes(case["kind"], actual, case["expected"], case.get("tol")):
        return True
    if excepted(name, case):
        return True
    if (name, case["line"]) in ROUNDING_EXCEPTIONS:
        e = float(case["expected"])
        return passes(case["kind"], actual, e + ROUNDING_SLACK * abs(e), case.get("tol"))
    return False


def load(name):
    with open(os.path.join(GOLDEN, "unit_%s.json" % name)) as f:
        doc = json.load(f)
    resolve_along_normal(doc)
    return doc


def resolve_along_normal(doc):
    """Points the test builds along the shape's own surface normal (p + t * normal after
    shape.Normal(p, normal), recorded by the extractor as "along_normal") are resolved with
    the oracle's Normal of the same shape, as Vector3D arithmetic does: base + (t * n)."""
    todo = [c for c in doc["cases"] if c.get("along_normal")]
    if not todo:
        return
    from oracle.oracle import OracleGeometry
    normals = {}
    for c in todo:
        a = c["along_normal"]
        key = (a["shape"], tuple(a["at"]))
        if key not in normals:
            o = OracleGeometry()
            s = add_shape(o, doc["shapes"][a["shape"]])
            normals[key] = o.shape_normal(s, a["at"])[0]
        n = normals[key]
        c["p"] = [float(b + a["scale"] * k) for b, k in zip(a["base"], n)]


def add_shape(geo, spec):
    t, a = spec["type"], spec["args"]
    if t == "box":
        return geo.add_box(*a[:3])
    if t == "tube":
        return geo.add_tube(*a[:5])
    if t == "cone":
        return geo.add_cone(*a[:7])
    if t == "torus2":
        return geo.add_torus2(*a[:5])
    if t == "sphere":
        return geo.add_sphere(*a[:6])
    if t == "gentrap":
        return geo.add_gentrap(a[0], a[1], a[2])
    if t == "hype":
        return geo.add_hype(*a[:5])
    if t == "trd":
        if len(a) == 4:  # Trd1 constructor (x1, x2, y, z)
            return geo.add_trd(a[0], a[1], a[2], a[2], a[3])
        return geo.add_trd(*a[:5])
    if t == "trap":
        if len(a) == 1:  # eight corners
            return geo.add_trap_corners(a[0])
        if len(a) == 4:  # Trd1-like (dx1, dx2, dy, dz)
            return geo.add_trap(a[3], 0.0, 0.0, a[2], a[0], a[0], 0.0, a[2], a[1], a[1], 0.0)
        if len(a) == 5:  # Trd2-like (dx1, dx2, dy1, dy2, dz)
            return geo.add_trap(a[4], 0.0, 0.0, a[2], a[0], a[0], 0.0, a[3], a[1], a[1], 0.0)
        return geo.add_trap(*a[:11])
    if t == "polyhedron":
        sphi, dphi, nsides, nz, z, rmin, rmax = a[:7]
        nz = int(nz)
        return geo.add_polyhedron(sphi, dphi, int(nsides), list(z)[:nz], list(rmin)[:nz], list(rmax)[:nz])
    if t == "polycone":
        sphi, dphi, nz, z, rmin, rmax = a[:6]
        nz = int(nz)
        return geo.add_polycone(sphi, dphi, list(z)[:nz], list(rmin)[:nz], list(rmax)[:nz])
    raise ValueError(t)


def build(geo, spec):
    """The shape placed alone with the identity transformation; returns its placed id."""
    pv = geo.place(geo.add_logical_volume(add_shape(geo, spec)))
    geo.close()
    return pv


def approx_equal(x, y):
    """ApproxEqual<double> of test/unit_tests/ApproxEqual.h."""
    if x == y:
        return True
    if x * y == 0.0:
        return abs(x - y) < APPROX_TOL
    if abs(x) > 1e100 or abs(y) > 1e100:
        return x * y > 0 and abs(x) > 1e100 and abs(y) > 1e100
    return abs(x - y) / (abs(x) + abs(y)) < APPROX_TOL


def passes(kind, actual, expected, tol=None):
    a, e = float(actual), float(expected)
    if kind == "any":  # one side of a comparison between two query results (doc["pairs"])
        return True
    if kind == "absdiff":  # std::fabs(actual - expected) < tol
        return abs(a - e) < tol
    if kind == "approx":
        return approx_equal(a, e)
    if kind == "range":
        return not (a < e - RANGE_DELTA or a > e + RANGE_DELTA)
    return {"==": a == e, "!=": a != e, "<": a < e, "<=": a <= e, ">": a > e, ">=": a >= e}[kind]


def approx_equal_vec(v, w):
    """ApproxEqual of two 3-vectors (component-wise, test/unit_tests/ApproxEqual.h:21-28)."""
    return all(approx_equal(float(a), float(b)) for a, b in zip(v, w))


def extent_cases(doc):
    """The Extent(lo, hi) known answers: (shape name, "ExtentMin" / "ExtentMax", expected)."""
    return [(c["shape"], c["query"], c["expected"]) for c in doc["cases"] if c["query"].startswith("Extent")]


def grouped(doc):
    """Cases grouped by (shape, query): arrays of points/directions and the case list
    (the point queries only; Extent cases are in extent_cases)."""
    groups = {}
    for c in doc["cases"]:
        if c["query"] not in QUERY_ID:
            continue
        groups.setdefault((c["shape"], c["query"]), []).append(c)
    for (shape, q), cs in groups.items():
        p = np.array([c["p"] for c in cs], dtype=np.float64)
        d = np.array([c["d"] if c["d"] else [0.0, 0.0, 1.0] for c in cs], dtype=np.float64)
        yield shape, q, cs, p, d
