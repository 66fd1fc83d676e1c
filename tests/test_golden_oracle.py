"""The oracle against the known answers of the reference's own shape unit tests
(test/unit_tests/Test{Box,Tube,Cons,Polycone,Torus2,Trd,Polyhedra,Trap,Sphere,GenTrap,Hype}.cpp, extracted as
text into tests/golden/unit_*.json): every extracted assert passes with the tests' own
comparison, except the few golden_util lists with the reason (rounding-only misses of the
reference's generic kernels, print-only checks its own code fails).
Soft checks (TestCons prints a mismatch instead of asserting) must pass too, except the
ones listed in golden_util.SOFT_EXCEPTIONS, where the reference's own code path gives a
different answer (each entry says why)."""
import numpy as np
import pytest

import golden_util as G


@pytest.mark.parametrize("name", G.FILES)
def test_oracle_matches_reference_unit_tests(name):
    from oracle.oracle import OracleGeometry
    doc = G.load(name)
    assert doc["cases"], "no cases extracted"
    fails = []
    for shape, q, cs, p, d in G.grouped(doc):
        o = OracleGeometry()
        pv = G.build(o, doc["shapes"][shape])
        qi = G.QUERY_ID[q]
        if qi in (2, 3):
            out, _ = o.query(pv, qi, p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy(), d[:, 0].copy(), d[:, 1].copy(),
                             d[:, 2].copy())
        else:
            out, _ = o.query(pv, qi, p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy())
        for c, v in zip(cs, out):
            if not G.case_passes(name, c, v):
                fails.append((c["line"], shape, q, c["p"], c["d"], c["kind"], c["expected"], float(v)))
    assert not fails, "%d of %d fail, first: %s" % (len(fails), len(doc["cases"]), fails[:5])


@pytest.mark.parametrize("name", G.FILES)
def test_extents_match_reference_unit_tests(name):
    """The Extent known answers of the same tests, for the oracle and for the product's host
    geometry builder (whose extents make the BVH boxes); the two also agree exactly."""
    import vecgeom_gb300 as vg
    from oracle.oracle import OracleGeometry
    doc = G.load(name)
    cases = G.extent_cases(doc)
    if not cases:
        pytest.skip("the test file checks no extents")
    for shape, q, expected in cases:
        spec = doc["shapes"][shape]
        got = []
        for geo in (OracleGeometry(), vg.Geometry()):
            s = G.add_shape(geo, spec)
            lo, hi = geo.shape_extent(s)
            got.append(np.array(lo if q == "ExtentMin" else hi))
        assert G.approx_equal_vec(got[0], expected), (name, shape, q, got[0], expected)
        assert np.array_equal(got[0], got[1]), (name, shape, q)


@pytest.mark.parametrize("name", [n for n in G.FILES if any(c["query"] == "Normal" for c in G.load(n)["cases"])])
def test_normals_match_reference_unit_tests(name):
    """The surface-normal known answers (the oracle restates Normal only where a test builds
    points along the shape's normal, which the query checks then use)."""
    from oracle.oracle import OracleGeometry
    doc = G.load(name)
    for c in doc["cases"]:
        if c["query"] != "Normal":
            continue
        o = OracleGeometry()
        n, valid = o.shape_normal(G.add_shape(o, doc["shapes"][c["shape"]]), c["p"])
        assert valid and G.approx_equal_vec(n, c["expected"]), (c["line"], n, c["expected"])


@pytest.mark.parametrize("name", [n for n in G.FILES if G.load(n).get("pairs")])
def test_paired_results_match_reference_unit_tests(name):
    """Asserts comparing two query results with each other (TestHype: ApproxEqual(Dist3, Dist4))."""
    from oracle.oracle import OracleGeometry
    doc = G.load(name)
    for pair in doc["pairs"]:
        vals = []
        for k in (pair["a"], pair["b"]):
            c = doc["cases"][k]
            o = OracleGeometry()
            pv = G.build(o, doc["shapes"][c["shape"]])
            qi = G.QUERY_ID[c["query"]]
            cols = [np.array([v]) for v in c["p"]] + ([np.array([v]) for v in c["d"]] if qi in (2, 3) else [])
            vals.append(float(o.query(pv, qi, *cols)[0][0]))
        assert G.approx_equal(*vals), (pair["line"], vals)


def test_pin_detects_a_planted_error():
    """The same checks on an oracle fed shapes 1e-3 mm larger than the tests construct
    must fail: the known answers are sharp enough to catch a wrong dimension."""
    from oracle.oracle import OracleGeometry
    doc = G.load("Box")
    bad = 0
    for shape, q, cs, p, d in G.grouped(doc):
        spec = dict(doc["shapes"][shape])
        spec["args"] = [a + 1e-3 for a in spec["args"]]
        o = OracleGeometry()
        pv = G.build(o, spec)
        qi = G.QUERY_ID[q]
        cols = [p[:, k].copy() for k in range(3)] + ([d[:, k].copy() for k in range(3)] if qi in (2, 3) else [])
        out, _ = o.query(pv, qi, *cols)
        bad += sum(not G.passes(c["kind"], v, c["expected"], c.get("tol")) for c, v in zip(cs, out))
    assert bad >= 20, bad
