"""The oracle's boolean subtraction against the known answers of the reference's boolean
unit test (tests/golden/unit_Booleans.json, made by tests/golden/extract_booleans.py from
test/unit_tests/TestBooleans.cpp): a box minus a union of two tubes, the union itself, and
a union of that union with a rotated slab. The union is test infrastructure of the oracle
only; the subtraction is the product's Box minus Tube logic, which the GPU kernels match
on the config-2 points. A planted error (the subtraction's push distance) fails the
answers, so the pin is sharp."""
import json
import os

import numpy as np
import pytest

from golden_util import GOLDEN, approx_equal, passes
from oracle.oracle import OracleGeometry

QUERY = {"Contains": 1, "DistanceToIn": 2, "DistanceToOut": 3, "PlacedDistanceToOut": 6}


def load():
    with open(os.path.join(GOLDEN, "unit_Booleans.json")) as f:
        return json.load(f)


def build(doc):
    """The test's geometry in the oracle, in the order the test creates it: name -> id."""
    o = OracleGeometry()
    ids = {"shape": {}, "lv": {}, "pv": {}}
    for kind, name in doc["order"]:
        if kind == "shape":
            s = doc["shapes"][name]
            a = s["args"]
            if s["type"] == "box":
                ids["shape"][name] = o.add_box(*a)
            elif s["type"] == "tube":
                ids["shape"][name] = o.add_tube(*a)
            elif s["type"] == "union":
                ids["shape"][name] = o.add_boolean_union(ids["pv"][a[0]], ids["pv"][a[1]])
            else:
                ids["shape"][name] = o.add_boolean_subtraction(ids["pv"][a[0]], ids["pv"][a[1]])
        elif kind == "lv":
            ids["lv"][name] = o.add_logical_volume(ids["shape"][doc["lvs"][name]])
        else:
            p = doc["pvs"][name]
            ids["pv"][name] = o.place(ids["lv"][p["lv"]], p["trans"], p["rot"])
    o.close()
    return o, ids["pv"]


def evaluate(o, pvs, call):
    q = QUERY[call["query"]]
    p = [np.array([v]) for v in call["p"]]
    d = [np.array([v]) for v in (call["d"] or [0.0, 0.0, 1.0])]
    out, _ = o.query(pvs[call["volume"]], q, *p, *d)
    return float(out[0])


def check_all(o, pvs, doc):
    fails = []
    for c in doc["cases"]:
        if c["kind"] == "approx_pair":
            a, b = evaluate(o, pvs, c["a"]), evaluate(o, pvs, c["b"])
            if not approx_equal(a, b):
                fails.append((c["line"], a, b))
            continue
        v = evaluate(o, pvs, c)
        if not passes(c["kind"], v, c["expected"]):
            fails.append((c["line"], c["volume"], c["query"], c["expected"], v))
    return fails


def test_fixture_covers_the_test():
    doc = load()
    assert len(doc["cases"]) == 40
    kinds = {(c.get("volume"), c.get("query")) for c in doc["cases"]}
    assert ("placedcombinedboolean", "DistanceToIn") in kinds and ("placedcombinedboolean", "DistanceToOut") in kinds
    assert ("placedcombinedboolean", "Contains") in kinds and ("placedtubesslabunion", "PlacedDistanceToOut") in kinds


def test_oracle_booleans_pass_reference_answers():
    doc = load()
    o, pvs = build(doc)
    assert check_all(o, pvs, doc) == []


def test_planted_error_fails():
    """The same answers with the box made 1e-3 mm larger: the subtraction's distances move
    and the reference's answers catch it."""
    doc = load()
    doc["shapes"]["box"]["args"] = [a + 1e-3 for a in doc["shapes"]["box"]["args"]]
    o, pvs = build(doc)
    assert len(check_all(o, pvs, doc)) >= 5


@pytest.mark.parametrize("shape", ["holes", "tubesandslabunion"])
def test_union_extent_bounds_its_operands(shape):
    """UnplacedBooleanVolume<kUnion>::Extent is the box around both operands' boxes."""
    doc = load()
    o, pvs = build(doc)
    sid = list(doc["shapes"]).index(shape)
    lo, hi = o.shape_extent(sid)
    # the tubes (radius 2.25 at +-(2.5, 2.5), half-length 10) bound both unions: the slab
    # rotated by 45 degrees reaches only +-3.21 in x and y
    r = doc["shapes"]["tube"]["args"][1]
    assert np.allclose(lo, (-2.5 - r, -2.5 - r, -10.0)) and np.allclose(hi, (2.5 + r, 2.5 + r, 10.0))
