"""GDML reader (vecgeom_gb300/gdml.py) on the CPU: the test detector loads into the product's
builder and into the oracle with identical NavIndex tables and BVHs; units, constants,
references and the rotation convention follow the reference's middleware; unsupported
input fails with a named error; and, where a VecGeom source tree is at hand, the reference's
own example GDML files load (supported solids) or fail cleanly (the others)."""
import math
import os

import numpy as np
import pytest

import vecgeom_gb300 as vg
from oracle.oracle import OracleGeometry
from test_cpu_build import HostOnly
from oracle import build_ref
from vecgeom_gb300 import gdml

HERE = os.path.dirname(os.path.abspath(__file__))
DETECTOR = os.path.join(HERE, "golden", "gdml", "detector.gdml")
# the reference's own example GDML files, where a VecGeom source tree is present (named by
# VECGEOM_SOURCE_DIR, else the tree the compiled-reference recipe reads); the tests that
# read them are skipped otherwise
REF_GDMLS = os.path.join(os.environ.get("VECGEOM_SOURCE_DIR", build_ref.REF), "persistency", "gdml", "gdmls")


def compare(path):
    p, o = vg.Geometry(), OracleGeometry()
    rp = gdml.load(path, HostOnly(p))
    ro = gdml.load(path, o)
    assert rp.world == ro.world and rp.volumes == ro.volumes and rp.solids == ro.solids
    assert np.array_equal(p.nav_table(), o.nav_table())
    info = p.info()
    for lv in range(info["n_lv"]):
        ob = o.bvh(lv)
        if ob is None:
            continue
        pb = p.bvh(lv)
        for k in ("prim", "offset", "nchild", "nodes", "boxes"):
            assert np.array_equal(pb[k], ob[k]), (lv, k)
    for s in rp.solids.values():
        assert np.array_equal(np.array(p.shape_extent(s)), np.array(o.shape_extent(s)))
    return p, o, rp, info


def test_detector_gdml_builds_identically():
    p, o, r, info = compare(DETECTOR)
    assert info["n_pv"] == 2 + 144 + 8 + 2 + 7 + 1 and info["max_depth"] == 3
    assert list(r.volumes) == ["module", "barrel", "wedge", "endcap", "trap", "holder", "ring", "cone", "drilled",
                               "World"]
    # units: the world box in m, the endcap polycone's z planes in cm, a position in cm
    lo, hi = p.shape_extent(r.solids["world_s"])
    assert np.array_equal(hi, (1500.0, 1500.0, 2000.0))
    lo, hi = p.shape_extent(r.solids["endcap_s"])
    assert np.array_equal(hi, (600.0, 600.0, 100.0))
    assert r.positions["endcap_pos"] == (0.0, 0.0, 1000.0) and r.positions["h_p"] == (1100.0, 1100.0, 1400.0)
    # a physvol's inline position is registered under its name; a boolean's is not
    # (Middleware.cpp:1340-1346 and :464-472)
    assert "hole_pos" not in r.positions and "mod5_p" in r.positions
    assert r.rotations["flip"] == (math.pi, 0.0, 0.0)


def test_rotation_convention():
    """makeRotationMatrixFromCartesianAngles: a GDML rotation is the inverse (frame)
    rotation, so z = +90 deg maps the local x axis to global -y."""
    r = np.array(gdml.rotation_from_angles(0.0, 0.0, math.pi / 2)).reshape(3, 3)
    assert np.allclose(r @ (1.0, 0.0, 0.0), (0.0, -1.0, 0.0), atol=1e-15)
    r = np.array(gdml.rotation_from_angles(0.3, -0.7, 1.1)).reshape(3, 3)
    assert np.allclose(r @ r.T, np.eye(3), atol=1e-15) and abs(np.linalg.det(r) - 1.0) < 1e-14


def test_attribute_values_follow_stod_and_constants():
    doc = """<gdml><define><constant name="L" value="25"/></define><solids>
      <box name="a" x="L" y="2*L" z="10.5mm" lunit="cm"/><tube name="t" rmax="5" z="10"/>
      </solids><structure><volume name="w"><solidref ref="a"/></volume></structure>
      <setup><world ref="w"/></setup></gdml>"""
    o = OracleGeometry()
    r = gdml.load(doc, o)
    # "L" -> the constant; "2*L" -> std::stod reads 2; "10.5mm" -> 10.5; lengths in cm, halved
    lo, hi = o.shape_extent(r.solids["a"])
    assert np.array_equal(hi, (125.0, 10.0, 52.5))
    # a tube without rmin / startphi / deltaphi gets 0 for each (the middleware's defaults)
    lo, hi = o.shape_extent(r.solids["t"])
    assert hi[2] == 5.0


def test_arb8_reads_vertices_without_the_length_unit():
    """Middleware::processGenTrap reads v1x..v8y as plain numbers and dz with the length unit."""
    doc = """<gdml><solids>
      <arb8 name="g" v1x="-3" v1y="-3" v2x="-3" v2y="3" v3x="3" v3y="3" v4x="3" v4y="-3"
            v5x="-2" v5y="-2" v6x="-2" v6y="2" v7x="2" v7y="2" v8x="2" v8y="-2" dz="5" lunit="cm"/>
      </solids><structure><volume name="w"><solidref ref="g"/></volume></structure>
      <setup><world ref="w"/></setup></gdml>"""
    for geo in (OracleGeometry(), HostOnly(vg.Geometry())):
        r = gdml.load(doc, geo)
        lo, hi = geo.shape_extent(r.solids["g"])
        assert np.array_equal(lo, (-3.0, -3.0, -50.0)) and np.array_equal(hi, (3.0, 3.0, 50.0))


def test_hype_reads_stereo_angles_without_the_angle_unit():
    """Middleware::processHype reads inst and outst as plain numbers (radians whatever aunit
    says), the radii and z with the length unit; z is the full length."""
    doc = """<gdml><solids>
      <hype name="h" rmin="1" rmax="2" inst="0.5" outst="0.25" z="10" lunit="cm" aunit="deg"/>
      </solids><structure><volume name="w"><solidref ref="h"/></volume></structure>
      <setup><world ref="w"/></setup></gdml>"""
    for geo in (OracleGeometry(), HostOnly(vg.Geometry())):
        r = gdml.load(doc, geo)
        lo, hi = geo.shape_extent(r.solids["h"])
        rmax = math.sqrt(20.0 ** 2 + math.tan(0.25) ** 2 * 50.0 ** 2)
        assert np.allclose(hi, (rmax, rmax, 50.0), rtol=1e-15)


@pytest.mark.parametrize("doc, msg", [
    ("<gdml><solids><orb name='o' r='1'/></solids></gdml>", "unsupported solid <orb>"),
    ("<gdml><solids><box name='b' x='1' y='1' z='1'/><box name='b' x='2' y='1' z='1'/></solids></gdml>",
     "defined twice"),
    ("<gdml><solids><box name='b' x='1' y='1' z='1'/></solids><structure><volume name='w'><solidref ref='b'/>"
     "<physvol><volumeref ref='nope'/></physvol></volume></structure></gdml>", "unknown volume"),
    ("<gdml><solids><box name='b' x='1' y='1' z='1'/></solids><structure><volume name='w'><solidref ref='b'/>"
     "</volume></structure></gdml>", "no <world>"),
])
def test_errors_are_named(doc, msg):
    with pytest.raises(gdml.GDMLError, match=msg):
        gdml.load(doc, OracleGeometry())


SUPPORTED_REF = ["oneBox", "oneTube", "oneConeSegment", "onePolycone", "onePolyhedron", "oneTorus", "oneTrapezoid",
                 "oneGeneralTrapezoid", "twoBoxes", "aPosition", "aRotation", "solidSubtraction", "oneCutTube",
                 "oneSphere", "oneHyperbolicTube"]
UNSUPPORTED_REF = ["oneOrb", "oneParallelepiped", "solidUnion", "solidIntersection",
                   "aConstant", "scaledPhysvol"]


@pytest.mark.skipif(not os.path.isdir(REF_GDMLS), reason="no VecGeom source tree")
def test_reference_arb8_file_with_duplicate_solid_name():
    """oneArbitraryTrapezoid.gdml names two solids "world" (a trd and the arb8): the reference's
    middleware fails the second insertion and its Load returns false
    (persistency/gdml/source/src/Middleware.cpp:643-647, :206-211); the reader raises."""
    with pytest.raises(gdml.GDMLError, match="defined twice"):
        gdml.load(os.path.join(REF_GDMLS, "oneArbitraryTrapezoid.gdml"), OracleGeometry())


@pytest.mark.skipif(not os.path.isdir(REF_GDMLS), reason="no VecGeom source tree")
@pytest.mark.parametrize("name", SUPPORTED_REF)
def test_reference_example_files_load(name):
    compare(os.path.join(REF_GDMLS, name + ".gdml"))


@pytest.mark.skipif(not os.path.isdir(REF_GDMLS), reason="no VecGeom source tree")
@pytest.mark.parametrize("name", UNSUPPORTED_REF)
def test_reference_example_files_unsupported(name):
    with pytest.raises(gdml.GDMLError, match="unsupported|not supported"):
        gdml.load(os.path.join(REF_GDMLS, name + ".gdml"), OracleGeometry())
