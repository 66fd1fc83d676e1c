"""The hand-written oracle against the reference's own code, compiled here (CPU only).

oracle/build_ref.py compiles the reference's sources in place (source/*.cpp and the VecGeom/
headers) against a scalar stand-in for the VecCore library (oracle/compiled_ref/shim), and
oracle/reference.py drives the result through the oracle's own interface, one geometry per
process. Every navigation geometry of the tests and every shape the product builds is then
run on both, on the same inputs:

* the NavIndex table word for word (padding words, which the reference leaves unwritten,
  masked);
* LocateGlobalPoint from the world on the config-5 track starts;
* whole transport histories (ComputeStepAndPropagatedState with BVHNavigator, the point
  moved by each step): every step's out-state and step length, bit for bit;
* 2^16 single steps and step + safety (ComputeStepAndSafetyAndPropagatedState) from
  pre-step states drawn from transport histories;
* whole transport histories in the reference's own example GDML files;
* the six queries of every unplaced shape (Inside, Contains, DistanceToIn/Out, SafetyToIn/
  Out) on points in the 1.2x extent box and on faces, edges and far points, and the same
  queries plus PlacedDistanceToOut through the VPlacedVolume interface of each shape placed
  with a rotation and a translation.

All of it is bit-identical, with one stated exception: for GenTraps whose lateral faces are
all planar, the reference's host build evaluates a TessellatedSection helper
(VecGeom/volumes/kernel/GenTrapImplementation.h:339-345 and the other `#ifndef VECCORE_CUDA`
branches) while its CUDA build, which the product and the oracle reproduce, evaluates the
generic second-order-surface kernels. Those shapes' queries are not compared; in the GenTrap
ring the next volumes and states are identical, the step lengths agree within 1e-9 mm +
1e-12 relative (5.7e-14 mm measured), and the safeties are not compared.

The reference-side bridge (include/vecgeom_gb300_mirror.hpp), compiled into the same build,
mirrors each closed reference geometry into a product geometry through the C-ABI; the result
equals the product geometry the builder makes directly (placed-volume and logical-volume
counts, NavIndex table, every BVH, the shapes' extents), and the oracle built from the
mirror's builder log transports the config-5 tracks exactly as the directly built one.

The compiled reference is itself pinned: the reference's own unit tests of every shape on the
path and of the navigation states (test/unit_tests/Test*.cpp, asserts enabled) are built
against the same library and pass.

Skipped where the reference tree is absent (the checker is built from it)."""
import os

import numpy as np
import pytest

import vecgeom_gb300 as vg
from oracle import reference as R
from oracle.oracle import OracleGeometry, transport_step_sample
from test_cpu_build import HostOnly
from test_cuttube import CUTS
from test_gpu_shapes import POLYHEDRA, edge_points
from test_gpu_sphere import SPHERES
from vecgeom_gb300 import workloads as W

pytestmark = pytest.mark.skipif(not R.available(), reason="the reference tree is not present")

HERE = os.path.dirname(os.path.abspath(__file__))
DETECTOR_GDML = os.path.join(HERE, "golden", "gdml", "detector.gdml")
NT = os.cpu_count() or 1

WL = "vecgeom_gb300.workloads"
GEOMETRIES = {
    "barrel": (WL, "build_barrel", {}),
    "detector": (WL, "build_detector", {}),
    "trap_ring": (WL, "build_trap_ring", {}),
    "gdml_detector": ("oracle.reference", "build_gdml", {"path": DETECTOR_GDML}),
    "cut_tube_ring": (WL, "build_cut_tube_ring", {}),
    "sphere_shells": (WL, "build_sphere_shells", {}),
    "gentrap_ring": (WL, "build_gentrap_ring", {}),
    "hype_ring": (WL, "build_hype_ring", {}),
}
# config-5 tracks transported to the world's edge, primaries whose histories give the 2^16
# sampled pre-step states, and the half-lengths of the box in which restarting tracks start
TRACKS = {"barrel": 1 << 14, "detector": 1 << 13, "gdml_detector": 1 << 14}
PRIMARIES = {"barrel": 16384, "detector": 2048, "gdml_detector": 32768, "sphere_shells": 1 << 15}
HALF = {"barrel": (2000.0, 2000.0, 3000.0), "detector": (2000.0, 2000.0, 3000.0),
        "gdml_detector": (1500.0, 1500.0, 2000.0), "sphere_shells": (600.0, 600.0, 600.0)}
PLANAR_GENTRAPS = ("planar", "pyramid", "anticlockwise")


@pytest.mark.parametrize("name", __import__("oracle.build_ref", fromlist=["UNIT_TESTS"]).UNIT_TESTS)
def test_reference_unit_tests_pass_on_the_stand_in(name):
    import subprocess

    from oracle import build_ref

    exe = build_ref.build_unit_tests()[name]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-2000:])


def test_reference_shape_testers_on_the_stand_in(tmp_path):
    """The reference's shape testers on the stand-in build (run in parallel): every one
    reports 0 errors except Torus2's, which reports 3 misclassified random points (2 inside,
    1 outside) on this build; the reference builds its shape testers but registers none of
    them as a test (test/CMakeLists.txt:300-350), so it states no expected outcome for them."""
    import subprocess
    from concurrent.futures import ThreadPoolExecutor

    from oracle import build_ref

    exes = build_ref.build_shape_testers()

    def run(name):
        d = tmp_path / name
        d.mkdir()
        r = subprocess.run([exes[name]], capture_output=True, text=True, timeout=600, cwd=d)
        last = [ln for ln in r.stdout.splitlines() if "Final Error count" in ln]
        return name, (int(last[-1].split("=")[-1]) if last else None), r.stdout[-2000:]

    with ThreadPoolExecutor(max_workers=NT) as ex:
        results = list(ex.map(run, build_ref.SHAPE_TESTERS))
    for name, errors, tail in results:
        assert errors == (3 if name == "shape_testTorus2" else 0), (name, tail)


def table_padding(t):
    """Mask of the NavIndex table words that hold nothing: the word that rounds a node's
    daughter list to an even count, and the word that aligns a cached matrix to 8 bytes
    (source/NavIndexTable.cpp:24-80; the reference allocates but never writes them)."""
    pad = np.zeros(t.size, bool)
    i = 1
    while i < t.size:
        nd = int(t[i + 2]) >> 16
        hasm = (int(t[i + 2]) >> 8) & 0xFF
        j = i + 3 + nd
        if (nd + 1) & 1:
            pad[j] = True
            j += 1
        if hasm & 0x04:
            if j & 1:
                pad[j] = True
                j += 1
            j += 24
        i = j
    return pad


def bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


@pytest.mark.parametrize("name", sorted(GEOMETRIES))
def test_navigation_equals_compiled_reference(name):
    mod, fn, kw = GEOMETRIES[name]
    o = OracleGeometry()
    getattr(__import__(mod, fromlist=[fn]), fn)(o, **kw)
    n = TRACKS.get(name, 1 << 15)
    (x, y, z), (dx, dy, dz), _ = W.stream_tracks(n, 0xC4EC, world_half=HALF.get(name, (600.0, 600.0, 400.0)))
    st, _ = o.locate(x, y, z, nthreads=NT)
    ns, fin, tr, trs, _ = o.transport(x, y, z, dx, dy, dz, st, 1000, trace=True, nthreads=NT)
    cols, sst, _ = transport_step_sample(o, 1 << 16, 0x5A11, PRIMARIES.get(name, 1 << 16), nthreads=NT)
    s_out, s_step, _, _ = o.step(*cols, sst, nthreads=NT)
    ss_out, ss_step, ss_saf, _ = o.step_safety(*cols, sst, nthreads=NT)

    ref = R.run((mod, fn), [
        ("nav_table", (), {}),
        ("locate", (x, y, z), {"nthreads": NT}),
        ("transport", (x, y, z, dx, dy, dz, st, 1000), {"trace": True, "nthreads": NT}),
        ("step", (*cols, sst), {"nthreads": NT}),
        ("step_safety", (*cols, sst), {"nthreads": NT}),
    ], kw)
    table = o.nav_table()
    assert ref[0].size == table.size
    used = ~table_padding(table)
    assert np.array_equal(ref[0][used], table[used]), "NavIndex table"
    assert np.array_equal(ref[1][0], st), "LocateGlobalPoint"
    r_ns, r_fin, r_tr, r_trs, _ = ref[2]
    assert ns.sum() > n
    assert np.array_equal(r_ns, ns) and np.array_equal(r_fin, fin) and np.array_equal(r_tr, tr), "transport states"
    assert np.array_equal(ref[3][0], s_out), "step out-states"
    assert np.array_equal(ref[4][0], ss_out), "step + safety out-states"
    if name == "gentrap_ring":
        # planar GenTraps: a different host algorithm in the reference (module docstring);
        # the safeties, which the world's include, are not compared
        for a, b in ((r_trs, trs), (ref[3][1], s_step), (ref[4][1], ss_step)):
            assert np.all(np.abs(a - b) <= 1e-9 + 1e-12 * np.abs(b))
    else:
        assert np.array_equal(bits(r_trs), bits(trs)), "transport step lengths"
        assert np.array_equal(bits(ref[3][1]), bits(s_step)), "step lengths"
        assert np.array_equal(bits(ref[4][1]), bits(ss_step)), "step + safety step lengths"
        assert np.array_equal(bits(ref[4][2]), bits(ss_saf)), "safety"


def _shapes():
    out = [(n, k, p) for n, (k, p) in {**W.SHAPES_CFG1, **W.SHAPES_CFG2}.items()]
    out += [("polyhedron_%d" % i, "polyhedron", p) for i, p in enumerate(POLYHEDRA)]
    out += [("sphere_%d" % i, "sphere", p) for i, p in enumerate(SPHERES)]
    out += [("cut_tube_%d" % i, "cut_tube", p) for i, p in enumerate(CUTS)]
    out += [("hype_" + n, "hype", p) for n, p in W.HYPES.items()]
    out += [("gentrap_" + n, "gentrap", p) for n, p in W.GENTRAPS.items()]
    out += [("trap_wedge", "trap", W.TRAP_WEDGE)]
    return out


def test_shape_queries_equal_compiled_reference():
    shapes = _shapes()
    o = OracleGeometry()
    ids = [W.add_shape(o, k, p) for _, k, p in shapes]
    calls, expect = [], []
    for i, ((name, _, _), sid) in enumerate(zip(shapes, ids)):
        if name in ["gentrap_" + k for k in PLANAR_GENTRAPS]:
            continue
        lo, hi = o.shape_extent(sid)
        for pts, dirs in (W.shape_points_box(lo, hi, 1 << 14, seed=77 + i), edge_points(lo, hi, 4096, 99 + i)):
            for q in range(6):
                d = dirs if q in (2, 3) else (None, None, None)
                calls.append(("shape_query", (sid, q, *pts, *d), {"nthreads": NT}))
                expect.append(((name, q), o.shape_query(sid, q, *pts, *d, nthreads=NT)))
    got = R.run(("oracle.reference", "build_shapes"), calls, {"shapes": [(k, p) for _, k, p in shapes]})
    bad = [key for (key, e), g in zip(expect, got) if not np.array_equal(bits(g), bits(e))]
    assert len(got) > 300
    assert not bad, bad


@pytest.mark.parametrize("name", sorted(GEOMETRIES))
def test_mirror_of_reference_geometry_equals_builder(name):
    mod, fn, kw = GEOMETRIES[name]
    builder = getattr(__import__(mod, fromlist=[fn]), fn)
    p = vg.Geometry()
    builder(HostOnly(p), **kw)
    direct = R.product_summary(p)
    mirror = R.run((mod, fn), [("mirror_to_product", (), {})], kw)[0]
    assert mirror["info"] == direct["info"]
    assert np.array_equal(mirror["nav_table"], direct["nav_table"])
    for lv, (a, b) in enumerate(zip(mirror["bvh"], direct["bvh"])):
        assert (a is None) == (b is None), lv
        if a is not None:
            assert all(np.array_equal(a[k], b[k]) for k in a), lv
    # shapes may be created in another order (a GDML file lists its solids first)
    key = lambda e: tuple(np.concatenate(e).view(np.uint64))
    assert sorted(map(key, mirror["extents"])) == sorted(map(key, direct["extents"]))

    o_direct = OracleGeometry()
    builder(o_direct, **kw)
    o_mirror = R.replay_builder_log(mirror["builder_log"], OracleGeometry())
    assert np.array_equal(o_mirror.nav_table(), o_direct.nav_table())
    (x, y, z), (dx, dy, dz), _ = W.stream_tracks(1 << 13, 0x3177, world_half=HALF.get(name, (600.0, 600.0, 400.0)))
    st, _ = o_direct.locate(x, y, z, nthreads=NT)
    st_m, _ = o_mirror.locate(x, y, z, nthreads=NT)
    assert np.array_equal(st_m, st)
    a = o_direct.transport(x, y, z, dx, dy, dz, st, 1000, trace=True, nthreads=NT)
    b = o_mirror.transport(x, y, z, dx, dy, dz, st, 1000, trace=True, nthreads=NT)
    assert a[0].sum() > 1 << 13
    for u, v in zip(a[:4], b[:4]):
        assert np.array_equal(bits(u), bits(v))


def test_placed_queries_equal_compiled_reference():
    from vecgeom_gb300.workloads import rot_z

    shapes = [(n, k, p) for n, k, p in _shapes() if n not in ["gentrap_" + g for g in PLANAR_GENTRAPS]]
    g = np.random.default_rng(5)
    placements = []
    for i in range(len(shapes)):
        c, s_ = np.cos(0.3 * i + 0.1), np.sin(0.3 * i + 0.1)
        rx = (1.0, 0.0, 0.0, 0.0, c, -s_, 0.0, s_, c)  # a tilt about x, then a turn about z
        rz = np.asarray(rot_z(0.7 * i)).reshape(3, 3)
        rot = tuple((rz @ np.asarray(rx).reshape(3, 3)).reshape(9))
        placements.append((tuple(g.uniform(-50.0, 50.0, 3)), rot))
    o = OracleGeometry()
    made = R.build_placed_shapes(o, [(k, p) for _, k, p in shapes], placements)
    calls, expect = [], []
    for i, ((name, _, _), (sid, pv), (t, _)) in enumerate(zip(shapes, made, placements)):
        lo, hi = o.shape_extent(sid)
        (px, py, pz), dirs = W.shape_points_box(lo, hi, 1 << 13, seed=500 + i, scale=1.5)
        pts = (px + t[0], py + t[1], pz + t[2])  # about the placed shape, in the mother's frame
        for q in range(7):
            d = dirs if q in (2, 3, 6) else (None, None, None)
            calls.append(("query", (pv, q, *pts, *d), {"nthreads": NT}))
            expect.append(((name, q), o.query(pv, q, *pts, *d, nthreads=NT)[0]))
    got = R.run(("oracle.reference", "build_placed_shapes"), calls,
                {"shapes": [(k, p) for _, k, p in shapes], "placements": placements})
    assert len(got) == 7 * len(shapes) > 200
    bad = [key for (key, e), r in zip(expect, got) if not np.array_equal(bits(r[0]), bits(e))]
    assert not bad, bad


def test_navigator_adapter_host_path_equals_reference():
    """The reference-side navigator adapter compiles against the reference's headers and,
    installed on every volume in place of BVHNavigator, steps the tracks as the reference
    does on the methods it keeps on the host (its vector entry point is the GPU call)."""
    mod, fn, kw = GEOMETRIES["detector"]
    o = OracleGeometry()
    getattr(__import__(mod, fromlist=[fn]), fn)(o, **kw)
    cols, sst, _ = transport_step_sample(o, 1 << 14, 0x5A11, PRIMARIES["detector"], nthreads=NT)
    out, step, _, _ = o.step(*cols, sst, nthreads=NT)
    r_out, r_step = R.run((mod, fn), [("adapter_step", (*cols, sst), {})], kw)[0]
    assert np.array_equal(r_out, out)
    assert np.array_equal(bits(r_step), bits(step))


@pytest.mark.parametrize("name", __import__("test_gdml").SUPPORTED_REF)
def test_reference_example_gdml_navigation_equals_compiled_reference(name):
    """The reference's own example GDML files (persistency/gdml/gdmls) read by the product's
    reader into the oracle and into the reference's own classes: whole transport histories
    bit-identical (planar GenTraps excepted, as above)."""
    from test_gdml import REF_GDMLS
    from vecgeom_gb300 import gdml

    path = os.path.join(REF_GDMLS, name + ".gdml")
    o = OracleGeometry()
    r = gdml.load(path, o)
    ext = [o.shape_extent(s) for s in sorted(set(r.solids.values()))]
    lo = np.min([e[0] for e in ext], axis=0)
    hi = np.max([e[1] for e in ext], axis=0)
    (x, y, z), (dx, dy, dz) = W.shape_points_box(lo, hi, 1 << 13, seed=0x6D1, scale=1.0)
    st, _ = o.locate(x, y, z, nthreads=NT)
    a = o.transport(x, y, z, dx, dy, dz, st, 1000, trace=True, nthreads=NT)
    ref = R.run(("oracle.reference", "build_gdml"), [
        ("locate", (x, y, z), {"nthreads": NT}),
        ("transport", (x, y, z, dx, dy, dz, st, 1000), {"trace": True, "nthreads": NT})], {"path": path})
    assert np.array_equal(ref[0][0], st)
    assert a[0].sum() > 300
    b = ref[1]
    assert np.array_equal(b[0], a[0]) and np.array_equal(b[1], a[1]) and np.array_equal(b[2], a[2])
    if name == "oneGeneralTrapezoid":
        assert np.all(np.abs(b[3] - a[3]) <= 1e-9 + 1e-12 * np.abs(a[3]))
    else:
        assert np.array_equal(bits(b[3]), bits(a[3]))


def test_mirror_rejects_a_shape_outside_the_product_set():
    """A closed reference geometry holding an Orb: MirrorGeometry returns VG_EINVAL and names
    the first placed volume it cannot mirror (the Orb, id 1), so the caller keeps that
    geometry on the reference's path."""
    with pytest.raises(RuntimeError, match=r"mirror failed \(-1\) at placed volume 1"):
        R.run(("oracle.reference", "build_with_orb"), [("mirror_to_product", (), {})])
