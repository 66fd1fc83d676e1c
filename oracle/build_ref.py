"""Build the compiled-reference oracle (test infrastructure; see compiled_ref/harness.cpp).

Compiles the reference's own C++ sources in place, where they lie in the reference tree
(VecGeom/ headers, source/*.cpp), against the scalar VecCore stand-in and the configuration
header in oracle/compiled_ref/shim/, together with oracle/compiled_ref/harness.cpp, into
oracle/_ref/libvgref.so. Nothing of the reference is copied into this repository and the
reference's own build system (CMake) is not run. The flags are the hand-written oracle's
(oracle/build.py): -O2 -std=c++17 -ffp-contract=off, so every +, -, *, / and sqrt rounds
as in the reference's scalar FP64 build on x86-64, plus -DNDEBUG as in the reference's
default Release build (CMakeLists.txt:40-42); its asserts are not meant to run there (the
one at source/NavIndexTable.cpp:81 fails whenever a node's matrix needs alignment padding).

Run only where the reference tree exists (VG_REFERENCE_DIR, default the sibling checkout
named below); elsewhere `available()` is False and the tests that use it skip.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("VG_REFERENCE_DIR", "/root/reference")
SHIM = os.path.join(HERE, "compiled_ref", "shim")
HARNESS = os.path.join(HERE, "compiled_ref", "harness.cpp")
ROOT = os.path.dirname(HERE)
PRODUCT_INCLUDE = os.path.join(ROOT, "include")  # the C-ABI and the reference-side bridge
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libvgref.so")
FLAGS = ["-O2", "-DNDEBUG", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-w"]

# The reference's translation units on the path: geometry (logical and placed volumes,
# transformations, the geometry manager, bounding boxes, BVHs, the navigation index table
# and states) and the shapes the builders make, with their helpers.
SOURCES = [
    "GeoManager", "LogicalVolume", "PlacedVolume", "UnplacedVolume", "Transformation3D", "ABBoxManager", "BVH",
    "BVHManager", "NavIndexTable", "NavStateIndex", "NavStatePath", "MessageLogger", "SOA3D", "AOS3D", "Vector",
    "Scale3D", "Wedge", "Wedge_Evolution", "Planes", "Plane", "Quadrilaterals", "Rectangles", "Utils3D",
    "ReducedPolycone", "CutPlanes", "TessellatedHelpers", "Tile", "SolidMesh", "HybridManager2",
    "UnplacedBox", "PlacedBox", "UnplacedTube", "PlacedTube", "UnplacedCone", "PlacedCone", "UnplacedPolycone",
    "PlacedPolycone", "UnplacedPolyhedron", "PlacedPolyhedron", "UnplacedTorus2", "PlacedTorus2", "UnplacedTrd",
    "PlacedTrd", "UnplacedBooleanVolume", "PlacedBooleanVolume", "UnplacedTrapezoid", "PlacedTrapezoid",
    "UnplacedSphere", "PlacedSphere", "UnplacedHype", "PlacedHype", "UnplacedGenTrap", "PlacedGenTrap",
    "UnplacedCutTube", "PlacedCutTube", "UnplacedAssembly", "PlacedAssembly", "UnplacedScaledShape",
    "PlacedScaledShape", "UnplacedOrb", "PlacedOrb", "UnplacedParallelepiped", "PlacedParallelepiped",
    "UnplacedMultiUnion", "PlacedMultiUnion", "UnplacedTessellated", "PlacedTessellated", "UnplacedExtruded",
    "PlacedExtruded", "UnplacedSExtruVolume", "PlacedSExtru", "UnplacedGenericPolycone", "PlacedGenericPolycone",
    "UnplacedCoaxialCones", "PlacedCoaxialCones", "UnplacedEllipticalTube", "PlacedEllipticalTube",
    "UnplacedEllipticalCone", "PlacedEllipticalCone", "UnplacedEllipsoid", "PlacedEllipsoid", "UnplacedParaboloid",
    "PlacedParaboloid", "UnplacedTet", "PlacedTet",
]


# The reference's own unit tests of the shapes and navigation states on the path
# (test/unit_tests/*.cpp, each a program of asserts), built against the same library: their
# passing pins the VecCore stand-in and the configuration header.
UNIT_TESTS = ["TestBox", "TestTube", "TestCons", "TestPolycone", "TestPolyhedra", "TestTorus2", "TestTrd",
              "TestBooleans", "TestTrap", "TestSphere", "TestHype", "TestGenTrap", "TestNavStateIndex",
              "TestReducedPolycone", "TestVecGeomPolycone"]
UNIT_DIR = os.path.join(OUT_DIR, "unit_tests")


# The reference's shape testers (test/shape_tester/shape_test*.cpp with ShapeTester.cpp and
# ConventionChecker.cpp: random inside, outside and surface points, the conventions of every
# query, distance accuracy), for the shapes on the path.
SHAPE_TESTERS = ["shape_testBox", "shape_testTube", "shape_testCone", "shape_testPolycone", "shape_testPolyhedron",
                 "shape_testTorus2", "shape_testTrd", "shape_testTrapezoid", "shape_testSphere", "shape_testHype",
                 "shape_testGenTrap", "shape_testCutTube"]


def available():
    return os.path.isdir(os.path.join(REF, "VecGeom")) and os.path.isdir(os.path.join(REF, "source"))


def build(force=False, verbose=False):
    if not available():
        raise FileNotFoundError("reference tree not found at %s (set VG_REFERENCE_DIR)" % REF)
    os.makedirs(OUT_DIR, exist_ok=True)
    from vecgeom_gb300 import build as product_build

    product_lib = product_build.LIB if os.path.exists(product_build.LIB) else product_build.build()
    inc = ["-I", SHIM, "-I", REF, "-I", PRODUCT_INCLUDE]
    shim_files = [os.path.join(d, f) for d, _, fs in os.walk(SHIM) for f in fs]
    newest_dep = max(os.path.getmtime(f) for f in shim_files + [__file__])
    bridge = [os.path.join(PRODUCT_INCLUDE, f)
              for f in ("vecgeom_gb300.h", "vecgeom_gb300_mirror.hpp", "vecgeom_gb300_navigator.hpp")]
    newest_bridge = max(os.path.getmtime(f) for f in bridge)
    units = [(os.path.join(REF, "source", s + ".cpp"), os.path.join(OUT_DIR, s + ".o")) for s in SOURCES]
    units.append((HARNESS, os.path.join(OUT_DIR, "harness.o")))
    jobs = []
    for src, obj in units:
        dep = max(os.path.getmtime(src), newest_dep, newest_bridge if src == HARNESS else 0.0)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < dep:
            jobs.append(["g++", *FLAGS, *inc, "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compiled-reference build failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(run, jobs))
    libdir = os.path.dirname(product_lib)
    if jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(product_lib):
        run(["g++", "-shared", "-o", LIB, *[o for _, o in units], "-L", libdir, "-lvecgeom_gb300",
             "-Wl,-rpath," + libdir, "-pthread", "-Wl,--no-undefined"])
    return LIB


def build_unit_tests(verbose=False):
    """Compile UNIT_TESTS (asserts enabled: no -DNDEBUG in these translation units) against
    the library; returns {name: executable path}."""
    lib = build(verbose=verbose)
    os.makedirs(UNIT_DIR, exist_ok=True)
    src_dir = os.path.join(REF, "test", "unit_tests")
    flags = [f for f in FLAGS if f not in ("-DNDEBUG", "-fPIC")]
    inc = ["-I", SHIM, "-I", REF, "-I", src_dir]
    libdir = os.path.dirname(lib)
    jobs, exes = [], {}
    for t in UNIT_TESTS:
        src, exe = os.path.join(src_dir, t + ".cpp"), os.path.join(UNIT_DIR, t)
        exes[t] = exe
        if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(src), os.path.getmtime(lib)):
            jobs.append(["g++", *flags, *inc, src, "-o", exe, "-L", libdir, "-lvgref", "-Wl,-rpath," + libdir])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("unit-test build failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(run, jobs))
    return exes


def build_shape_testers(verbose=False):
    """Compile SHAPE_TESTERS against the library; returns {name: executable path}."""
    lib = build(verbose=verbose)
    os.makedirs(UNIT_DIR, exist_ok=True)
    src_dir = os.path.join(REF, "test", "shape_tester")
    flags = [f for f in FLAGS if f not in ("-DNDEBUG", "-fPIC")]
    inc = ["-I", SHIM, "-I", REF, "-I", src_dir]
    libdir = os.path.dirname(lib)
    common = [os.path.join(src_dir, f) for f in ("ShapeTester.cpp", "ConventionChecker.cpp")]
    jobs, exes = [], {}
    for t in SHAPE_TESTERS:
        src, exe = os.path.join(src_dir, t + ".cpp"), os.path.join(UNIT_DIR, t)
        exes[t] = exe
        newest = max(os.path.getmtime(f) for f in [src, lib] + common)
        if not os.path.exists(exe) or os.path.getmtime(exe) < newest:
            jobs.append(["g++", *flags, *inc, src, *common, "-o", exe, "-L", libdir, "-lvgref",
                         "-Wl,-rpath," + libdir])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("shape-tester build failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(run, jobs))
    return exes


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
