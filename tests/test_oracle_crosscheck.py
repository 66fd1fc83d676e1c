"""The navigation oracle checked the way the reference checks its own navigators (CPU only).

* persistency/gdml/test/TestVGDMLNavigation/TestVGDMLNavigation.cpp:54-91 validates the BVH
  navigator by stepping tracks to the edge of the world and comparing every step with the
  brute-force NewSimpleNavigator (VecGeom/navigation/NewSimpleNavigator.h:33-63), which
  shares no traversal code with the BVH. The oracle holds both navigators (the brute-force
  one relocates with SimpleLevelLocator as well), and they must agree on every step: the
  reference's nearly_equal criterion, and here also every bit of the step and every field
  of the out-state.
* The same comparison on single steps from 2^16 pre-step states drawn from transport
  histories (states on boundaries, with a last-exited volume, in every kind of volume).
* test/benchmark/TestNavIndex.cpp: the NavIndex table's invariants over every placed-volume
  path (index recomputed from the path, top volume, level, push/pop, daughter count, cached
  global matrix equal to the product of the path's transformations), for the oracle's table
  and for the product's (built by the product's host-side geometry builder)."""
import os

import numpy as np
import pytest

import vecgeom_gb300 as vg
from oracle.oracle import OracleGeometry, transport_step_sample
from test_cpu_build import HostOnly
from vecgeom_gb300 import gdml
from vecgeom_gb300 import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
DETECTOR_GDML = os.path.join(HERE, "golden", "gdml", "detector.gdml")
NT = os.cpu_count() or 1


def _gdml(geo):
    gdml.load(DETECTOR_GDML, geo)


GEOMETRIES = {"barrel": W.build_barrel, "detector": W.build_detector, "trap_ring": W.build_trap_ring,
              "gdml_detector": _gdml, "cut_tube_ring": W.build_cut_tube_ring,
              "sphere_shells": W.build_sphere_shells, "gentrap_ring": W.build_gentrap_ring,
              "hype_ring": W.build_hype_ring}
# full-track cross-checks per geometry (the config-4 detector's brute force is the slowest),
# and the half-lengths of the box in which restarting tracks start (about the world's)
TRACKS = {"barrel": 1 << 16, "detector": 1 << 13, "trap_ring": 1 << 16, "gdml_detector": 1 << 16,
          "cut_tube_ring": 1 << 16, "sphere_shells": 1 << 16, "gentrap_ring": 1 << 16, "hype_ring": 1 << 16}
# primaries whose transport histories give at least 2^16 pre-step states
PRIMARIES = {"barrel": 16384, "detector": 2048, "trap_ring": 1 << 16, "gdml_detector": 32768,
             "cut_tube_ring": 1 << 16, "sphere_shells": 1 << 15, "gentrap_ring": 1 << 16, "hype_ring": 1 << 16}
HALF = {"barrel": (2000.0, 2000.0, 3000.0), "detector": (2000.0, 2000.0, 3000.0), "trap_ring": (600.0, 600.0, 400.0),
        "gdml_detector": (1500.0, 1500.0, 2000.0), "cut_tube_ring": (600.0, 600.0, 400.0),
        "sphere_shells": (600.0, 600.0, 600.0), "gentrap_ring": (600.0, 600.0, 400.0),
        "hype_ring": (600.0, 600.0, 400.0)}


@pytest.fixture(scope="module", params=sorted(GEOMETRIES))
def geometry(request):
    o = OracleGeometry()
    GEOMETRIES[request.param](o)
    return request.param, o


def test_bvh_navigator_equals_brute_force_along_tracks(geometry):
    name, o = geometry
    n = TRACKS[name]
    # the config-5 track mix: primaries from the origin (eta in [-3, 3]) and 20 % restarting
    # at uniform points of a box around the geometry
    (x, y, z), (dx, dy, dz), _ = W.stream_tracks(n, 0xC4EC, world_half=HALF[name])
    c = o.crosscheck(x, y, z, dx, dy, dz, max_steps=1000, nthreads=NT)
    assert c["steps"] > n
    assert c["not_nearly_equal"] == 0, c
    assert c["bit_different"] == 0, c
    assert c["state_different"] == 0, c
    assert c["start_state_different"] == 0, c


def test_bvh_navigator_equals_brute_force_on_sampled_steps(geometry):
    name, o = geometry
    cols, st, total = transport_step_sample(o, 1 << 16, 0x5A11, PRIMARIES[name], nthreads=NT)
    assert len(st) == 1 << 16
    a_out, a_step, _, _ = o.step(*cols, st, nthreads=NT)
    b_out, b_step, _, _ = o.step(*cols, st, nthreads=NT, navigator="simple")
    for f in ("nav_ind", "last_exited", "on_boundary"):
        assert np.array_equal(a_out[f], b_out[f]), f
    assert np.array_equal(a_step.view(np.int64), b_step.view(np.int64))
    # the sample covers boundary states and states with a last-exited volume
    assert (st["on_boundary"] == 1).mean() > 0.2 and (st["last_exited"] != 0).mean() > 0.2
    # the two level locators place the sampled points identically
    la, _ = o.locate(*cols[:3], nthreads=NT)
    lb, _ = o.locate(*cols[:3], nthreads=NT, navigator="simple")
    assert np.array_equal(la["nav_ind"], lb["nav_ind"])


def test_nav_index_table_invariants(geometry):
    name, o = geometry
    err, paths = o.check_nav_index()
    assert err == 0, err
    assert paths > 0
    p = vg.Geometry()
    GEOMETRIES[name](HostOnly(p))
    err_p, paths_p = o.check_nav_index(p.nav_table())
    assert err_p == 0 and paths_p == paths


def test_nav_index_check_is_sharp():
    """A table with one corrupted word (a daughter pointer, a level byte, a cached matrix
    element) fails the reference's checks."""
    o = OracleGeometry()
    W.build_trap_ring(o)
    tab = o.nav_table()
    assert o.check_nav_index(tab)[0] == 0
    # world: [mother, pv id, level|flags|ndaughters, daughter indices...]
    bad = tab.copy()
    bad[1 + 3] = bad[1 + 4]  # first daughter index points at the second daughter's entry
    assert o.check_nav_index(bad)[0] != 0
    bad = tab.copy()
    d0 = int(tab[1 + 3])
    bad[d0 + 2] ^= 0x01  # the first daughter's level byte
    assert o.check_nav_index(bad)[0] != 0
    bad = tab.copy()
    nd = (int(tab[d0 + 2]) >> 16) & 0xFFFF
    w = d0 + 3 + nd + ((nd + 1) & 1)
    w += w & 1
    m = bad[w:w + 24].view(np.float64).copy()
    m[0] += 1e-3  # the cached translation of the first daughter
    bad[w:w + 24] = m.view(np.uint32)
    assert o.check_nav_index(bad)[0] == 7
