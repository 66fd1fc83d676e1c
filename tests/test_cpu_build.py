"""CPU tests: the C-ABI library loads and exports every declared symbol, and the product's
host geometry builder reproduces the oracle's daughter boxes, BVHs and NavIndex table
bit-for-bit (no GPU needed: vg_geom_build flattens on the host only)."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

from conftest import ROOT
import __graft_entry__

__graft_entry__.build()

import vecgeom_gb300 as vg  # noqa: E402
from vecgeom_gb300 import workloads as W  # noqa: E402
from oracle.oracle import OracleGeometry  # noqa: E402


def declared_symbols():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"\b(vg_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(vg.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_abi():
    bound = set(vg._SIGS)
    assert set(declared_symbols()) <= bound | set()


class HostOnly:
    """Forwards construction calls; close() only flattens on the host (no GPU)."""

    def __init__(self, g):
        self.g = g

    def __getattr__(self, n):
        return getattr(self.g, n)

    def close(self):
        self.g.build()


def compare_builders(builder, **kw):
    p, o = vg.Geometry(), OracleGeometry()
    builder(HostOnly(p), **kw)
    builder(o, **kw)
    assert np.array_equal(p.nav_table(), o.nav_table())
    info = p.info()
    assert info["max_depth"] == o.max_depth()
    nbvh = 0
    for lv in range(info["n_lv"]):
        ob = o.bvh(lv)
        if ob is None:
            continue
        pb = p.bvh(lv)
        nbvh += 1
        assert pb["depth"] == ob["depth"]
        for k in ("prim", "offset", "nchild", "nodes", "boxes"):
            assert np.array_equal(pb[k], ob[k]), (lv, k)
    return info, nbvh


def test_barrel_tables_match_oracle():
    info, nbvh = compare_builders(W.build_barrel)
    assert info["n_pv"] > 3500 and info["max_depth"] == 4 and nbvh == 12


def test_small_barrel_variants_match_oracle():
    for seed in (1, 2, 3):
        compare_builders(W.build_barrel, seed=seed, nlayers=4, n0=20, n1=300)


def test_trap_ring_tables_match_oracle():
    info, nbvh = compare_builders(W.build_trap_ring)
    assert info["n_pv"] == 1 + 48 + 1 and nbvh >= 1


def test_trap_records_match_oracle_and_reference_extents():
    """Trapezoid extents from the host records equal the oracle's, and the published ones of
    test/unit_tests/TestTrap.cpp (TestVECGEOM393: Trap(60, 20 deg, 5 deg, 40, 30, 40, 10 deg,
    16, 10, 14, 10 deg); trap2 from corners)."""
    deg = np.arctan(1.0) / 45.0
    par = (60.0, 20 * deg, 5 * deg, 40.0, 30.0, 40.0, 10 * deg, 16.0, 10.0, 14.0, 10 * deg)
    corners = [(-10.0, -20.0, -40.0), (10.0, -20.0, -40.0), (-10.0, 20.0, -40.0), (10.0, 20.0, -40.0),
               (-30.0, -40.0, 40.0), (30.0, -40.0, 40.0), (-30.0, 40.0, 40.0), (30.0, 40.0, 40.0)]
    p, o = vg.Geometry(), OracleGeometry()
    for geo in (p, o):
        geo.add_trap(*par)
        geo.add_trap_corners(corners)
        geo.add_trap(*W.TRAP_WEDGE)
        geo.add_trap_corners(0.5 * W.trap_corners(*W.TRAP_WEDGE))
    for s in range(4):
        assert np.array_equal(np.array(p.shape_extent(s)), np.array(o.shape_extent(s))), s
    lo, hi = p.shape_extent(0)
    assert np.allclose(lo, (-58.80819229, -41.90332577, -60.0), rtol=0, atol=1e-8)
    assert np.allclose(hi, (38.57634475, 38.09667423, 60.0), rtol=0, atol=1e-8)
    lo, hi = p.shape_extent(1)
    assert np.allclose(lo, (-30.0, -40.0, -40.0)) and np.allclose(hi, (30.0, 40.0, 40.0))
    with pytest.raises(vg.VGError):
        p.add_trap(0.0, 0.0, 0.0, 1.0, 1.0, 1.0, 0.0, 1.0, 1.0, 1.0, 0.0)


def planes_from_corners(c):
    """The four side planes (a, b, c, d) of a trapezoid from its corners, in plain float
    arithmetic in the order of UnplacedTrapezoid.cpp:569-620 (so bit-equal to the C++)."""
    out = []
    for f in ((0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)):
        p1, p2, p3, p4 = (tuple(float(v) for v in c[k]) for k in f)
        u = [p3[j] - p1[j] for j in range(3)]
        v = [p4[j] - p2[j] for j in range(3)]
        n = [u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]]
        inv = 1.0 / math.sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2])
        n = [x * inv for x in n]
        ctr = [0.25 * (((p1[j] + p2[j]) + p3[j]) + p4[j]) for j in range(3)]
        out += [n[0], n[1], n[2], -(n[0] * ctr[0] + n[1] * ctr[1] + n[2] * ctr[2])]
    return out


def test_trap_from_planes_equals_trap_from_corners():
    """vg_geom_add_trap_planes (the exact mirror of an existing trapezoid) gives the same
    record as the corner constructor when fed that constructor's planes."""
    corners = W.trap_corners(*W.TRAP_WEDGE)
    p, o = vg.Geometry(), OracleGeometry()
    for geo in (p, o):
        geo.add_trap_corners(corners)
        geo.add_trap_planes(float(corners[7][2]), planes_from_corners(corners))
    for geo in (p, o):
        assert np.array_equal(np.array(geo.shape_extent(0)), np.array(geo.shape_extent(1)))
    assert np.array_equal(np.array(p.shape_extent(1)), np.array(o.shape_extent(1)))


def test_builder_rejects_bad_ids():
    g = vg.Geometry()
    with pytest.raises(vg.VGError):
        g.add_logical_volume(5)
    s = g.add_box(1, 1, 1)
    lv = g.add_logical_volume(s)
    with pytest.raises(vg.VGError):
        g.place_daughter(7, lv)
    with pytest.raises(vg.VGError):
        g.set_world(3)


def declared_arity():
    """Parameter count of every vg_* function declared in include/*.h."""
    out = {}
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            src = re.sub(r"/\*.*?\*/", "", open(os.path.join(inc, f)).read(), flags=re.S)
            for name, params in re.findall(r"\b(vg_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
                params = params.strip()
                out[name] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_binding_arity_matches_header():
    ar = declared_arity()
    assert len(ar) >= 25
    for name, (res, args) in vg._SIGS.items():
        assert name in ar, name
        assert len(args) == ar[name], (name, len(args), ar[name])


def test_geometry_save_and_load_replay(tmp_path):
    """vg_geom_save / vg_geom_load: a detector-like geometry (GDML: every supported solid,
    a boolean, rotations) and the barrel, saved and loaded into a new handle, give the same
    NavIndex table, BVHs and shape extents; a missing or foreign file fails."""
    from vecgeom_gb300 import gdml
    det = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gdml", "detector.gdml")
    for build in (lambda g: gdml.load(det, g, close=False), lambda g: W.build_barrel(g, nlayers=4, close=False)):
        a = vg.Geometry()
        build(a)
        path = str(tmp_path / "geom.vgg")
        a.save(path)
        b = vg.Geometry.load(path)
        assert b.pv_lv == a.pv_lv
        a.build()
        b.build()
        ia = a.info()
        assert ia == b.info() and ia["n_pv"] > 100
        assert np.array_equal(a.nav_table(), b.nav_table())
        for lv in range(ia["n_lv"]):  # the logical volumes with daughters have a BVH
            try:
                pa = a.bvh(lv)
            except vg.VGError:
                with pytest.raises(vg.VGError):
                    b.bvh(lv)
                continue
            pb = b.bvh(lv)
            for k in ("prim", "offset", "nchild", "nodes", "boxes"):
                assert np.array_equal(pa[k], pb[k]), (lv, k)
        for s in range(ia["n_shapes"]):
            assert np.array_equal(np.array(a.shape_extent(s)), np.array(b.shape_extent(s)))
    with pytest.raises(vg.VGError):
        vg.Geometry.load(str(tmp_path / "missing.vgg"))
    bad = tmp_path / "bad.vgg"
    bad.write_bytes(b"not a geometry file at all")
    with pytest.raises(vg.VGError):
        vg.Geometry.load(str(bad))


def test_workspace_sizes_and_no_allocation_capacity():
    """Workspace sizes are host arithmetic (no GPU): the scheduled step's workspace grows by
    its parts (work-queue counter and relocation points, proposal slots, sort arrays), and
    the no-allocation entry point's fixed scratch (documented as 41.5 MiB) holds the
    workspace of its largest call, 2^20 tracks with every scheduling flag."""
    lib = vg.load_library()
    ws = lib.vg_nav_step_workspace_bytes
    n = 1 << 20
    align = lambda b: (b + 255) & ~255
    every = vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE | vg.NAV_LEARNED
    assert ws(n, vg.PREC_FP64) == 0 and ws(n, vg.PREC_MIXED) == 0
    assert ws(n, vg.PREC_MIXED | vg.NAV_QUEUE) == 256 + align(3 * 8 * n)
    assert ws(n, every) - ws(n, every & ~vg.NAV_LEARNED) == align(n)
    sort_only = ws(n, vg.NAV_SORT)
    assert ws(n, every) == 256 + align(3 * 8 * n) + align(n) + sort_only
    assert 4 * 4 * n < sort_only < 4 * 4 * n + 2 * 512 * 4 * (n // 4096 + 1) + 4096
    assert round(ws(n, every) / 2 ** 20, 1) == 41.5  # the size the header and noalloc.cu state
