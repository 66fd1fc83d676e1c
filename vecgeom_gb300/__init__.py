"""Python binding of libvecgeom_gb300 (ctypes over the C-ABI in include/vecgeom_gb300.h).

The names mirror the reference's API for the query path: a ``Geometry`` is assembled
with shape constructors, logical volumes and placements (UnplacedBox, LogicalVolume,
PlaceDaughter, GeoManager::SetWorldAndClose), after which its placed volumes answer the
SoA queries of VPlacedVolume (Inside, Contains, DistanceToIn/Out, SafetyToIn/Out) and the
BVH navigator answers LocatePoint and ComputeStepAndNextVolume, all on the GPU.

Query methods take CUDA tensors (torch is used only for device memory and streams) and
launch on torch's current stream. There is no CPU fallback: if the CUDA library is not
built, loading fails with an error that says so.
"""
import ctypes
import os

import numpy as np

__all__ = ["Geometry", "load_library", "NAVSTATE_DTYPE", "PREC_FP64", "PREC_MIXED", "NAV_SORT", "NAV_QUEUE",
           "NAV_LEARNED", "VGError",
           "kInside", "kSurface", "kOutside", "kInfLength", "IDENTITY_ROT", "ZERO_TRANS"]

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libvecgeom_gb300.so")

PREC_FP64 = 0
PREC_MIXED = 1
NAV_SORT = 2   # visit tracks sorted by (logical volume, Morton cell); results unchanged
NAV_QUEUE = 4  # persistent step kernel fed from a global work counter (with PREC_MIXED)
NAV_LEARNED = 8  # explore the BVH subtree proposed by the attached model first (with PREC_MIXED)
kInside, kSurface, kOutside = 1, 2, 3
kInfLength = np.finfo(np.float64).max
IDENTITY_ROT = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)
ZERO_TRANS = (0.0, 0.0, 0.0)

# vg_navstate / vecgeom::NavStateIndex {uint32 nav_ind; uint32 last_exited; bool on_boundary}
NAVSTATE_DTYPE = np.dtype([("nav_ind", "<u4"), ("last_exited", "<u4"), ("on_boundary", "u1"), ("pad", "u1", 3)])
assert NAVSTATE_DTYPE.itemsize == 12

SHAPE_BOX, SHAPE_TUBE, SHAPE_CONE, SHAPE_POLYCONE, SHAPE_POLYHEDRON, SHAPE_TORUS2, SHAPE_TRD, SHAPE_BOOLMINUS = range(1, 9)
SHAPE_TRAPEZOID = 9
SHAPE_CUT_TUBE = 10
SHAPE_SPHERE = 11
SHAPE_GENTRAP = 12
SHAPE_HYPE = 13


class VGError(RuntimeError):
    pass


_lib = None
_c_dp = ctypes.POINTER(ctypes.c_double)
_c_vp = ctypes.c_void_p

# name -> (restype, argtypes)
_SIGS = {
    "vg_last_error": (ctypes.c_char_p, []),
    "vg_version": (ctypes.c_char_p, []),
    "vg_geom_create": (ctypes.c_int, [ctypes.POINTER(_c_vp)]),
    "vg_geom_destroy": (None, [_c_vp]),
    "vg_geom_add_box": (ctypes.c_int32, [_c_vp] + [ctypes.c_double] * 3),
    "vg_geom_add_tube": (ctypes.c_int32, [_c_vp] + [ctypes.c_double] * 5),
    "vg_geom_add_cone": (ctypes.c_int32, [_c_vp] + [ctypes.c_double] * 7),
    "vg_geom_add_polycone": (ctypes.c_int32, [_c_vp, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                              _c_dp, _c_dp, _c_dp]),
    "vg_geom_add_polyhedron": (ctypes.c_int32, [_c_vp, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                                ctypes.c_int32, _c_dp, _c_dp, _c_dp]),
    "vg_geom_add_torus2": (ctypes.c_int32, [_c_vp] + [ctypes.c_double] * 5),
    "vg_geom_add_trd": (ctypes.c_int32, [_c_vp] + [ctypes.c_double] * 5),
    "vg_geom_add_trap": (ctypes.c_int32, [_c_vp] + [ctypes.c_double] * 11),
    "vg_geom_add_trap_corners": (ctypes.c_int32, [_c_vp, _c_dp]),
    "vg_geom_add_cut_tube": (ctypes.c_int32, [_c_vp] + [ctypes.c_double] * 11),
    "vg_geom_add_sphere": (ctypes.c_int32, [_c_vp] + [ctypes.c_double] * 6),
    "vg_geom_add_gentrap": (ctypes.c_int32, [_c_vp, _c_dp, _c_dp, ctypes.c_double]),
    "vg_geom_add_hype": (ctypes.c_int32, [_c_vp] + [ctypes.c_double] * 5),
    "vg_geom_add_trap_planes": (ctypes.c_int32, [_c_vp, ctypes.c_double, _c_dp]),
    "vg_geom_save": (ctypes.c_int, [_c_vp, ctypes.c_char_p]),
    "vg_geom_load": (ctypes.c_int, [_c_vp, ctypes.c_char_p]),
    "vg_geom_add_boolean_subtraction": (ctypes.c_int32, [_c_vp, ctypes.c_int32, ctypes.c_int32]),
    "vg_geom_add_logical_volume": (ctypes.c_int32, [_c_vp, ctypes.c_int32]),
    "vg_geom_place": (ctypes.c_int32, [_c_vp, ctypes.c_int32, _c_dp, _c_dp]),
    "vg_geom_place_daughter": (ctypes.c_int32, [_c_vp, ctypes.c_int32, ctypes.c_int32, _c_dp, _c_dp]),
    "vg_geom_set_world": (ctypes.c_int, [_c_vp, ctypes.c_int32]),
    "vg_geom_close": (ctypes.c_int, [_c_vp]),
    "vg_geom_build": (ctypes.c_int, [_c_vp]),
    "vg_geom_info": (ctypes.c_int, [_c_vp] + [ctypes.POINTER(ctypes.c_int32)] * 4 +
                     [ctypes.POINTER(ctypes.c_size_t)] * 2),
    "vg_geom_nav_table": (ctypes.c_int, [_c_vp, _c_vp, ctypes.c_size_t]),
    "vg_geom_bvh_sizes": (ctypes.c_int, [_c_vp, ctypes.c_int32] + [ctypes.POINTER(ctypes.c_int32)] * 3),
    "vg_geom_bvh_arrays": (ctypes.c_int, [_c_vp, ctypes.c_int32] + [_c_vp] * 5),
    "vg_geom_shape_extent": (ctypes.c_int, [_c_vp, ctypes.c_int32, _c_dp, _c_dp]),
    "vg_placed_inside": (ctypes.c_int, [_c_vp, ctypes.c_int32, _c_vp, _c_vp, _c_vp, ctypes.c_size_t, _c_vp,
                                        ctypes.c_uint32, _c_vp]),
    "vg_placed_contains": (ctypes.c_int, [_c_vp, ctypes.c_int32, _c_vp, _c_vp, _c_vp, ctypes.c_size_t, _c_vp,
                                          ctypes.c_uint32, _c_vp]),
    "vg_placed_distance_to_in": (ctypes.c_int, [_c_vp, ctypes.c_int32] + [_c_vp] * 7 +
                                 [ctypes.c_size_t, _c_vp, ctypes.c_uint32, _c_vp]),
    "vg_placed_distance_to_out": (ctypes.c_int, [_c_vp, ctypes.c_int32] + [_c_vp] * 7 +
                                  [ctypes.c_size_t, _c_vp, ctypes.c_uint32, _c_vp]),
    "vg_placed_safety_to_in": (ctypes.c_int, [_c_vp, ctypes.c_int32, _c_vp, _c_vp, _c_vp, ctypes.c_size_t, _c_vp,
                                              ctypes.c_uint32, _c_vp]),
    "vg_placed_safety_to_out": (ctypes.c_int, [_c_vp, ctypes.c_int32, _c_vp, _c_vp, _c_vp, ctypes.c_size_t,
                                               _c_vp, ctypes.c_uint32, _c_vp]),
    "vg_nav_locate_point": (ctypes.c_int, [_c_vp, _c_vp, _c_vp, _c_vp, ctypes.c_size_t, _c_vp, _c_vp]),
    "vg_nav_approach_next_daughter": (ctypes.c_int, [_c_vp] + [_c_vp] * 9 + [ctypes.c_size_t, _c_vp]),
    "vg_nav_compute_step_and_next_volume": (ctypes.c_int, [_c_vp] + [_c_vp] * 11 +
                                            [ctypes.c_size_t, ctypes.c_uint32, _c_vp]),
    "vg_nav_compute_step_and_next_volume_host": (ctypes.c_int, [_c_vp] + [_c_vp] * 11 +
                                                 [ctypes.c_size_t, ctypes.c_uint32, _c_vp]),
    "vg_nav_step_workspace_bytes": (ctypes.c_size_t, [ctypes.c_size_t, ctypes.c_uint32]),
    "vg_nav_compute_step_and_safety": (ctypes.c_int, [_c_vp] * 13 + [ctypes.c_size_t, ctypes.c_uint32, _c_vp]),
    "vg_nav_transport_workspace_bytes": (ctypes.c_size_t, [ctypes.c_size_t, ctypes.c_uint32]),
    "vg_nav_transport": (ctypes.c_int, [_c_vp] * 8 + [ctypes.c_size_t, ctypes.c_int32, ctypes.c_uint32, _c_vp, _c_vp,
                                                      _c_vp, _c_vp, ctypes.c_size_t, _c_vp, _c_vp, ctypes.c_size_t,
                                                      _c_vp]),
    "vg_nav_sort_tracks": (ctypes.c_int, [_c_vp] * 5 + [ctypes.c_size_t, _c_vp, _c_vp, _c_vp, ctypes.c_size_t,
                                                        _c_vp]),
    "vg_nav_sort_key_params": (ctypes.c_int, [_c_vp] * 5),
    "vg_nav_set_tuning": (ctypes.c_int, [_c_vp, ctypes.c_int32, ctypes.c_int32]),
    "vg_device_fp64_rate": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double), _c_vp]),
    "vg_mlp_create": (ctypes.c_int, [_c_vp, ctypes.c_uint64, ctypes.POINTER(_c_vp)]),
    "vg_mlp_destroy": (None, [_c_vp]),
    "vg_mlp_param_count": (ctypes.c_size_t, [_c_vp]),
    "vg_mlp_get_params": (ctypes.c_int, [_c_vp, _c_vp, ctypes.c_size_t]),
    "vg_mlp_set_params": (ctypes.c_int, [_c_vp, _c_vp, ctypes.c_size_t]),
    "vg_learn_features": (ctypes.c_int, [_c_vp] * 8 + [ctypes.c_size_t, _c_vp, _c_vp, _c_vp, _c_vp]),
    "vg_mlp_gradients": (ctypes.c_int, [_c_vp] * 4 + [ctypes.c_size_t, _c_vp, _c_vp, _c_vp]),
    "vg_mlp_train": (ctypes.c_int, [_c_vp] * 4 + [ctypes.c_size_t, ctypes.c_int32, ctypes.c_int32, ctypes.c_float,
                                                  ctypes.c_uint64, _c_vp, _c_vp]),
    "vg_mlp_infer": (ctypes.c_int, [_c_vp] * 3 + [ctypes.c_size_t, _c_vp, _c_vp, ctypes.c_uint32, _c_vp]),
    "vg_geom_set_proposer": (ctypes.c_int, [_c_vp, _c_vp]),
    "vg_nav_set_proposal_kernel": (ctypes.c_int, [_c_vp, ctypes.c_int32]),
    "vg_mlp_error": (ctypes.c_int, [_c_vp, _c_vp]),
    "vg_nav_propose": (ctypes.c_int, [_c_vp] * 8 + [ctypes.c_size_t, _c_vp, ctypes.c_uint32, _c_vp]),
    "vg_nav_compute_step_and_next_volume_noalloc": (ctypes.c_int, [_c_vp] + [_c_vp] * 11 +
                                                    [ctypes.c_size_t, ctypes.c_uint32, _c_vp]),
    "vg_nav_compute_step_and_next_volume_ws": (ctypes.c_int, [_c_vp] + [_c_vp] * 12 +
                                               [ctypes.c_size_t, ctypes.c_uint32, _c_vp, ctypes.c_size_t,
                                                _c_vp]),
}
# the unplaced (shape-frame) queries take the same arguments, with a shape id for the placed id
for _q in ("inside", "contains", "distance_to_in", "distance_to_out", "safety_to_in", "safety_to_out"):
    _SIGS["vg_shape_" + _q] = _SIGS["vg_placed_" + _q]


def load_library(path=None):
    """Load libvecgeom_gb300.so (built in-tree by ``__graft_entry__.build()``)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise VGError("libvecgeom_gb300.so is not built (%s); run `python -c \"import __graft_entry__ as g; "
                      "g.build()\"` first — there is no CPU fallback" % p)
    lib = ctypes.CDLL(p)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _check(rc, what):
    if rc < 0:
        msg = _lib.vg_last_error().decode()
        raise VGError("%s failed (%d): %s" % (what, rc, msg))
    return rc


def _darr(v, n=None):
    a = np.ascontiguousarray(np.asarray(v, dtype=np.float64))
    if n is not None:
        assert a.size == n, (a.size, n)
    return a, a.ctypes.data_as(_c_dp)


def _ptr(t):
    """Device pointer of a CUDA tensor (or None)."""
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous():
        raise VGError("query arrays must be contiguous CUDA tensors")
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def device_fp64_rate():
    """FP64 FMA instructions per second of the current CUDA device (a timed probe kernel):
    the peak for the navigation kernels' FP64 roofline."""
    load_library()
    r = ctypes.c_double()
    _check(_lib.vg_device_fp64_rate(ctypes.byref(r), _stream()), "vg_device_fp64_rate")
    return r.value


class Geometry:
    """A geometry handle: construction API + device queries (see module docstring)."""

    def __init__(self):
        load_library()
        h = ctypes.c_void_p()
        _check(_lib.vg_geom_create(ctypes.byref(h)), "vg_geom_create")
        self._h = h
        self.closed = False
        self.pv_lv = []  # logical volume of each placed volume, indexed by placed-volume id

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.vg_geom_destroy(self._h)
            self._h = None

    # ---------------------------------------------------------------- construction
    def add_box(self, dx, dy, dz):
        return _check(_lib.vg_geom_add_box(self._h, dx, dy, dz), "add_box")

    def add_tube(self, rmin, rmax, dz, sphi, dphi):
        return _check(_lib.vg_geom_add_tube(self._h, rmin, rmax, dz, sphi, dphi), "add_tube")

    def add_cone(self, rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi):
        return _check(_lib.vg_geom_add_cone(self._h, rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi), "add_cone")

    def add_polycone(self, sphi, dphi, z, rmin, rmax):
        n = len(z)
        za, zp = _darr(z, n)
        ra, rp = _darr(rmin, n)
        sa, sp = _darr(rmax, n)
        return _check(_lib.vg_geom_add_polycone(self._h, sphi, dphi, n, zp, rp, sp), "add_polycone")

    def add_polyhedron(self, phistart, phidelta, nsides, z, rmin, rmax):
        n = len(z)
        za, zp = _darr(z, n)
        ra, rp = _darr(rmin, n)
        sa, sp = _darr(rmax, n)
        return _check(_lib.vg_geom_add_polyhedron(self._h, phistart, phidelta, nsides, n, zp, rp, sp),
                      "add_polyhedron")

    def add_torus2(self, rmin, rmax, rtor, sphi, dphi):
        return _check(_lib.vg_geom_add_torus2(self._h, rmin, rmax, rtor, sphi, dphi), "add_torus2")

    def add_trd(self, dx1, dx2, dy1, dy2, dz):
        return _check(_lib.vg_geom_add_trd(self._h, dx1, dx2, dy1, dy2, dz), "add_trd")

    def add_trap(self, dz, theta, phi, dy1, dx1, dx2, alpha1, dy2, dx3, dx4, alpha2):
        """UnplacedTrapezoid(dz, theta, phi, dy1, dx1, dx2, alpha1, dy2, dx3, dx4, alpha2), angles
        in radians."""
        return _check(_lib.vg_geom_add_trap(self._h, dz, theta, phi, dy1, dx1, dx2, alpha1, dy2, dx3, dx4, alpha2),
                      "add_trap")

    def add_trap_corners(self, corners):
        """UnplacedTrapezoid(TrapCorners): eight (x, y, z) corners, (---) (+--) (-+-) (++-) (--+)
        (+-+) (-++) (+++)."""
        c = np.ascontiguousarray(np.asarray(corners, dtype=np.float64).reshape(24))
        return _check(_lib.vg_geom_add_trap_corners(self._h, c.ctypes.data_as(_c_dp)), "add_trap_corners")

    def add_sphere(self, rmin, rmax, sphi=0.0, dphi=2 * np.pi, stheta=0.0, dtheta=np.pi):
        """UnplacedSphere: a spherical shell section (angles in radians)."""
        return _check(_lib.vg_geom_add_sphere(self._h, rmin, rmax, sphi, dphi, stheta, dtheta), "add_sphere")

    def add_hype(self, rmin, rmax, stereo_in, stereo_out, dz):
        """UnplacedHype: radii at z = 0 of the inner and outer hyperboloids, their stereo
        angles (radians) and the half-length dz."""
        return _check(_lib.vg_geom_add_hype(self._h, rmin, rmax, stereo_in, stereo_out, dz), "add_hype")

    def add_gentrap(self, vertices_x, vertices_y, dz):
        """UnplacedGenTrap: x and y of the eight vertices (four at -dz, then four at +dz) and
        the half-length dz; faces planar or twisted."""
        vx = np.ascontiguousarray(np.asarray(vertices_x, dtype=np.float64).reshape(8))
        vy = np.ascontiguousarray(np.asarray(vertices_y, dtype=np.float64).reshape(8))
        return _check(_lib.vg_geom_add_gentrap(self._h, vx.ctypes.data_as(_c_dp), vy.ctypes.data_as(_c_dp), dz),
                      "add_gentrap")

    def add_cut_tube(self, rmin, rmax, dz, sphi, dphi, bottom_normal, top_normal):
        """UnplacedCutTube: a tube section between two cut planes through (0, 0, -dz) and
        (0, 0, dz) with the given outward normals (bottom z < 0, top z > 0)."""
        b, t = [float(v) for v in bottom_normal], [float(v) for v in top_normal]
        return _check(_lib.vg_geom_add_cut_tube(self._h, rmin, rmax, dz, sphi, dphi, *b, *t), "add_cut_tube")

    def add_trap_planes(self, dz, planes):
        """A trapezoid from dz and its four side planes (a, b, c, d), ordered -Y, +Y, -X, +X, as
        an existing UnplacedTrapezoid holds them."""
        c = np.ascontiguousarray(np.asarray(planes, dtype=np.float64).reshape(16))
        return _check(_lib.vg_geom_add_trap_planes(self._h, dz, c.ctypes.data_as(_c_dp)), "add_trap_planes")

    def add_boolean_subtraction(self, left_pv, right_pv):
        return _check(_lib.vg_geom_add_boolean_subtraction(self._h, left_pv, right_pv), "add_boolean_subtraction")

    def save(self, path):
        """Write the builder calls made so far (shapes, volumes, placements, world) to `path`."""
        _check(_lib.vg_geom_save(self._h, os.fsencode(path)), "vg_geom_save")

    @classmethod
    def load(cls, path):
        """A new, open geometry replaying the builder calls saved in `path` (close it to use it)."""
        g = cls()
        _check(_lib.vg_geom_load(g._h, os.fsencode(path)), "vg_geom_load")
        # the placed volumes' logical volumes, from the placements in the log
        log = np.fromfile(path, dtype=np.float64, offset=20)
        i = 0
        while i < len(log):
            op = int(log[i])
            if op == 1:
                i += 3 + int(log[i + 2])
            elif op == 3:
                g.pv_lv.append(int(log[i + 1]))
                i += 15
            else:
                i += 2
        return g

    def add_logical_volume(self, shape):
        return _check(_lib.vg_geom_add_logical_volume(self._h, shape), "add_logical_volume")

    def place(self, lv, trans=ZERO_TRANS, rot=IDENTITY_ROT):
        t, tp = _darr(trans, 3)
        r, rp = _darr(rot, 9)
        pv = _check(_lib.vg_geom_place(self._h, lv, tp, rp), "place")
        self.pv_lv.append(lv)
        return pv

    def place_daughter(self, mother_lv, lv, trans=ZERO_TRANS, rot=IDENTITY_ROT):
        t, tp = _darr(trans, 3)
        r, rp = _darr(rot, 9)
        pv = _check(_lib.vg_geom_place_daughter(self._h, mother_lv, lv, tp, rp), "place_daughter")
        self.pv_lv.append(lv)
        return pv

    def set_world(self, pv):
        _check(_lib.vg_geom_set_world(self._h, pv), "set_world")

    def build(self):
        """Host-side flattening only (BVHs, NavIndex table); needs no GPU."""
        _check(_lib.vg_geom_build(self._h), "build")

    def close(self):
        _check(_lib.vg_geom_close(self._h), "close")
        self.closed = True

    # ---------------------------------------------------------------- introspection
    def info(self):
        a, b, c, d = (ctypes.c_int32() for _ in range(4))
        e, f = ctypes.c_size_t(), ctypes.c_size_t()
        _check(_lib.vg_geom_info(self._h, *(ctypes.byref(v) for v in (a, b, c, d, e, f))), "info")
        return dict(n_shapes=a.value, n_lv=b.value, n_pv=c.value, max_depth=d.value, nav_words=e.value,
                    device_bytes=f.value)

    def nav_table(self):
        n = self.info()["nav_words"]
        out = np.zeros(n, dtype=np.uint32)
        _check(_lib.vg_geom_nav_table(self._h, out.ctypes.data_as(_c_vp), n), "nav_table")
        return out

    def bvh(self, lv):
        nn, npr, dep = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _check(_lib.vg_geom_bvh_sizes(self._h, lv, ctypes.byref(nn), ctypes.byref(npr), ctypes.byref(dep)),
               "bvh_sizes")
        prim = np.zeros(npr.value, np.int32)
        off = np.zeros(nn.value, np.int32)
        nch = np.zeros(nn.value, np.int32)
        nodes = np.zeros((nn.value, 6))
        boxes = np.zeros((npr.value, 6))
        _check(_lib.vg_geom_bvh_arrays(self._h, lv, *(a.ctypes.data_as(_c_vp) for a in (prim, off, nch, nodes, boxes))),
               "bvh_arrays")
        return dict(depth=dep.value, prim=prim, offset=off, nchild=nch, nodes=nodes, boxes=boxes)

    def shape_extent(self, shape):
        lo, lp = _darr(np.zeros(3))
        hi, hp = _darr(np.zeros(3))
        _check(_lib.vg_geom_shape_extent(self._h, shape, lp, hp), "shape_extent")
        return lo, hi

    # ---------------------------------------------------------------- SoA queries (CUDA tensors)
    def inside(self, pv, x, y, z, out, flags=PREC_FP64):
        _check(_lib.vg_placed_inside(self._h, pv, _ptr(x), _ptr(y), _ptr(z), x.numel(), _ptr(out), flags,
                                     _stream()), "vg_placed_inside")

    def contains(self, pv, x, y, z, out, flags=PREC_FP64):
        _check(_lib.vg_placed_contains(self._h, pv, _ptr(x), _ptr(y), _ptr(z), x.numel(), _ptr(out), flags,
                                       _stream()), "vg_placed_contains")

    def distance_to_in(self, pv, x, y, z, dx, dy, dz, out, step_max=None, flags=PREC_FP64):
        _check(_lib.vg_placed_distance_to_in(self._h, pv, _ptr(x), _ptr(y), _ptr(z), _ptr(dx), _ptr(dy), _ptr(dz),
                                             _ptr(step_max), x.numel(), _ptr(out), flags, _stream()),
               "vg_placed_distance_to_in")

    def distance_to_out(self, pv, x, y, z, dx, dy, dz, out, step_max=None, flags=PREC_FP64):
        _check(_lib.vg_placed_distance_to_out(self._h, pv, _ptr(x), _ptr(y), _ptr(z), _ptr(dx), _ptr(dy),
                                              _ptr(dz), _ptr(step_max), x.numel(), _ptr(out), flags, _stream()),
               "vg_placed_distance_to_out")

    def safety_to_in(self, pv, x, y, z, out, flags=PREC_FP64):
        _check(_lib.vg_placed_safety_to_in(self._h, pv, _ptr(x), _ptr(y), _ptr(z), x.numel(), _ptr(out), flags,
                                           _stream()), "vg_placed_safety_to_in")

    def safety_to_out(self, pv, x, y, z, out, flags=PREC_FP64):
        _check(_lib.vg_placed_safety_to_out(self._h, pv, _ptr(x), _ptr(y), _ptr(z), x.numel(), _ptr(out), flags,
                                            _stream()), "vg_placed_safety_to_out")

    # ---------------------------------------------------------------- unplaced queries (shape frame)
    def shape_query(self, q, shape, x, y, z, out, dx=None, dy=None, dz=None, flags=PREC_FP64):
        """One of the six queries on shape `shape` with points (and directions) in its own
        frame: q = "inside", "contains", "distance_to_in", "distance_to_out", "safety_to_in"
        or "safety_to_out" (VUnplacedVolume)."""
        fn = getattr(_lib, "vg_shape_" + q)
        if q.startswith("distance"):
            _check(fn(self._h, shape, _ptr(x), _ptr(y), _ptr(z), _ptr(dx), _ptr(dy), _ptr(dz), None, x.numel(),
                      _ptr(out), flags, _stream()), "vg_shape_" + q)
        else:
            _check(fn(self._h, shape, _ptr(x), _ptr(y), _ptr(z), x.numel(), _ptr(out), flags, _stream()),
                   "vg_shape_" + q)

    # ---------------------------------------------------------------- navigation (CUDA tensors)
    def locate_point(self, x, y, z, out_states):
        """GlobalLocator::LocateGlobalPoint(world, p, state, true); out_states: uint8 tensor (n*12)."""
        _check(_lib.vg_nav_locate_point(self._h, _ptr(x), _ptr(y), _ptr(z), x.numel(), _ptr(out_states),
                                        _stream()), "vg_nav_locate_point")

    def approach_next_daughter(self, x, y, z, dx, dy, dz, in_states, step, status=None):
        """BVH::ApproachNextDaughter per track in its state's volume (CUDA tensors): `step`
        (float64, in/out) is lowered to the distance at which the ray first reaches a
        daughter's bounding box."""
        _check(_lib.vg_nav_approach_next_daughter(self._h, _ptr(x), _ptr(y), _ptr(z), _ptr(dx), _ptr(dy), _ptr(dz),
                                                  _ptr(in_states), _ptr(step), _ptr(status), x.numel(), _stream()),
               "vg_nav_approach_next_daughter")

    def compute_step_and_next_volume(self, x, y, z, dx, dy, dz, in_states, out_states, step, step_limit=None,
                                     status=None, flags=PREC_FP64, workspace=None, nodes_visited=None):
        """One navigation step for n tracks (CUDA tensors). With NAV_SORT / NAV_QUEUE in
        `flags` a device workspace is needed: pass a uint8 CUDA tensor of at least
        step_workspace_bytes(n, flags) bytes, or leave it to the geometry, which keeps one
        cached workspace (calls running concurrently on different streams need their own)."""
        n = x.numel()
        if flags & (NAV_SORT | NAV_QUEUE | NAV_LEARNED) or nodes_visited is not None:
            need = int(_lib.vg_nav_step_workspace_bytes(n, flags))
            if workspace is None:
                ws = getattr(self, "_ws", None)
                if ws is None or ws.numel() < need or ws.device != x.device:
                    import torch
                    ws = torch.empty(max(need, 256), dtype=torch.uint8, device=x.device)
                    self._ws = ws
                workspace = ws
            _check(_lib.vg_nav_compute_step_and_next_volume_ws(
                self._h, _ptr(x), _ptr(y), _ptr(z), _ptr(dx), _ptr(dy), _ptr(dz), _ptr(step_limit),
                _ptr(in_states), _ptr(out_states), _ptr(step), _ptr(status), _ptr(nodes_visited), n, flags,
                _ptr(workspace), workspace.numel(), _stream()), "vg_nav_compute_step_and_next_volume_ws")
            return
        _check(_lib.vg_nav_compute_step_and_next_volume(
            self._h, _ptr(x), _ptr(y), _ptr(z), _ptr(dx), _ptr(dy), _ptr(dz), _ptr(step_limit), _ptr(in_states),
            _ptr(out_states), _ptr(step), _ptr(status), n, flags, _stream()),
            "vg_nav_compute_step_and_next_volume")

    def compute_step_and_next_volume_noalloc(self, x, y, z, dx, dy, dz, in_states, out_states, step,
                                             step_limit=None, status=None, flags=PREC_MIXED | NAV_SORT | NAV_QUEUE):
        """The scheduled step on the library's fixed device scratch (no allocation, at most
        2^20 tracks per call; overlapping calls race; the first call per device is setup)."""
        _check(_lib.vg_nav_compute_step_and_next_volume_noalloc(
            self._h, _ptr(x), _ptr(y), _ptr(z), _ptr(dx), _ptr(dy), _ptr(dz), _ptr(step_limit), _ptr(in_states),
            _ptr(out_states), _ptr(step), _ptr(status), x.numel(), flags, _stream()),
            "vg_nav_compute_step_and_next_volume_noalloc")

    def compute_step_and_safety(self, x, y, z, dx, dy, dz, in_states, out_states, step, safety, step_limit=None,
                                status=None, flags=PREC_FP64):
        """Step (as compute_step_and_next_volume) plus the FP64 safety of each input point."""
        _check(_lib.vg_nav_compute_step_and_safety(
            self._h, _ptr(x), _ptr(y), _ptr(z), _ptr(dx), _ptr(dy), _ptr(dz), _ptr(step_limit), _ptr(in_states),
            _ptr(out_states), _ptr(step), _ptr(safety), _ptr(status), x.numel(), flags, _stream()),
            "vg_nav_compute_step_and_safety")

    def transport(self, x, y, z, dx, dy, dz, states, max_steps=400, flags=PREC_FP64, trace_tracks=0):
        """Transport stream: steps every track until it leaves the world or makes max_steps
        steps. x, y, z and states (CUDA tensors) are updated in place. Returns (nsteps,
        status, iterations, trace_states, trace_steps); the traces hold the first
        `trace_tracks` tracks ([track, step] layout) or are None."""
        import torch
        n = x.numel()
        dev = x.device
        nsteps = torch.empty(n, dtype=torch.int32, device=dev)
        status = torch.empty(n, dtype=torch.int32, device=dev)
        tst = torch.zeros(max(trace_tracks, 0) * max_steps * 12, dtype=torch.uint8, device=dev) if trace_tracks else None
        tsp = torch.zeros(max(trace_tracks, 0) * max_steps, dtype=torch.float64, device=dev) if trace_tracks else None
        ws = torch.empty(max(int(_lib.vg_nav_transport_workspace_bytes(n, flags)), 256), dtype=torch.uint8, device=dev)
        it = ctypes.c_int32()
        _check(_lib.vg_nav_transport(self._h, _ptr(x), _ptr(y), _ptr(z), _ptr(dx), _ptr(dy), _ptr(dz), _ptr(states), n,
                                     max_steps, flags, _ptr(nsteps), _ptr(status), _ptr(tst), _ptr(tsp), trace_tracks,
                                     ctypes.byref(it), _ptr(ws), ws.numel(), _stream()), "vg_nav_transport")
        return nsteps, status, it.value, tst, tsp

    def sort_tracks(self, x, y, z, in_states, order, keys=None, workspace=None):
        """The visiting order NAV_SORT uses: `order` (int32/uint32 CUDA tensor of n) gets the
        track indices sorted stably by key; `keys` (optional) the sorted keys."""
        n = x.numel()
        need = int(_lib.vg_nav_step_workspace_bytes(n, NAV_SORT))
        if workspace is None:
            import torch
            workspace = torch.empty(max(need, 256), dtype=torch.uint8, device=x.device)
        _check(_lib.vg_nav_sort_tracks(self._h, _ptr(x), _ptr(y), _ptr(z), _ptr(in_states), n, _ptr(order),
                                       _ptr(keys), _ptr(workspace), workspace.numel(), _stream()),
               "vg_nav_sort_tracks")

    def sort_key_params(self):
        """(lo[3], scale[3], cell_bits, lv_bits) of the sort key of this closed geometry."""
        lo = (ctypes.c_float * 3)()
        sc = (ctypes.c_float * 3)()
        cb, lb = ctypes.c_int32(), ctypes.c_int32()
        _check(_lib.vg_nav_sort_key_params(self._h, lo, sc, ctypes.byref(cb), ctypes.byref(lb)),
               "vg_nav_sort_key_params")
        return tuple(lo), tuple(sc), cb.value, lb.value

    def set_tuning(self, cell_bits=0, queue_blocks_per_sm=0):
        """Sort-key Morton bits per axis and the work-queue kernel configuration (1: 256 x 1,
        2: 256 x 2, 3: 128 x 3, 4: 128 x 5 threads x blocks per SM; 5-8: the same budgets with the
        step split into a step kernel and a relocation kernel; 0: defaults). Results do not depend
        on them."""
        _check(_lib.vg_nav_set_tuning(self._h, cell_bits, queue_blocks_per_sm), "vg_nav_set_tuning")

    @staticmethod
    def step_workspace_bytes(n, flags):
        return int(_lib.vg_nav_step_workspace_bytes(n, flags))

    def compute_step_and_next_volume_host(self, x, y, z, dx, dy, dz, in_states, out_states, step, step_limit=None,
                                          status=None, flags=PREC_FP64, stream=None):
        """Host-array variant (numpy arrays or pinned CPU tensors): copies in, steps, copies out."""
        def hp(a):
            if a is None:
                return None
            if hasattr(a, "data_ptr"):
                return ctypes.c_void_p(a.data_ptr())
            return a.ctypes.data_as(_c_vp)
        _check(_lib.vg_nav_compute_step_and_next_volume_host(
            self._h, hp(x), hp(y), hp(z), hp(dx), hp(dy), hp(dz), hp(step_limit), hp(in_states), hp(out_states),
            hp(step), hp(status), len(x), flags, stream if stream is not None else _stream()),
            "vg_nav_compute_step_and_next_volume_host")
