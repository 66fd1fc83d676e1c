"""ctypes wrapper of the oracle (TEST INFRASTRUCTURE ONLY — see ref_base.h).

Mirrors the construction methods of ``vecgeom_gb300.Geometry`` so that the same builder
function (vecgeom_gb300.workloads) produces identical geometries on both sides, and
exposes batched CPU queries on numpy arrays. Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg use it.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p
NAVSTATE_DTYPE = np.dtype([("nav_ind", "<u4"), ("last_exited", "<u4"), ("on_boundary", "u1"), ("pad", "u1", 3)])


_SIGNATURES = {
    "oracle_geom_create": (_vp, []),
    "oracle_geom_destroy": (None, [_vp]),
    "oracle_add_shape": (ctypes.c_int, [_vp, ctypes.c_int, _dp, ctypes.c_int]),
    "oracle_add_lv": (ctypes.c_int, [_vp, ctypes.c_int]),
    "oracle_place": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp]),
    "oracle_place_daughter": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp, _dp]),
    "oracle_set_world": (None, [_vp, ctypes.c_int]),
    "oracle_close": (ctypes.c_int, [_vp]),
    "oracle_shape_extent": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp]),
    "oracle_shape_normal": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp]),
    "oracle_gentrap_valid": (ctypes.c_int, [_dp, _dp, ctypes.c_double]),
    "oracle_placed_query": (ctypes.c_double, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_size_t] + [_vp] * 6 +
                            [ctypes.c_double, _vp, _vp, ctypes.c_int]),
    "oracle_nav_table_words": (ctypes.c_size_t, [_vp]),
    "oracle_nav_table": (None, [_vp, _vp]),
    "oracle_max_depth": (ctypes.c_int, [_vp]),
    "oracle_bvh_sizes": (ctypes.c_int, [_vp, ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 3),
    "oracle_bvh_arrays": (ctypes.c_int, [_vp, ctypes.c_int] + [_vp] * 5),
    "oracle_nav_locate": (ctypes.c_double, [_vp, ctypes.c_size_t, _vp, _vp, _vp, _vp, ctypes.c_int]),
    "oracle_nav_step": (ctypes.c_double, [_vp, ctypes.c_size_t] + [_vp] * 11 + [ctypes.c_int]),
    "oracle_nav_step_safety": (ctypes.c_double, [_vp, ctypes.c_size_t] + [_vp] * 11 + [ctypes.c_int]),
    "oracle_shape_query": (ctypes.c_double, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_size_t] + [_vp] * 6 +
                           [ctypes.c_double, _vp, _vp, ctypes.c_int]),
    "oracle_nav_approach": (ctypes.c_double, [_vp, ctypes.c_size_t] + [_vp] * 8 + [ctypes.c_int]),
    "oracle_nav_transport": (ctypes.c_double, [_vp, ctypes.c_size_t] + [_vp] * 7 +
                             [ctypes.c_int, _vp, _vp, _vp, _vp, ctypes.c_int]),
    "oracle_nav_step_simple": (ctypes.c_double, [_vp, ctypes.c_size_t] + [_vp] * 10 + [ctypes.c_int]),
    "oracle_nav_locate_simple": (ctypes.c_double, [_vp, ctypes.c_size_t, _vp, _vp, _vp, _vp, ctypes.c_int]),
    "oracle_nav_crosscheck": (ctypes.c_double, [_vp, ctypes.c_size_t] + [_vp] * 6 +
                              [ctypes.c_int, _vp, ctypes.c_int]),
    "oracle_check_nav_index": (ctypes.c_int, [_vp, _vp, ctypes.c_size_t, _vp]),
}


def bind(lib, required=True):
    """Set the ctypes signatures of the oracle's extern "C" surface on `lib`; with
    required=False, functions `lib` does not export are skipped."""
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            if required:
                raise AttributeError(name)
            continue
        fn.restype = res
        fn.argtypes = args
    return lib


def load():
    global _lib
    if _lib is None:
        path = _build.LIB if os.path.exists(_build.LIB) else _build.build()
        _lib = bind(ctypes.CDLL(path))
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_vp)


def _d(v):
    a = np.ascontiguousarray(np.asarray(v, dtype=np.float64))
    return a, a.ctypes.data_as(_dp)


class OracleGeometry:
    """Same construction surface as vecgeom_gb300.Geometry, evaluated on the CPU."""

    def __init__(self):
        self._lib = load()
        self._h = self._lib.oracle_geom_create()

    def __del__(self):
        if getattr(self, "_h", None) and getattr(self, "_lib", None) is not None:
            self._lib.oracle_geom_destroy(self._h)
            self._h = None

    def _shape(self, t, params):
        a, p = _d(params)
        r = self._lib.oracle_add_shape(self._h, t, p, a.size)
        if r < 0:
            raise RuntimeError("oracle: unsupported shape type %d" % t)
        return r

    def add_box(self, dx, dy, dz):
        return self._shape(1, [dx, dy, dz])

    def add_tube(self, rmin, rmax, dz, sphi, dphi):
        return self._shape(2, [rmin, rmax, dz, sphi, dphi])

    def add_cone(self, rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi):
        return self._shape(3, [rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi])

    def add_polycone(self, sphi, dphi, z, rmin, rmax):
        return self._shape(4, [sphi, dphi, len(z), *z, *rmin, *rmax])

    def add_polyhedron(self, phistart, phidelta, nsides, z, rmin, rmax):
        return self._shape(5, [phistart, phidelta, nsides, len(z), *z, *rmin, *rmax])

    def add_torus2(self, rmin, rmax, rtor, sphi, dphi):
        return self._shape(6, [rmin, rmax, rtor, sphi, dphi])

    def add_trd(self, dx1, dx2, dy1, dy2, dz):
        return self._shape(7, [dx1, dx2, dy1, dy2, dz])

    def add_boolean_subtraction(self, left_pv, right_pv):
        return self._shape(8, [left_pv, right_pv])

    def add_sphere(self, rmin, rmax, sphi=0.0, dphi=2 * np.pi, stheta=0.0, dtheta=np.pi):
        return self._shape(12, [rmin, rmax, sphi, dphi, stheta, dtheta])

    def add_hype(self, rmin, rmax, stereo_in, stereo_out, dz):
        """Hype (UnplacedHype): inner and outer radius at z = 0, inner and outer stereo angles
        (radians) and the half-length dz."""
        return self._shape(14, [rmin, rmax, stereo_in, stereo_out, dz])

    def add_gentrap(self, vertices_x, vertices_y, dz):
        """GenTrap (UnplacedGenTrap): x and y of the eight vertices (four at -dz, then four
        at +dz) and the half-length dz."""
        return self._shape(13, [*vertices_x, *vertices_y, dz])

    @staticmethod
    def gentrap_valid(vertices_x, vertices_y, dz):
        """Whether the reference's GenTrapStruct::Initialize accepts these vertices."""
        ax, px = _d(vertices_x)
        ay, py = _d(vertices_y)
        return bool(load().oracle_gentrap_valid(px, py, dz))

    def shape_normal(self, shape, p):
        """VUnplacedVolume::Normal at p (shape frame): (normal, valid)."""
        n = np.zeros(3)
        a, pp = _d(p)
        ok = self._lib.oracle_shape_normal(self._h, shape, pp, n.ctypes.data_as(_dp))
        return n, bool(ok)

    def add_cut_tube(self, rmin, rmax, dz, sphi, dphi, bottom_normal, top_normal):
        return self._shape(11, [rmin, rmax, dz, sphi, dphi, *bottom_normal, *top_normal])

    def add_boolean_union(self, left_pv, right_pv):
        """Union of two placed volumes (oracle only: the product has no union)."""
        return self._shape(10, [left_pv, right_pv])

    def add_trap(self, dz, theta, phi, dy1, dx1, dx2, alpha1, dy2, dx3, dx4, alpha2):
        return self._shape(9, [dz, theta, phi, dy1, dx1, dx2, alpha1, dy2, dx3, dx4, alpha2])

    def add_trap_planes(self, dz, planes):
        return self._shape(9, [dz] + list(np.asarray(planes, dtype=np.float64).reshape(16)))

    def add_trap_corners(self, corners):
        c = np.asarray(corners, dtype=np.float64).reshape(24)
        return self._shape(9, list(c))

    def add_logical_volume(self, shape):
        return self._lib.oracle_add_lv(self._h, shape)

    def place(self, lv, trans=(0.0, 0.0, 0.0), rot=(1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0)):
        t, tp = _d(trans)
        r, rp = _d(rot)
        return self._lib.oracle_place(self._h, lv, tp, rp)

    def place_daughter(self, mother_lv, lv, trans=(0.0, 0.0, 0.0), rot=(1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0)):
        t, tp = _d(trans)
        r, rp = _d(rot)
        return self._lib.oracle_place_daughter(self._h, mother_lv, lv, tp, rp)

    def set_world(self, pv):
        self._lib.oracle_set_world(self._h, pv)

    def close(self):
        if self._lib.oracle_close(self._h) != 0:
            raise RuntimeError("oracle close failed")

    def shape_extent(self, shape):
        lo, lp = _d(np.zeros(3))
        hi, hp = _d(np.zeros(3))
        self._lib.oracle_shape_extent(self._h, shape, lp, hp)
        return lo, hi

    # ------------------------------------------------------------ queries (numpy, CPU)
    def query(self, pv, q, x, y, z, dx=None, dy=None, dz=None, step_max=np.finfo(np.float64).max, nthreads=1):
        """q: 0 Inside, 1 Contains, 2 DistanceToIn, 3 DistanceToOut, 4 SafetyToIn, 5 SafetyToOut,
        6 PlacedDistanceToOut (DistanceToOut of a point and direction in the mother's frame)."""
        n = len(x)
        outd = np.empty(n, np.float64)
        outi = np.empty(n, np.int32)
        t = self._lib.oracle_placed_query(self._h, pv, q, n, _p(x), _p(y), _p(z), _p(dx), _p(dy), _p(dz), step_max,
                                     _p(outd), _p(outi), nthreads)
        return (outi if q in (0, 1) else outd), t

    def shape_query(self, shape, q, x, y, z, dx=None, dy=None, dz=None, step_max=np.finfo(np.float64).max,
                    nthreads=1):
        """The query q (as in query()) on an unplaced shape, points in its own frame."""
        n = len(x)
        outd = np.empty(n, np.float64)
        outi = np.empty(n, np.int32)
        self._lib.oracle_shape_query(self._h, shape, q, n, _p(x), _p(y), _p(z), _p(dx), _p(dy), _p(dz), step_max,
                                _p(outd), _p(outi), nthreads)
        return outi if q in (0, 1) else outd

    def nav_table(self):
        n = self._lib.oracle_nav_table_words(self._h)
        out = np.zeros(n, np.uint32)
        self._lib.oracle_nav_table(self._h, _p(out))
        return out

    def max_depth(self):
        return self._lib.oracle_max_depth(self._h)

    def bvh(self, lv):
        nn, npr, dep = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        if self._lib.oracle_bvh_sizes(self._h, lv, ctypes.byref(nn), ctypes.byref(npr), ctypes.byref(dep)) != 0:
            return None
        prim = np.zeros(npr.value, np.int32)
        off = np.zeros(nn.value, np.int32)
        nch = np.zeros(nn.value, np.int32)
        nodes = np.zeros((nn.value, 6))
        boxes = np.zeros((npr.value, 6))
        self._lib.oracle_bvh_arrays(self._h, lv, _p(prim), _p(off), _p(nch), _p(nodes), _p(boxes))
        return dict(depth=dep.value, prim=prim, offset=off, nchild=nch, nodes=nodes, boxes=boxes)

    def locate(self, x, y, z, nthreads=1, navigator="bvh"):
        """GlobalLocator::LocateGlobalPoint from the world with BVHLevelLocator, or with
        navigator="simple" the brute-force SimpleLevelLocator."""
        out = np.zeros(len(x), NAVSTATE_DTYPE)
        fn = self._lib.oracle_nav_locate_simple if navigator == "simple" else self._lib.oracle_nav_locate
        t = fn(self._h, len(x), _p(x), _p(y), _p(z), _p(out), nthreads)
        return out, t

    def step(self, x, y, z, dx, dy, dz, states, step_limit=None, nthreads=1, count_nodes=False, navigator="bvh"):
        """One ComputeStepAndPropagatedState per track with BVHNavigator, or with
        navigator="simple" the brute-force NewSimpleNavigator (+ SimpleLevelLocator)."""
        n = len(x)
        if step_limit is None:
            step_limit = np.full(n, np.finfo(np.float64).max)
        out = np.zeros(n, NAVSTATE_DTYPE)
        step = np.zeros(n)
        if navigator == "simple":
            t = self._lib.oracle_nav_step_simple(self._h, n, _p(x), _p(y), _p(z), _p(dx), _p(dy), _p(dz), _p(step_limit),
                                            _p(states), _p(out), _p(step), nthreads)
            return out, step, None, t
        nv = np.zeros(n, np.int32) if count_nodes else None
        t = self._lib.oracle_nav_step(self._h, n, _p(x), _p(y), _p(z), _p(dx), _p(dy), _p(dz), _p(step_limit),
                                 _p(states), _p(out), _p(step), _p(nv), nthreads)
        return out, step, nv, t

    def crosscheck(self, x, y, z, dx, dy, dz, max_steps=1000, nthreads=1):
        """The reference's TestVGDMLNavigation loop: every track stepped to the world's edge by
        the BVH navigator, each step compared with the brute-force navigator's from the same
        state. Returns counts: steps, not_nearly_equal, bit_different, state_different,
        start_state_different."""
        c = np.zeros(5, np.int64)
        self._lib.oracle_nav_crosscheck(self._h, len(x), _p(x), _p(y), _p(z), _p(dx), _p(dy), _p(dz), max_steps, _p(c),
                                   nthreads)
        return dict(zip(("steps", "not_nearly_equal", "bit_different", "state_different",
                         "start_state_different"), (int(v) for v in c)))

    def check_nav_index(self, table=None):
        """test/benchmark/TestNavIndex.cpp's checks of a NavIndex table (this geometry's own
        when `table` is None) over every placed-volume path: (error code, paths visited)."""
        paths = np.zeros(1, np.int64)
        if table is None:
            err = self._lib.oracle_check_nav_index(self._h, None, 0, _p(paths))
        else:
            tab = np.ascontiguousarray(table, dtype=np.uint32)
            err = self._lib.oracle_check_nav_index(self._h, _p(tab), tab.size, _p(paths))
        return int(err), int(paths[0])

    def step_safety(self, x, y, z, dx, dy, dz, states, step_limit=None, nthreads=1):
        n = len(x)
        if step_limit is None:
            step_limit = np.full(n, np.finfo(np.float64).max)
        out = np.zeros(n, NAVSTATE_DTYPE)
        step = np.zeros(n)
        saf = np.zeros(n)
        t = self._lib.oracle_nav_step_safety(self._h, n, _p(x), _p(y), _p(z), _p(dx), _p(dy), _p(dz), _p(step_limit),
                                        _p(states), _p(out), _p(step), _p(saf), nthreads)
        return out, step, saf, t

    def approach_next_daughter(self, x, y, z, dx, dy, dz, states, step, nthreads=1):
        """BVH::ApproachNextDaughter per track; returns the new step array (a copy of `step`
        lowered to the first daughter bounding box the ray reaches)."""
        out = np.array(step, dtype=np.float64, copy=True)
        self._lib.oracle_nav_approach(self._h, len(x), _p(x), _p(y), _p(z), _p(dx), _p(dy), _p(dz), _p(states), _p(out),
                                 nthreads)
        return out

    def transport(self, x, y, z, dx, dy, dz, states, max_steps, trace=False, nthreads=1):
        n = len(x)
        nsteps = np.zeros(n, np.int32)
        final = np.zeros(n, NAVSTATE_DTYPE)
        tr = np.zeros((n, max_steps), np.uint32) if trace else None
        trs = np.zeros((n, max_steps)) if trace else None
        t = self._lib.oracle_nav_transport(self._h, n, _p(x), _p(y), _p(z), _p(dx), _p(dy), _p(dz), _p(states),
                                      max_steps, _p(nsteps), _p(final), _p(tr), _p(trs), nthreads)
        return nsteps, final, tr, trs, t


def transport_step_sample(o, n_samples, seed, n_primaries, max_steps=200, nthreads=1, first=None):
    """The step inputs of vecgeom_gb300.workloads.sample_transport_steps reproduced on the
    CPU: the same primaries transported by the oracle's FP64 navigator (positions advanced as
    p + step * d), every pre-step (point, direction, state) of the alive tracks pooled in the
    same order, and the same seeded uniform draw (torch.randperm on a CPU generator) of
    `n_samples` of them. The GPU's FP64 step equals the oracle's bit for bit, so the result
    is the GPU sample itself; `first` keeps only that many leading samples. Two transport
    passes: the first counts the pool, the second gathers the drawn entries. Returns
    ([x, y, z, dx, dy, dz], states, pool size)."""
    import torch

    from vecgeom_gb300 import workloads as W
    (x0, y0, z0), (dx, dy, dz) = W.primaries_eta_phi(n_primaries, seed)

    def transport(visit):
        x, y, z = x0.copy(), y0.copy(), z0.copy()
        st, _ = o.locate(x, y, z, nthreads=nthreads)
        for it in range(max_steps):
            idx = np.flatnonzero(st["nav_ind"] != 0)
            if idx.size == 0:
                break
            a = [np.ascontiguousarray(v[idx]) for v in (x, y, z, dx, dy, dz)]
            sa = np.ascontiguousarray(st[idx])
            visit(it, a, sa)
            out, step, _, _ = o.step(*a, sa, nthreads=nthreads)
            x[idx] = a[0] + step * a[3]
            y[idx] = a[1] + step * a[4]
            z[idx] = a[2] + step * a[5]
            st[idx] = out

    counts = []
    transport(lambda it, a, sa: counts.append(len(sa)))
    total = int(sum(counts))
    gen = torch.Generator(device="cpu").manual_seed(seed & 0x7FFFFFFF)
    pick = torch.randperm(total, generator=gen)[:n_samples].numpy()
    if first is not None:
        pick = pick[:first]
    starts = np.concatenate([[0], np.cumsum(counts)])
    cols = [np.empty(len(pick)) for _ in range(6)]
    states = np.zeros(len(pick), NAVSTATE_DTYPE)
    order = np.argsort(pick, kind="stable")
    sorted_pick = pick[order]

    def gather(it, a, sa):
        lo, hi = np.searchsorted(sorted_pick, [starts[it], starts[it + 1]])
        if hi > lo:
            rows = order[lo:hi]
            local = sorted_pick[lo:hi] - starts[it]
            for k in range(6):
                cols[k][rows] = a[k][local]
            states[rows] = sa[local]

    transport(gather)
    return cols, states, total
