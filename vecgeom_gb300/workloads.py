"""Seeded synthetic workloads: the shapes, geometries and track samples the benchmarks and
tests run on.

Every builder takes a ``geo`` object with the construction surface of
``vecgeom_gb300.Geometry`` (add_box, add_tube, ..., place_daughter, set_world, close) and
issues the same call sequence to it, so two implementations fed by the same builder get
identical placed-volume ids. Random numbers come from numpy's Philox generator keyed by
SplitMix64-derived sub-seeds; all arrays are FP64 and generated once on the host.
"""
import math

import numpy as np

MASK64 = (1 << 64) - 1
TWO_PI = 2.0 * math.pi


def splitmix64(x):
    """One SplitMix64 output for state x (the published constants of the generator)."""
    z = (x + 0x9E3779B97F4A7C15) & MASK64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


def rng(seed, stream=0):
    """Independent Philox stream `stream` of master seed `seed`."""
    return np.random.Generator(np.random.Philox(key=splitmix64((seed * 0x100000001B3 + stream) & MASK64)))


def isotropic(g, n):
    """Isotropic unit vectors: z = 2u - 1, phi = 2 pi v."""
    cz = 2.0 * g.random(n) - 1.0
    ph = TWO_PI * g.random(n)
    s = np.sqrt(np.maximum(0.0, 1.0 - cz * cz))
    return s * np.cos(ph), s * np.sin(ph), cz


def rot_z(phi):
    """Row-major rotation about z by phi (p_master = R p_local)."""
    c, s = math.cos(phi), math.sin(phi)
    return (c, -s, 0.0, s, c, 0.0, 0.0, 0.0, 1.0)


IDENT = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)

# ---------------------------------------------------------------------- shape catalogue
# Config 1: plain FP64 shape queries (Box, full-phi Tube, Cone), 2^20 points each.
SHAPES_CFG1 = {
    "box": ("box", (10.0, 20.0, 30.0)),
    "tube": ("tube", (10.0, 20.0, 30.0, 0.0, TWO_PI)),
    "cone": ("cone", (5.0, 10.0, 8.0, 15.0, 25.0, 0.0, TWO_PI)),
}


def _polycone_cfg2(seed=0x5EED):
    """12 z-planes evenly in [-500, 500]; rmin in [50,120], rmax in [150,400] from a seeded
    monotone random walk (increasing with z)."""
    g = rng(seed, 17)
    z = np.linspace(-500.0, 500.0, 12)
    rmin = np.sort(50.0 + 70.0 * g.random(12))
    rmax = np.sort(150.0 + 250.0 * g.random(12))
    return (0.0, TWO_PI, tuple(z), tuple(rmin), tuple(rmax))


def _polyhedron_cfg2():
    """8 sides, 6 z-planes, full phi; the z/r values chosen here are recorded with the
    benchmark output."""
    z = (-300.0, -200.0, -100.0, 100.0, 200.0, 300.0)
    rmin = (50.0, 60.0, 70.0, 70.0, 60.0, 50.0)
    rmax = (150.0, 180.0, 200.0, 200.0, 180.0, 150.0)
    return (0.0, TWO_PI, 8, z, rmin, rmax)


SHAPES_CFG2 = {
    "tube_phi": ("tube", (10.0, 20.0, 30.0, 0.3, 1.8)),
    "polycone": ("polycone", _polycone_cfg2()),
    "polyhedron": ("polyhedron", _polyhedron_cfg2()),
    "torus2": ("torus2", (5.0, 15.0, 100.0, 0.0, TWO_PI)),
    "trd": ("trd", (30.0, 10.0, 40.0, 15.0, 60.0)),
    # Box(5,5,5) minus Tube(0.5,2,2,0,2pi) placed at (-2.5,0,0): the reference's own benchmark
    # pair (test/benchmark/BoxMinusHollowTubeBenchmark_virtual.cpp:22-31).
    "box_minus_tube": ("boolminus", None),
}


def add_shape(geo, kind, params):
    """Create one shape on `geo`; returns the shape id (boolean operands placed first)."""
    if kind == "boolminus":
        lb = geo.add_logical_volume(geo.add_box(5.0, 5.0, 5.0))
        lt = geo.add_logical_volume(geo.add_tube(0.5, 2.0, 2.0, 0.0, TWO_PI))
        left = geo.place(lb)
        right = geo.place(lt, (-2.5, 0.0, 0.0), IDENT)
        return geo.add_boolean_subtraction(left, right)
    return getattr(geo, "add_" + kind)(*params)


def build_single_shape(geo, kind, params):
    """One shape placed with the identity transformation: returns (shape id, placed id)."""
    s = add_shape(geo, kind, params)
    pv = geo.place(geo.add_logical_volume(s))
    geo.close()
    return s, pv


def shape_points_box(lo, hi, n, seed, scale=1.2):
    """Points uniform in the extent box scaled `scale` about its centre, isotropic directions."""
    g = rng(seed, 1)
    lo, hi = np.asarray(lo), np.asarray(hi)
    c, h = 0.5 * (lo + hi), 0.5 * (hi - lo) * scale
    pts = [c[k] + h[k] * (2.0 * g.random(n) - 1.0) for k in range(3)]
    d = isotropic(rng(seed, 2), n)
    return tuple(pts), d


# ---------------------------------------------------------------------- navigation geometries
def barrel_layers(nlayers, r0, r1, n0, n1):
    radii = np.linspace(r0, r1, nlayers)
    counts = np.round(np.linspace(n0, n1, nlayers)).astype(int)
    return radii, counts


MODULE_HALF = (1.0, 10.0, 50.0)   # 2 x 20 x 100 mm module, thin along the radius
SENSOR_HALF = (0.5, 9.0, 49.0)
TANGENTIAL_PITCH = 22.0
Z_PITCH = 104.0


def _place_barrel_layer(geo, world_lv, module_lv, r, n, g, jitter):
    """One layer: a Tube holding n phi-rotated modules arranged in z-rings; returns the pv."""
    per_ring = max(1, int(math.floor(TWO_PI * r / TANGENTIAL_PITCH)))
    rings = int(math.ceil(n / per_ring))
    halfz = 0.5 * rings * Z_PITCH + 4.0
    rmin = r - MODULE_HALF[0] - jitter - 1.0
    rout = r + MODULE_HALF[0] + jitter + 1.0
    rmax = math.sqrt(rout * rout + (MODULE_HALF[1] + 1.0) ** 2) + 1.0
    layer_lv = geo.add_logical_volume(geo.add_tube(rmin, rmax, halfz, 0.0, TWO_PI))
    placed = 0
    for ring in range(rings):
        m = min(per_ring, n - placed)
        zc = -0.5 * rings * Z_PITCH + (ring + 0.5) * Z_PITCH
        for k in range(m):
            phi = TWO_PI * k / per_ring + (0.5 * TWO_PI / per_ring) * (ring & 1)
            dr, dz = jitter * (2.0 * g.random(2) - 1.0)
            rr = r + dr
            t = (rr * math.cos(phi), rr * math.sin(phi), zc + dz)
            geo.place_daughter(layer_lv, module_lv, t, rot_z(phi))
        placed += m
    return geo.place_daughter(world_lv, layer_lv)


def build_barrel(geo, seed=0xBA44E1, nlayers=10, r0=50.0, r1=1200.0, n0=64, n1=640, jitter=1.0, close=True):
    """Config 3 barrel: world box 2000 x 2000 x 3000 mm half-lengths, 10 tube layers
    (r 50..1200 mm) holding 64..640 phi-rotated 2x20x100 mm box modules with +-1 mm seeded
    radial/z jitter, each module holding one sensor box (nesting depth 4). Modules are laid
    out in 104 mm z-rings at 22 mm tangential pitch, so no two volumes overlap."""
    g = rng(seed, 3)
    world_lv = geo.add_logical_volume(geo.add_box(2000.0, 2000.0, 3000.0))
    sensor_lv = geo.add_logical_volume(geo.add_box(*SENSOR_HALF))
    module_lv = geo.add_logical_volume(geo.add_box(*MODULE_HALF))
    geo.place_daughter(module_lv, sensor_lv)
    radii, counts = barrel_layers(nlayers, r0, r1, n0, n1)
    for r, n in zip(radii, counts):
        _place_barrel_layer(geo, world_lv, module_lv, float(r), int(n), g, jitter)
    world = geo.place(world_lv)
    geo.set_world(world)
    if close:
        geo.close()
    return world


def build_detector(geo, seed=0xDE7EC7, nlayers=20, total_modules=150000, wedges_per_side=2000, ndisks=12,
                   close=True):
    """Config 4 detector: a 20-layer barrel totalling `total_modules` box modules (counts
    proportional to radius, r 100..1150 mm) plus two endcaps of `ndisks` Polycone holders
    (8 z-planes each) carrying `wedges_per_side` Trd wedges per side."""
    g = rng(seed, 4)
    world_lv = geo.add_logical_volume(geo.add_box(2000.0, 2000.0, 3000.0))
    sensor_lv = geo.add_logical_volume(geo.add_box(*SENSOR_HALF))
    module_lv = geo.add_logical_volume(geo.add_box(*MODULE_HALF))
    geo.place_daughter(module_lv, sensor_lv)
    radii = np.linspace(100.0, 1150.0, nlayers)
    counts = np.floor(total_modules * radii / radii.sum()).astype(int)
    counts[-1] += total_modules - counts.sum()
    for r, n in zip(radii, counts):
        _place_barrel_layer(geo, world_lv, module_lv, float(r), int(n), g, 1.0)
    # endcaps: Polycone holders (an annulus r 290..1100 with a stepped outer profile) with
    # Trd wedges pointing radially (local z -> radial, local y -> global z).
    zs = (-20.0, -15.0, -10.0, -5.0, 5.0, 10.0, 15.0, 20.0)
    rmins = (290.0,) * 8
    rmaxs = (1100.0, 1105.0, 1110.0, 1110.0, 1110.0, 1110.0, 1105.0, 1100.0)
    holder_lv = geo.add_logical_volume(geo.add_polycone(0.0, TWO_PI, zs, rmins, rmaxs))
    per_disk = int(math.ceil(wedges_per_side / ndisks))
    dphi = TWO_PI / per_disk
    rin, rout = 310.0, 1080.0
    dx1 = 0.45 * rin * dphi
    dx2 = 0.45 * rout * dphi
    wedge_lv = geo.add_logical_volume(geo.add_trd(dx1, dx2, 5.0, 5.0, 0.5 * (rout - rin)))
    rc = 0.5 * (rin + rout)
    for k in range(per_disk):
        phi = k * dphi
        c, s = math.cos(phi), math.sin(phi)
        rot = (-s, 0.0, c, c, 0.0, s, 0.0, 1.0, 0.0)
        geo.place_daughter(holder_lv, wedge_lv, (rc * c, rc * s, 0.0), rot)
    for side in (-1.0, 1.0):
        for d in range(ndisks):
            z = side * (2300.0 + 55.0 * d)
            geo.place_daughter(world_lv, holder_lv, (0.0, 0.0, z))
    world = geo.place(world_lv)
    geo.set_world(world)
    if close:
        geo.close()
    return world


def trap_corners(dz, theta, phi, dy1, dx1, dx2, alpha1, dy2, dx3, dx4, alpha2):
    """The eight corners of UnplacedTrapezoid(dz, theta, phi, ...) (UnplacedTrapezoid.cpp:447-466),
    shape (8, 3), in the order (---) (+--) (-+-) (++-) (--+) (+-+) (-++) (+++)."""
    t1, t2 = math.tan(alpha1) * dy1, math.tan(alpha2) * dy2
    xz, yz = math.tan(theta) * math.cos(phi) * dz, math.tan(theta) * math.sin(phi) * dz
    c = []
    for z, xc, yc, dy, a, dxm, dxp in ((-dz, -xz, -yz, dy1, t1, dx1, dx2), (dz, xz, yz, dy2, t2, dx3, dx4)):
        c += [(xc - a - dxm, yc - dy, z), (xc - a + dxm, yc - dy, z), (xc + a - dxp, yc + dy, z),
              (xc + a + dxp, yc + dy, z)]
    return np.array(c)


TRAP_WEDGE = (60.0, 0.1, 0.4, 40.0, 20.0, 30.0, 0.15, 50.0, 25.0, 35.0, 0.15)


def build_trap_ring(geo, n_phi=16, radius=300.0, z_rings=(-120.0, 0.0, 120.0), close=True):
    """Rings of general trapezoids (tilted by theta/phi, sheared by alpha) pointing radially,
    each holding a half-size trapezoid made from its corners, in a 1.2 m box: a calorimeter-like
    test geometry for the trapezoid kernels inside the navigator."""
    world_lv = geo.add_logical_volume(geo.add_box(600.0, 600.0, 400.0))
    wedge_lv = geo.add_logical_volume(geo.add_trap(*TRAP_WEDGE))
    inner_lv = geo.add_logical_volume(geo.add_trap_corners(0.5 * trap_corners(*TRAP_WEDGE)))
    geo.place_daughter(wedge_lv, inner_lv)
    for z in z_rings:
        for j in range(n_phi):
            ph = TWO_PI * j / n_phi
            c, s = math.cos(ph), math.sin(ph)
            # local x -> tangential, local y -> global z, local z -> radial
            rot = (-s, 0.0, c, c, 0.0, s, 0.0, 1.0, 0.0)
            geo.place_daughter(world_lv, wedge_lv, (radius * c, radius * s, z), rot)
    world = geo.place(world_lv)
    geo.set_world(world)
    if close:
        geo.close()
    return world


def build_sphere_shells(geo, close=True):
    """Spherical shells in a 1.2 m box: a hollow shell cut to a band of polar angles around
    the equator holding a ring of boxes, a polar cap (theta 0 to 0.5 rad) and its opposite
    cap (theta beyond pi - 0.6 rad) each holding a smaller full sphere, and a phi sector of
    a hemisphere (theta up to pi / 2, phi 0.2 to 2.4 rad). Tests the sphere kernels (phi
    wedge and theta cone in every regime) inside the navigator."""
    world_lv = geo.add_logical_volume(geo.add_box(600.0, 600.0, 600.0))
    band_lv = geo.add_logical_volume(geo.add_sphere(300.0, 380.0, 0.0, TWO_PI, 1.2, 0.74))
    tile_lv = geo.add_logical_volume(geo.add_box(10.0, 10.0, 10.0))
    for j in range(16):
        ph = TWO_PI * (j + 0.5) / 16
        geo.place_daughter(band_lv, tile_lv, (340.0 * math.cos(ph), 340.0 * math.sin(ph), 0.0), rot_z(ph))
    geo.place_daughter(world_lv, band_lv)
    cap_lv = geo.add_logical_volume(geo.add_sphere(150.0, 280.0, 0.0, TWO_PI, 0.0, 0.5))
    ball_lv = geo.add_logical_volume(geo.add_sphere(0.0, 25.0))
    geo.place_daughter(cap_lv, ball_lv, (0.0, 0.0, 220.0))
    geo.place_daughter(world_lv, cap_lv)
    low_lv = geo.add_logical_volume(geo.add_sphere(0.0, 280.0, 0.0, TWO_PI, math.pi - 0.6, 0.6))
    geo.place_daughter(low_lv, ball_lv, (0.0, 0.0, -200.0))
    geo.place_daughter(world_lv, low_lv)
    sector_lv = geo.add_logical_volume(geo.add_sphere(30.0, 120.0, 0.2, 2.2, 0.0, 0.5 * math.pi))
    geo.place_daughter(world_lv, sector_lv, (0.0, 0.0, 10.0))
    world = geo.place(world_lv)
    geo.set_world(world)
    if close:
        geo.close()
    return world


def build_cut_tube_ring(geo, n_phi=12, radius=300.0, close=True):
    """Cut tubes in a 1.2 m box: a ring of hollow pipes along z with tilted end cuts, each
    holding a box in its wall, rotated about z to face the centre; a phi-section cut tube
    in the middle. Tests the cut tube kernels inside the navigator."""
    world_lv = geo.add_logical_volume(geo.add_box(600.0, 600.0, 400.0))
    pipe_lv = geo.add_logical_volume(geo.add_cut_tube(20.0, 40.0, 150.0, 0.0, TWO_PI, (0.0, -0.3, -1.0),
                                                      (0.2, 0.0, 1.0)))
    bar_lv = geo.add_logical_volume(geo.add_box(5.0, 5.0, 40.0))
    geo.place_daughter(pipe_lv, bar_lv, (30.0, 0.0, 0.0))
    for j in range(n_phi):
        ph = TWO_PI * j / n_phi
        geo.place_daughter(world_lv, pipe_lv, (radius * math.cos(ph), radius * math.sin(ph), 0.0), rot_z(ph))
    mid_lv = geo.add_logical_volume(geo.add_cut_tube(50.0, 100.0, 80.0, 0.3, 2.0, (0.1, 0.1, -1.0),
                                                     (-0.2, 0.05, 1.0)))
    geo.place_daughter(world_lv, mid_lv)
    world = geo.place(world_lv)
    geo.set_world(world)
    if close:
        geo.close()
    return world


# GenTrap vertex sets (x of the eight vertices, y of the eight, half-length): four at -dz,
# then four at +dz.
GENTRAPS = {
    # planar faces (a trapezoid-like box tapering in x and y), clockwise
    "planar": ([-40.0, -40.0, 40.0, 40.0, -30.0, -30.0, 30.0, 30.0],
               [-20.0, 20.0, 20.0, -20.0, -15.0, 15.0, 15.0, -15.0], 100.0),
    # the top square turned against the bottom one: all four faces twisted
    "twisted": ([-30.0, -30.0, 30.0, 30.0, -25.0, -35.0, 25.0, 35.0],
                [-30.0, 30.0, 30.0, -30.0, -35.0, 25.0, 35.0, -25.0], 80.0),
    # one twisted face and three planar ones (the unit test's trap2 shape scaled by 10)
    "one_twisted": ([-30.0, -30.0, 30.0, 30.0, -20.0, -20.0, 20.0, 20.0],
                    [-30.0, 30.0, 30.0, -30.0, -19.0, 20.0, 20.0, -20.0], 50.0),
    # triangular bases: edge 1 collapsed on both (a degenerated face)
    "triangle": ([-20.0, 0.0, 0.0, 20.0, -10.0, 0.0, 0.0, 10.0],
                 [-20.0, 25.0, 25.0, -20.0, -10.0, 12.0, 12.0, -10.0], 50.0),
    # the top collapsed to a point (a pyramid)
    "pyramid": ([-25.0, -25.0, 25.0, 25.0, 0.0, 0.0, 0.0, 0.0],
                [-25.0, 25.0, 25.0, -25.0, 0.0, 0.0, 0.0, 0.0], 40.0),
    # given anticlockwise: the constructor reorders it
    "anticlockwise": ([-35.0, 35.0, 35.0, -35.0, -30.0, 30.0, 30.0, -30.0],
                      [-35.0, -35.0, 35.0, 35.0, -25.0, -25.0, 25.0, 25.0], 30.0),
}


def build_gentrap_ring(geo, close=True):
    """Generic trapezoids in a 1.2 m box: a ring of eight twisted cells (r = 300 mm), six
    planar cells (r = 150 mm) each holding a box, a triangular-base cell above the centre, a
    pyramid below it, a one-twisted-face cell and an anticlockwise-given cell at the centre.
    Tests the GenTrap kernels (planar and twisted faces, degenerated edges) inside the
    navigator."""
    world_lv = geo.add_logical_volume(geo.add_box(600.0, 600.0, 400.0))
    lv = {k: geo.add_logical_volume(geo.add_gentrap(*v)) for k, v in GENTRAPS.items()}
    bar_lv = geo.add_logical_volume(geo.add_box(10.0, 5.0, 40.0))
    geo.place_daughter(lv["planar"], bar_lv)
    for j in range(8):
        ph = TWO_PI * (j + 0.5) / 8
        geo.place_daughter(world_lv, lv["twisted"], (300.0 * math.cos(ph), 300.0 * math.sin(ph), 0.0), rot_z(ph))
    for j in range(6):
        ph = TWO_PI * j / 6
        geo.place_daughter(world_lv, lv["planar"], (150.0 * math.cos(ph), 150.0 * math.sin(ph), 0.0), rot_z(ph))
    geo.place_daughter(world_lv, lv["triangle"], (0.0, 0.0, 200.0))
    geo.place_daughter(world_lv, lv["pyramid"], (0.0, 0.0, -200.0))
    geo.place_daughter(world_lv, lv["one_twisted"], (0.0, 0.0, 90.0))
    geo.place_daughter(world_lv, lv["anticlockwise"], (0.0, 0.0, -40.0))
    world = geo.place(world_lv)
    geo.set_world(world)
    if close:
        geo.close()
    return world


# Hyperboloids (rmin, rmax, inner stereo angle, outer stereo angle, dz)
HYPES = {
    "hollow": (20.0, 40.0, 0.3, 0.5, 100.0),   # both surfaces hyperbolic
    "solid": (0.0, 30.0, 0.0, 0.7, 60.0),      # no inner surface
    "cylinder_in": (15.0, 35.0, 0.0, 0.4, 50.0),  # inner surface a cylinder
    "cone_in": (0.0, 40.0, 0.5, 0.6, 50.0),    # inner surface a double cone (rmin 0)
}


def build_hype_ring(geo, close=True):
    """Hyperboloids in a 1.2 m box: a ring of six hollow hyperboloids (r = 250 mm) each
    holding a box in its wall, and along the axis a solid one, one with a cylindrical inner
    surface and one whose inner surface is a double cone. Tests the Hype kernels inside the
    navigator."""
    world_lv = geo.add_logical_volume(geo.add_box(600.0, 600.0, 400.0))
    lv = {k: geo.add_logical_volume(geo.add_hype(*v)) for k, v in HYPES.items()}
    bar_lv = geo.add_logical_volume(geo.add_box(4.0, 4.0, 20.0))
    geo.place_daughter(lv["hollow"], bar_lv, (30.0, 0.0, 0.0))
    for j in range(6):
        ph = TWO_PI * (j + 0.5) / 6
        geo.place_daughter(world_lv, lv["hollow"], (250.0 * math.cos(ph), 250.0 * math.sin(ph), 0.0), rot_z(ph))
    geo.place_daughter(world_lv, lv["solid"], (0.0, 0.0, -150.0))
    geo.place_daughter(world_lv, lv["cylinder_in"])
    geo.place_daughter(world_lv, lv["cone_in"], (0.0, 0.0, 150.0))
    world = geo.place(world_lv)
    geo.set_world(world)
    if close:
        geo.close()
    return world


def tracks_in_cylinder(n, seed, rmax=30.0, halfz=500.0):
    """Config 3 track starts: uniform in the cylinder r < rmax, |z| < halfz, isotropic."""
    g = rng(seed, 5)
    r = rmax * np.sqrt(g.random(n))
    ph = TWO_PI * g.random(n)
    z = halfz * (2.0 * g.random(n) - 1.0)
    d = isotropic(rng(seed, 6), n)
    return (r * np.cos(ph), r * np.sin(ph), z), d


def primaries_eta_phi(n, seed, eta_max=3.0):
    """Config 5 primaries from the origin: pseudorapidity uniform in [-eta_max, eta_max],
    phi uniform."""
    g = rng(seed, 7)
    eta = eta_max * (2.0 * g.random(n) - 1.0)
    ph = TWO_PI * g.random(n)
    theta = 2.0 * np.arctan(np.exp(-eta))
    st = np.sin(theta)
    d = (st * np.cos(ph), st * np.sin(ph), np.cos(theta))
    z = np.zeros(n)
    return (z.copy(), z.copy(), z.copy()), d


def shape_points_mixed(lo, hi, n, seed, inside_fn, dist_out_fn, surface_band=1e-6):
    """Config-2 point mix for one shape: a third strictly inside, a third outside (uniform in
    the 1.2x extent box, classified with `inside_fn`), and a third within `surface_band` mm
    of the surface (an inside point moved along a random direction to where `dist_out_fn`
    puts the boundary, then offset by U(-band, band) along that direction). Directions are
    isotropic. `inside_fn(x, y, z)` and `dist_out_fn(x, y, z, dx, dy, dz)` evaluate the shape
    (on the GPU in the benchmark, on the CPU checker in tests)."""
    n3 = n // 3
    ins, outs = [], []
    it = 0
    while (sum(len(a[0]) for a in ins) < n - 2 * n3 + n3 or sum(len(a[0]) for a in outs) < n3) and it < 64:
        m = max(4 * n, 1024)
        (x, y, z), _ = shape_points_box(lo, hi, m, seed + 1000 * it)
        cls = np.asarray(inside_fn(x, y, z))
        ins.append((x[cls == 1], y[cls == 1], z[cls == 1]))
        outs.append((x[cls == 3], y[cls == 3], z[cls == 3]))
        it += 1
    ix, iy, iz = (np.concatenate([a[k] for a in ins]) for k in range(3))
    ox, oy, oz = (np.concatenate([a[k] for a in outs]) for k in range(3))
    n_in = n - 2 * n3
    g = rng(seed, 11)
    sx, sy, sz = ix[n_in:n_in + n3], iy[n_in:n_in + n3], iz[n_in:n_in + n3]
    sdx, sdy, sdz = isotropic(rng(seed, 12), len(sx))
    d = np.asarray(dist_out_fn(sx, sy, sz, sdx, sdy, sdz))
    d = np.where((d > 0) & (d < 1e30), d, 0.0) + surface_band * (2.0 * g.random(len(sx)) - 1.0)
    px = np.concatenate([ix[:n_in], ox[:n3], sx + d * sdx])
    py = np.concatenate([iy[:n_in], oy[:n3], sy + d * sdy])
    pz = np.concatenate([iz[:n_in], oz[:n3], sz + d * sdz])
    perm = rng(seed, 13).permutation(len(px))
    dirs = isotropic(rng(seed, 14), len(px))
    return (px[perm].copy(), py[perm].copy(), pz[perm].copy()), dirs


def stream_tracks(n, seed, restart_fraction=0.2, world_half=(2000.0, 2000.0, 3000.0)):
    """Config 5 track starts: primaries from the origin (pseudorapidity uniform in [-3, 3],
    phi uniform), except a seeded `restart_fraction` that start at a point drawn uniformly in
    the world box with an isotropic direction (tracks restarting inside random volumes)."""
    (x, y, z), (dx, dy, dz) = primaries_eta_phi(n, seed)
    g = rng(seed, 11)
    restart = g.random(n) < restart_fraction
    m = int(restart.sum())
    for arr, h in zip((x, y, z), world_half):
        arr[restart] = h * (2.0 * g.random(m) - 1.0)
    rd = isotropic(rng(seed, 12), m)
    for arr, v in zip((dx, dy, dz), rd):
        arr[restart] = v
    return (x, y, z), (dx, dy, dz), restart


def sample_transport_steps(geo, n_samples, seed, torch, device, n_primaries=1 << 20, max_steps=200, flags=0):
    """Realistic step inputs: straight primaries from the origin (config-5 distribution) are
    transported on the GPU with the FP64 navigator; every (point, direction, state) before
    a step is a candidate, and `n_samples` of them are drawn uniformly (seeded). Returns
    device tensors x, y, z, dx, dy, dz (FP64) and states (uint8, 12 B each)."""
    (x, y, z), (dx, dy, dz) = primaries_eta_phi(n_primaries, seed)
    t = [torch.from_numpy(a).to(device) for a in (x, y, z, dx, dy, dz)]
    st = torch.empty(n_primaries * 12, dtype=torch.uint8, device=device)
    geo.locate_point(t[0], t[1], t[2], st)
    out = torch.empty_like(st)
    step = torch.empty(n_primaries, dtype=torch.float64, device=device)
    pool = [[] for _ in range(7)]
    px, py, pz, ddx, ddy, ddz = t
    for _ in range(max_steps):
        nav = st.view(torch.int32).view(-1, 3)[:, 0]
        alive = nav != 0
        if not bool(alive.any()):
            break
        idx = alive.nonzero().squeeze(1)
        for k, a in enumerate((px, py, pz, ddx, ddy, ddz)):
            pool[k].append(a[idx])
        pool[6].append(st.view(-1, 12)[idx])
        geo.compute_step_and_next_volume(px, py, pz, ddx, ddy, ddz, st, out, step, flags=flags)
        m = alive.to(torch.float64)
        px = px + m * (step * ddx)
        py = py + m * (step * ddy)
        pz = pz + m * (step * ddz)
        st = torch.where(alive.unsqueeze(1), out.view(-1, 12), st.view(-1, 12)).reshape(-1).contiguous()
    cat = [torch.cat(p) for p in pool]
    total = cat[0].numel()
    gen = torch.Generator(device="cpu").manual_seed(seed & 0x7FFFFFFF)
    pick = torch.randperm(total, generator=gen)[:n_samples].to(device)
    res = [c[pick].contiguous() for c in cat[:6]]
    states = cat[6][pick].reshape(-1).contiguous()
    return res, states, total
