"""GDML reader: a GDML file (or string) into a geometry of this package, following the
reference's Xerces middleware (persistency/gdml/source/src/Middleware.cpp) node by node, so
that shapes, logical volumes and placed volumes are created in the same order and with the
same values as `vgdml::Frontend::Load` creates them:

* nodes are processed in document order (Middleware.cpp:165-213): `constant`, `position`,
  `rotation`, `scale` definitions, solids, `volume` (with its `physvol` children) and
  `world`; material nodes and `userinfo` are skipped (they are not on the query path);
* a numeric attribute is the leading number of its text as `std::stod` reads it, or else
  the value of the constant of that name, 0 when there is none (Middleware.cpp:141-150,
  Helper.cpp:58-68); lengths are multiplied by the node's `lunit` (`unit` on a position),
  angles by its `aunit` (`unit` on a rotation) (Middleware.cpp:665-695);
* full lengths of box, tube, cone, trd and trap are halved (DECLAREHALF);
* a placement's rotation (x, y, z angles) becomes the matrix of
  makeRotationMatrixFromCartesianAngles (Middleware.cpp:111-129) in a Transformation3D
  with the position as translation (Middleware.cpp:1305-1388);
* `subtraction` places its first solid at the identity and its second with the given
  position and rotation, then builds the boolean from the two (Middleware.cpp:415-499);
* `world` places its logical volume, sets it as the world and closes the geometry
  (Middleware.cpp:1446-1465).

Supported solids are the shapes this package implements: box, tube, cone, polycone,
polyhedra, torus, trd, trap and subtraction. Any other solid, a scaled (reflected)
placement, union or intersection raises GDMLError naming it. The reader drives the
geometry only through its builder methods (add_box, add_logical_volume, place_daughter,
...), so it builds a `vecgeom_gb300.Geometry` and the CPU oracle's geometry alike.
"""
import math
import re
import xml.etree.ElementTree as ET

SOLID_TAGS = {
    "multiUnion", "reflectedSolid", "scaledSolid", "union", "subtraction", "intersection", "box", "twistedbox",
    "twistedtrap", "twistedtrd", "paraboloid", "sphere", "ellipsoid", "tube", "twistedtubs", "cutTube", "cone",
    "elcone", "polycone", "genericPolycone", "para", "trd", "trap", "torus", "orb", "polyhedra", "genericPolyhedra",
    "xtru", "hype", "eltube", "tet", "arb8", "tessellated",
}
_LEN_UNIT = {"mm": 1.0, "m": 1e3, "km": 1e6, "um": 1e-3, "nm": 1e-6, "cm": 10.0}
_NUM = re.compile(r"\s*([+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan))", re.I)
_INT = re.compile(r"\s*([+-]?\d+)")


class GDMLError(RuntimeError):
    pass


def rotation_from_angles(x, y, z):
    """Row-major rotation matrix of GDML x, y, z rotation angles (radians), as the reference
    forms it (Middleware.cpp:111-129)."""
    s1, c1 = -math.sin(x), math.cos(x)
    s2, c2 = -math.sin(y), math.cos(y)
    s3, c3 = -math.sin(z), math.cos(z)
    return (c2 * c3, -c2 * s3, s2,
            c1 * s3 + c3 * s1 * s2, c1 * c3 - s1 * s2 * s3, -c2 * s1,
            s1 * s3 - c1 * c3 * s2, c3 * s1 + c1 * s2 * s3, c1 * c2)


class GDMLGeometry:
    """What a load produced: the world placed-volume id and the name -> id maps."""

    def __init__(self):
        self.world = None
        self.solids = {}
        self.volumes = {}
        self.constants = {}
        self.positions = {}
        self.rotations = {}
        self.scales = {}


class _Reader:
    def __init__(self, geo, close):
        self.geo = geo
        self.close = close
        self.out = GDMLGeometry()

    # ------------------------------------------------------------------ attributes
    def _double(self, node, name):
        s = node.get(name, "")
        m = _NUM.match(s)
        if m:
            return float(m.group(1))
        return self.out.constants.setdefault(s, 0.0)

    @staticmethod
    def _int(node, name):
        s = node.get(name, "")
        if not s:
            return 0
        m = _INT.match(s)
        if not m:
            raise GDMLError("bad integer attribute %s=%r" % (name, s))
        return int(m.group(1))

    @staticmethod
    def _lmul(node):
        tag = "unit" if node.tag == "position" else ("auxunit" if node.tag == "auxiliary" else "lunit")
        return _LEN_UNIT.get(node.get(tag, ""), 1.0)

    @staticmethod
    def _amul(node):
        tag = "unit" if node.tag == "rotation" else "aunit"
        return math.pi / 180.0 if node.get(tag, "") == "deg" else 1.0

    def _len(self, node, name, mul):
        return mul * self._double(node, name)

    # ------------------------------------------------------------------ nodes
    def node(self, n):
        tag = n.tag
        if tag in SOLID_TAGS:
            return self.solid(n)
        if tag == "constant":
            name = n.get("name", "")
            m = _NUM.match(n.get("value", ""))
            return self._insert(self.out.constants, name, float(m.group(1)) if m else math.nan, "constant")
        if tag == "position":
            return self.position(n)
        if tag == "rotation":
            return self.rotation(n)
        if tag == "scale":
            v = tuple(self._double(n, k) for k in "xyz")
            return self._insert(self.out.scales, n.get("name", ""), v, "scale")
        if tag in ("isotope", "element", "material", "userinfo"):
            return True
        if tag == "volume":
            return self.volume(n)
        if tag == "world":
            return self.world(n)
        ok = True
        for c in n:
            ok = self.node(c) and ok
        return ok

    @staticmethod
    def _insert(table, name, value, what):
        if name in table:
            raise GDMLError("%s %r defined twice" % (what, name))
        table[name] = value
        return True

    def position(self, n):
        mul = self._lmul(n)
        v = tuple(self._len(n, k, mul) for k in "xyz")
        return self._insert(self.out.positions, n.get("name", ""), v, "position")

    def rotation(self, n):
        mul = self._amul(n)
        v = tuple(mul * self._double(n, k) for k in "xyz")
        return self._insert(self.out.rotations, n.get("name", ""), v, "rotation")

    def solid(self, n):
        tag, g = n.tag, self.geo
        L, A = self._lmul(n), self._amul(n)
        ln = lambda k: self._len(n, k, L)
        an = lambda k: A * self._double(n, k)
        if tag == "box":
            s = g.add_box(ln("x") / 2.0, ln("y") / 2.0, ln("z") / 2.0)
        elif tag == "tube":
            s = g.add_tube(ln("rmin"), ln("rmax"), ln("z") / 2.0, an("startphi"), an("deltaphi"))
        elif tag == "cone":
            s = g.add_cone(ln("rmin1"), ln("rmax1"), ln("rmin2"), ln("rmax2"), ln("z") / 2.0, an("startphi"),
                           an("deltaphi"))
        elif tag in ("polycone", "polyhedra"):
            sphi, dphi = an("startphi"), an("deltaphi")
            z, rmin, rmax = [], [], []
            for c in n:
                if isinstance(c.tag, str):
                    rmax.append(self._len(c, "rmax", L))
                    rmin.append(self._len(c, "rmin", L))
                    z.append(self._len(c, "z", L))
            if tag == "polycone":
                s = g.add_polycone(sphi, dphi, z, rmin, rmax)
            else:
                s = g.add_polyhedron(sphi, dphi, self._int(n, "numsides"), z, rmin, rmax)
        elif tag == "sphere":
            s = g.add_sphere(ln("rmin"), ln("rmax"), an("startphi"), an("deltaphi"), an("starttheta"),
                             an("deltatheta"))
        elif tag == "cutTube":
            # Middleware::processCutTube: the normals' components are read as lengths
            s = g.add_cut_tube(ln("rmin"), ln("rmax"), ln("z") / 2.0, an("startphi"), an("deltaphi"),
                               (ln("lowX"), ln("lowY"), ln("lowZ")), (ln("highX"), ln("highY"), ln("highZ")))
        elif tag == "hype":
            # Middleware::processHype: the stereo angles are read without the angle unit
            # (DECLAREANDGETPLAINVAR), z is the full length
            s = g.add_hype(ln("rmin"), ln("rmax"), self._double(n, "inst"), self._double(n, "outst"), ln("z") / 2.0)
        elif tag == "arb8":
            # Middleware::processGenTrap: the vertex coordinates are read without the length
            # unit (DECLAREANDGETPLAINVAR), dz with it; dz is the half-length
            vx = [self._double(n, "v%dx" % k) for k in range(1, 9)]
            vy = [self._double(n, "v%dy" % k) for k in range(1, 9)]
            s = g.add_gentrap(vx, vy, ln("dz"))
        elif tag == "torus":
            s = g.add_torus2(ln("rmin"), ln("rmax"), ln("rtor"), an("startphi"), an("deltaphi"))
        elif tag == "trd":
            s = g.add_trd(ln("x1") / 2.0, ln("x2") / 2.0, ln("y1") / 2.0, ln("y2") / 2.0, ln("z") / 2.0)
        elif tag == "trap":
            s = g.add_trap(ln("z") / 2.0, an("theta"), an("phi"), ln("y1") / 2.0, ln("x1") / 2.0, ln("x2") / 2.0,
                           an("alpha1"), ln("y2") / 2.0, ln("x3") / 2.0, ln("x4") / 2.0, an("alpha2"))
        elif tag == "subtraction":
            s = self.subtraction(n)
        else:
            raise GDMLError("unsupported solid <%s> %r" % (tag, n.get("name", "")))
        return self._insert(self.out.solids, n.get("name", ""), s, "solid")

    def _solid_ref(self, c):
        name = c.get("ref", "")
        if name not in self.out.solids:
            raise GDMLError("unknown solid %r" % name)
        return self.out.solids[name]

    def subtraction(self, n):
        first = second = None
        pos, rot = (0.0, 0.0, 0.0), (0.0, 0.0, 0.0)
        for c in n:
            if c.tag == "first":
                first = self._solid_ref(c)
            elif c.tag == "second":
                second = self._solid_ref(c)
            elif c.tag == "positionref":
                pos = self.out.positions.setdefault(c.get("ref", ""), (0.0, 0.0, 0.0))
            elif c.tag == "rotationref":
                rot = self.out.rotations.setdefault(c.get("ref", ""), (0.0, 0.0, 0.0))
            elif c.tag == "position":
                mul = self._lmul(c)
                pos = tuple(self._len(c, k, mul) for k in "xyz")
            elif c.tag == "rotation":
                mul = self._amul(c)
                rot = tuple(mul * self._double(c, k) for k in "xyz")
        if first is None or second is None:
            raise GDMLError("subtraction %r without both operands" % n.get("name", ""))
        g = self.geo
        lf, ls = g.add_logical_volume(first), g.add_logical_volume(second)
        left = g.place(lf)
        right = g.place(ls, pos, rotation_from_angles(*rot))
        return g.add_boolean_subtraction(left, right)

    def volume(self, n):
        name = n.get("name", "")
        lv = None
        for c in n:
            if c.tag == "solidref":
                lv = self.geo.add_logical_volume(self._solid_ref(c))
                self.out.volumes.setdefault(name, lv)
            elif c.tag == "physvol":
                if lv is None:
                    raise GDMLError("physvol before the solidref of volume %r" % name)
                self.physvol(c, lv)
        if lv is None:
            raise GDMLError("volume %r has no solid" % name)
        return True

    def physvol(self, n, mother):
        lv = None
        pos, rot, scale = (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
        for c in n:
            if c.tag == "volumeref":
                ref = c.get("ref", "")
                if ref not in self.out.volumes:
                    raise GDMLError("unknown volume %r" % ref)
                lv = self.out.volumes[ref]
            elif c.tag == "position":
                self.position(c)
                pos = self.out.positions[c.get("name", "")]
            elif c.tag == "rotation":
                self.rotation(c)
                rot = self.out.rotations[c.get("name", "")]
            elif c.tag == "scale":
                self.node(c)
                scale = self.out.scales[c.get("name", "")]
            elif c.tag == "scaleref":
                scale = self.out.scales.setdefault(c.get("ref", ""), (0.0, 0.0, 0.0))
            elif c.tag == "positionref":
                pos = self.out.positions.setdefault(c.get("ref", ""), (0.0, 0.0, 0.0))
            elif c.tag == "rotationref":
                rot = self.out.rotations.setdefault(c.get("ref", ""), (0.0, 0.0, 0.0))
            elif isinstance(c.tag, str):
                raise GDMLError("unknown physvol child <%s>" % c.tag)
        if lv is None:
            raise GDMLError("physvol %r without volumeref" % n.get("name", ""))
        if scale != (1.0, 1.0, 1.0):
            raise GDMLError("scaled (reflected) placement %r is not supported" % n.get("name", ""))
        self.geo.place_daughter(mother, lv, pos, rotation_from_angles(*rot))

    def world(self, n):
        ref = n.get("ref", "")
        if ref not in self.out.volumes:
            raise GDMLError("unknown world volume %r" % ref)
        pv = self.geo.place(self.out.volumes[ref])
        self.geo.set_world(pv)
        if self.close:
            self.geo.close()
        self.out.world = pv
        return True


def load(source, geo, close=True):
    """Build the GDML geometry `source` (a path, or the document text when it starts with
    '<') on `geo`; returns a GDMLGeometry. `close=False` leaves the geometry open."""
    if source.lstrip().startswith("<"):
        text = source
    else:
        with open(source, encoding="utf-8") as f:
            text = f.read()
    root = ET.fromstring(text)
    r = _Reader(geo, close)
    r.node(root)
    if r.out.world is None:
        raise GDMLError("no <world> in the setup")
    return r.out
