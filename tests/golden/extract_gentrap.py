"""Extract the known answers of VecGeom's generic-trapezoid unit test into a JSON fixture.

Reads test/unit_tests/TestGenTrap.cpp of a VecGeom source tree AS TEXT (nothing of it is
compiled or run) and replays its straight-line statements with a small interpreter of the
forms the file uses: vertex arrays, SimpleGenTrap constructions, Vec_t points (with +, -,
scalar *, Mag, Normalize, Set), scalar assignments, the loop that shoots at the eight
vertices, Normal / Inside / DistanceToIn / DistanceToOut / SafetyToIn / SafetyToOut /
Extent calls and the asserts on their results. Each assert becomes one case:

    shape, query, point, direction, comparison (==, <, <=, ApproxEqual) and expected value

A point the test builds along the shape's own surface normal (testp = p + t * normal after
trap.Normal(p, normal)) is recorded as {"at": p, "scale": t} and resolved at test time with
the oracle's Normal, as the test resolves it with the shape's. The capacity and surface-area
asserts are not on the query path, and the loop over SamplePointOnSurface draws points from
the reference's random generator, which cannot be replayed; both are listed as skipped (the
surface-shooting property is tested with seeded points of this repository instead).

Usage: python tests/golden/extract_gentrap.py <VecGeom source tree> [out dir]
       (or set VECGEOM_SOURCE_DIR). Writes tests/golden/unit_GenTrap.json.
"""
import json
import math
import os
import re
import sys

DBL_MAX = sys.float_info.max
QUERIES = ("Inside", "Contains", "DistanceToIn", "DistanceToOut", "SafetyToIn", "SafetyToOut")
INSIDE = {"kInside": 1, "kSurface": 2, "kOutside": 3}


class V:
    """Vector3D<double> with the operations the test uses, in IEEE double."""

    def __init__(self, x, y, z):
        self.v = [float(x), float(y), float(z)]

    def __add__(self, o):
        if isinstance(o, AlongNormal):
            return o.offset(self, 1.0)
        return V(*(a + b for a, b in zip(self.v, o.v)))

    def __sub__(self, o):
        if isinstance(o, AlongNormal):
            return o.offset(self, -1.0)
        return V(*(a - b for a, b in zip(self.v, o.v)))

    def __rmul__(self, s):
        return V(*(s * a for a in self.v))

    def __neg__(self):
        return V(*(-a for a in self.v))

    def Mag(self):
        x, y, z = self.v
        return math.sqrt(x * x + y * y + z * z)

    def Normalize(self):  # Vector3D.h:198: *this *= 1 / Length()
        s = 1.0 / self.Mag()
        self.v = [a * s for a in self.v]

    def Set(self, x, y, z):
        self.v = [float(x), float(y), float(z)]


class NormalRef:
    """The `normal` a trap.Normal(p, normal) call filled in, known only to the shape."""

    def __init__(self, shape, at):
        self.shape, self.at = shape, at

    def __rmul__(self, s):
        return AlongNormal(self, s)


class AlongNormal:
    def __init__(self, ref, scale):
        self.ref, self.scale = ref, scale

    def offset(self, base, sign):
        return PointAlongNormal(self.ref.shape, self.ref.at, base, sign * self.scale)


class PointAlongNormal:
    def __init__(self, shape, at, base, scale):
        self.shape, self.at, self.base, self.scale = shape, at, base, scale


def strip_comments(src):
    src = re.sub(r"/\*.*?\*/", lambda m: "\n" * m.group(0).count("\n"), src, flags=re.S)
    return "\n".join(line.split("//")[0] for line in src.split("\n"))


def split_args(s):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
            continue
        depth += ch in "({["
        depth -= ch in ")}]"
        cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


class Interp:
    def __init__(self):
        self.env = {"kInfLength": DBL_MAX, "true": True, "false": False}
        self.shapes, self.cases, self.skipped = {}, [], []
        self.pending = None  # (shape, query, p, d) of the last Dist = ... call
        self.line = 0

    # -------------------------------------------------------------- expressions
    def ev(self, e):
        e = e.strip()
        e = re.sub(r"std::(cos|sin|atan2|sqrt)", r"math.\1", e)
        e = re.sub(r"\bVec_t\(", "V(", e)
        e = re.sub(r"(\d)\.(?!\d)", r"\1.0", e)
        m = re.fullmatch(r"\((.+?)\)\s*\?\s*(.+?)\s*:\s*(.+)", e)
        if m:
            e = "(%s if %s else %s)" % (m.group(2), m.group(1), m.group(3))
        e = re.sub(r"(\w+)\[(\w+)\]", r"\1[\2]", e)
        return eval(e, {"math": math, "V": V}, self.env)

    def point(self, e):
        v = self.ev(e)
        if isinstance(v, PointAlongNormal):
            return None, {"shape": v.shape, "at": v.at.v, "base": v.base.v, "scale": v.scale}
        return list(v.v), None

    # -------------------------------------------------------------- statements
    def call(self, shape, method, args):
        a = split_args(args)
        p, along = self.point(a[0])
        d = list(self.ev(a[1]).v) if len(a) > 1 else None
        return (shape, method, p, along, d)

    def record(self, query, kind, expected, shape=None, p=None, along=None, d=None):
        c = {"shape": shape, "query": query, "p": p, "d": d, "kind": kind, "expected": expected,
             "line": self.line, "soft": False}
        if along is not None:
            c["along_normal"] = along
        self.cases.append(c)

    def statement(self, s):
        s = s.strip()
        if not s or s.startswith(("using ", "bool valid", "Precision vol",
                                  "Precision surf", "Precision Dist,", "Precision testValue")):
            if s.startswith("Precision testValue"):
                self.env["testValue"] = self.ev(s.split("=", 1)[1])
            return
        m = re.fullmatch(r"Precision (\w+)\[8\]\s*=\s*\{(.*)\}", s, flags=re.S)
        if m:
            self.env[m.group(1)] = [float(self.ev(x)) for x in split_args(m.group(2))]
            return
        m = re.fullmatch(r"SimpleGenTrap (\w+)\(\"[^\"]*\",\s*(\w+),\s*(\w+),\s*([^)]+)\)", s)
        if m:
            name, vx, vy, dz = m.groups()
            self.shapes[name] = {"type": "gentrap", "args": [self.env[vx], self.env[vy], float(self.ev(dz))]}
            return
        if s.startswith("Vec_t "):
            for decl in split_args(s[len("Vec_t "):]):
                m = re.fullmatch(r"(\w+)\((.*)\)", decl, flags=re.S)
                if m:
                    self.env[m.group(1)] = V(*(self.ev(x) for x in split_args(m.group(2))))
                else:  # Vec_t name;  (Vector3D's default constructor: zeros)
                    self.env[decl] = V(0.0, 0.0, 0.0)
            return
        m = re.fullmatch(r"Precision (\w+)\s*=\s*(.+)", s, flags=re.S)
        if m:
            self.env[m.group(1)] = self.ev(m.group(2))
            return
        m = re.fullmatch(r"valid\s*=\s*(\w+)\.Normal\((\w+),\s*normal\)", s)
        if m:
            self.env["normal"] = NormalRef(m.group(1), self.env[m.group(2)])
            return
        m = re.fullmatch(r"(vol|surf|volCheck\d|surfCheck)\s*=.*", s, flags=re.S)
        if m:
            if "Capacity" in s or "SurfaceArea" in s:
                self.skipped.append((self.line, s))
            return
        m = re.fullmatch(r"Dist\s*=\s*(\w+)\.(\w+)\((.*)\)", s, flags=re.S)
        if m:
            assert m.group(2) in QUERIES, s
            self.pending = self.call(m.group(1), m.group(2), m.group(3))
            return
        m = re.fullmatch(r"(\w+)\.(Normalize|Set)\((.*)\)", s, flags=re.S)
        if m:
            if m.group(2) == "Normalize":
                self.env[m.group(1)].Normalize()
            else:
                self.env[m.group(1)] = V(*(self.ev(x) for x in split_args(m.group(3))))
            return
        m = re.fullmatch(r"(\w+)\.Extent\((\w+),\s*(\w+)\)", s)
        if m:
            self.env["__extent__"] = (m.group(1), m.group(2), m.group(3))
            return
        if "GetBBox(" in s:
            return
        m = re.fullmatch(r"(\w+)\s*=\s*(.+)", s, flags=re.S)
        if m:
            val = self.ev(m.group(2))
            if isinstance(val, V):
                val = V(*val.v)
            self.env[m.group(1)] = val
            return
        if s.startswith("assert("):
            return self.assertion(s[len("assert("):-1].strip())
        raise ValueError("unhandled statement at line %d: %s" % (self.line, s))

    def assertion(self, a):
        a = re.sub(r"\s*&&\s*\"[^\"]*\"$", "", a)
        m = re.fullmatch(r"(\w+)\.Inside\((\w+)\)\s*==\s*vecgeom::EInside::(\w+)", a)
        if m:
            return self.record("Inside", "==", float(INSIDE[m.group(3)]), m.group(1), self.env[m.group(2)].v)
        m = re.fullmatch(r"ApproxEqual\(normal,\s*(Vec_t\(.*\))\)", a)
        if m:
            ref = self.env["normal"]
            return self.record("Normal", "approx_vec", self.ev(m.group(1)).v, ref.shape, ref.at.v)
        if re.search(r"\b(vol|surf)\b", a):
            self.skipped.append((self.line, "assert(" + a + ")"))
            return
        if a == "valid == true":
            return
        m = re.fullmatch(r"ApproxEqual\((minExtent|maxExtent),\s*(Vec_t\(.*\))\)", a)
        if m:
            shape = self.env["__extent__"][0]
            q = "ExtentMin" if m.group(1) == "minExtent" else "ExtentMax"
            return self.record(q, "approx_vec", self.ev(m.group(2)).v, shape)
        if re.fullmatch(r"ApproxEqual\((minExtent|maxExtent),\s*(minBBox|maxBBox)\)", a):
            self.skipped.append((self.line, "assert(" + a + ")  (the cached box is the extent)"))
            return
        shape, query, p, along, d = self.pending
        m = re.fullmatch(r"ApproxEqual<Precision>\(Dist,\s*(.+)\)", a)
        if m:
            return self.record(query, "approx", float(self.ev(m.group(1))), shape, p, along, d)
        m = re.fullmatch(r"Dist\s*(<=|<|>=|>)\s*(.+)", a)
        if m:
            return self.record(query, m.group(1), float(self.ev(m.group(2))), shape, p, along, d)
        raise ValueError("unhandled assert at line %d: %s" % (self.line, a))

    # -------------------------------------------------------------- the function body
    def run(self, body, first_line):
        lines = body.split("\n")
        i = 0
        stmt, start = "", None
        while i < len(lines):
            line = lines[i]
            m = re.match(r"\s*for \(int i = 0; i < (\d+); i\+\+\) \{", line)
            if m:
                depth, j, block = 1, i + 1, []
                while depth:
                    depth += lines[j].count("{") - lines[j].count("}")
                    block.append((j, lines[j]))
                    j += 1
                block[-1] = (block[-1][0], block[-1][1].rsplit("}", 1)[0])
                text = " ".join(l for _, l in block)
                if "SamplePointOnSurface" in text:
                    self.skipped.append((first_line + i, "for-loop over SamplePointOnSurface (random points)"))
                else:
                    for k in range(int(m.group(1))):
                        self.env["i"] = k
                        for s in text.split(";"):
                            self.line = first_line + i
                            self.statement(s)
                i = j
                continue
            if not stmt.strip():
                start = first_line + i
            stmt += " " + line
            while ";" in stmt:
                s, stmt = stmt.split(";", 1)
                self.line = start
                if s.strip().startswith("return"):
                    return
                self.statement(s)
                start = first_line + i
            i += 1


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VECGEOM_SOURCE_DIR")
    out_dir = sys.argv[2] if len(sys.argv) > 2 else os.path.dirname(os.path.abspath(__file__))
    if not root:
        sys.exit(__doc__)
    path = os.path.join(root, "test", "unit_tests", "TestGenTrap.cpp")
    src = strip_comments(open(path).read())
    m = re.search(r"bool TestGenTrap\(\)\s*\{", src)
    depth, k = 1, m.end()
    while depth:
        depth += {"{": 1, "}": -1}.get(src[k], 0)
        k += 1
    body = src[m.end():k - 1]
    first_line = src[:m.end()].count("\n") + 1  # the line of the opening brace: body line 0
    it = Interp()
    it.run(body, first_line)
    doc = {"source": "test/unit_tests/TestGenTrap.cpp", "shapes": it.shapes, "cases": it.cases,
           "skipped_statements": [{"line": l, "text": t} for l, t in it.skipped],
           "note": "GenTrap(vertices x[8], vertices y[8], dz); points along a normal are resolved with the "
                   "shape's Normal at test time"}
    with open(os.path.join(out_dir, "unit_GenTrap.json"), "w") as f:
        json.dump(doc, f, indent=1)
    print("%d cases, %d skipped" % (len(it.cases), len(it.skipped)))


if __name__ == "__main__":
    main()
