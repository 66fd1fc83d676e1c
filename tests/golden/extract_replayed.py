"""Extract the known answers of VecGeom unit tests that compute their points and directions
in code (TestGenTrap.cpp, TestHype.cpp) into JSON fixtures.

Reads the test file of a VecGeom source tree AS TEXT (nothing of it is compiled or run) and
replays the straight-line statements of its test function with a small interpreter of the
forms these files use: numeric and vertex-array declarations, the shape's construction,
Vec_t points (with +, -, unary -, scalar *, Mag, Mag2, Normalize, Set), scalar assignments,
counted for-loops, query calls (Inside, DistanceToIn, DistanceToOut, SafetyToIn,
SafetyToOut, Normal, Extent) and the asserts on their results. Each assert becomes one case:

    shape, query, point, direction, comparison (==, <, <=, ApproxEqual) and expected value

Special forms:
* a point built along the shape's own surface normal (p + t * normal after
  shape.Normal(p, normal)) is recorded as "along_normal" and resolved at test time with
  the oracle's Normal, as the test resolves it with the shape's;
* an assert comparing two query results (ApproxEqual(Dist3, Dist4)) is recorded as a
  "pairs" entry, both queries also as cases of kind "any";
* an assert on a normal at a point that depends on a query result (the exit point
  p + Dist * v) is skipped: Normal is not on the query path;
* capacity and surface-area asserts are not on the query path, and loops over
  SamplePointOnSurface draw from the reference's random generator, which cannot be
  replayed: both are listed as skipped.

Usage: python tests/golden/extract_replayed.py <VecGeom source tree> [out dir]
       (or set VECGEOM_SOURCE_DIR). Writes tests/golden/unit_GenTrap.json and unit_Hype.json.
"""
import json
import math
import os
import re
import sys

DBL_MAX = sys.float_info.max
QUERIES = ("Inside", "Contains", "DistanceToIn", "DistanceToOut", "SafetyToIn", "SafetyToOut")
INSIDE = {"kInside": 1, "kSurface": 2, "kOutside": 3}

# test file -> (test function, shape class in the file, fixture shape type, note)
FILES = {
    "GenTrap": ("TestGenTrap", "SimpleGenTrap", "gentrap",
                "GenTrap(vertices x[8], vertices y[8], dz); points along a normal are resolved with the shape's "
                "Normal at test time"),
    "Hype": ("TestHype", "Hype_t", "hype", "Hype(rmin, rmax, stereo angle in, stereo angle out, dz)"),
}


class V:
    """Vector3D<double> with the operations the tests use, in IEEE double."""

    def __init__(self, x, y, z):
        self.v = [float(x), float(y), float(z)]

    def __add__(self, o):
        if isinstance(o, AlongNormal):
            return o.offset(self, 1.0)
        if isinstance(o, Along):
            return o.offset(self)
        return V(*(a + b for a, b in zip(self.v, o.v)))

    def __sub__(self, o):
        if isinstance(o, AlongNormal):
            return o.offset(self, -1.0)
        return V(*(a - b for a, b in zip(self.v, o.v)))

    def __rmul__(self, s):
        if isinstance(s, QueryRef):
            return Along(s, self)
        return V(*(s * a for a in self.v))

    def __neg__(self):
        return V(*(-a for a in self.v))

    def Mag2(self):
        x, y, z = self.v
        return x * x + y * y + z * z

    def Mag(self):
        return math.sqrt(self.Mag2())

    def Normalize(self):  # Vector3D.h:198: *this *= 1 / Length()
        s = 1.0 / self.Mag()
        self.v = [a * s for a in self.v]


class NormalRef:
    """The `normal` a shape.Normal(p, normal) call filled in, known only to the shape."""

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


class QueryRef:
    """The result of a query call, known only to the shape."""

    def __init__(self, shape, query, p, along, d):
        self.shape, self.query, self.p, self.along, self.d = shape, query, p, along, d


class Along:
    """p + Dist * v with Dist a query result (only used for a normal at the exit point)."""

    def __init__(self, ref, v):
        self.ref, self.v = ref, v

    def offset(self, base):
        return ResultPoint()


class ResultPoint:
    pass


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
    def __init__(self, shape_class, shape_type):
        self.shape_class, self.shape_type = shape_class, shape_type
        self.env = {"kInfLength": DBL_MAX, "kPi": math.pi, "kTolerance": 1e-9, "true": True, "false": False}
        self.shapes, self.cases, self.pairs, self.skipped = {}, [], [], []
        self.line = 0

    # -------------------------------------------------------------- expressions
    def ev(self, e):
        e = e.strip()
        e = re.sub(r"\bvecgeom::(cxx::)?", "", e)
        e = re.sub(r"std::(cos|sin|tan|atan2|sqrt)", r"math.\1", e)
        e = re.sub(r"\bVec_t\(", "V(", e)
        e = re.sub(r"(\d)\.(?!\d)", r"\1.0", e)
        m = re.fullmatch(r"\((.+?)\)\s*\?\s*(.+?)\s*:\s*(.+)", e)
        if m:
            e = "(%s if %s else %s)" % (m.group(2), m.group(1), m.group(3))
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
        return QueryRef(shape, method, p, along, d)

    def record(self, query, kind, expected, shape=None, p=None, along=None, d=None):
        c = {"shape": shape, "query": query, "p": p, "d": d, "kind": kind, "expected": expected,
             "line": self.line, "soft": False}
        if along is not None:
            c["along_normal"] = along
        self.cases.append(c)

    def record_query(self, ref, kind, expected):
        self.record(ref.query, kind, expected, ref.shape, ref.p, ref.along, ref.d)

    def statement(self, s):
        s = re.sub(r"^\s*(vecgeom::)?", "", s.strip())
        if not s or s.startswith(("using ", "std::cout", "bool valid", "Precision vol", "Precision surf",
                                  "Precision Dist,")):
            return
        if re.fullmatch(r"(?:Precision|double|bool) \w+", s):  # declaration without a value
            return
        m = re.fullmatch(r"Precision (\w+)\[8\]\s*=\s*\{(.*)\}", s, flags=re.S)
        if m:
            self.env[m.group(1)] = [float(self.ev(x)) for x in split_args(m.group(2))]
            return
        m = re.fullmatch(self.shape_class + r" (\w+)\(\"[^\"]*\",\s*(.*)\)", s, flags=re.S)
        if m:
            args = [self.ev(x) for x in split_args(m.group(2))]
            args = [a if isinstance(a, list) else float(a) for a in args]
            self.shapes[m.group(1)] = {"type": self.shape_type, "args": args}
            return
        if s.startswith("Vec_t "):
            for decl in split_args(s[len("Vec_t "):]):
                m = re.fullmatch(r"(\w+)\((.*)\)", decl, flags=re.S)
                if m:
                    self.env[m.group(1)] = V(*(self.ev(x) for x in split_args(m.group(2))))
                else:  # Vec_t name;  (Vector3D's default constructor: zeros)
                    self.env[decl] = V(0.0, 0.0, 0.0)
            return
        m = re.fullmatch(r"(?:Precision|double) (\w+\s*=.*)", s, flags=re.S)
        if m:  # one or more scalar declarations
            for decl in split_args(m.group(1)):
                name, expr = decl.split("=", 1)
                self.statement("%s = %s" % (name.strip(), expr))
            return
        m = re.fullmatch(r"valid\s*=\s*(\w+)\.Normal\((.+),\s*normal\)", s, flags=re.S)
        if m:
            at = self.ev(m.group(2))
            self.env["normal"] = NormalRef(m.group(1), at) if isinstance(at, V) else None
            return
        m = re.fullmatch(r"(vol|surf|volCheck\d|surfCheck)\s*=.*", s, flags=re.S)
        if m:
            if "Capacity" in s or "SurfaceArea" in s:
                self.skipped.append((self.line, s))
            return
        m = re.fullmatch(r"if \((\w+) >= kInfLength\) \1 = kInfLength", s)
        if m:  # clamping a result to kInfLength: ApproxEqual treats both as infinite already
            return
        m = re.fullmatch(r"(\w+)\s*=\s*(\w+)\.(\w+)\((.*)\)", s, flags=re.S)
        if m and m.group(3) in QUERIES:
            self.env[m.group(1)] = self.call(m.group(2), m.group(3), m.group(4))
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
        if a.startswith("!strcmp("):
            return
        if re.search(r"\b(vol|surf)\b", a):
            self.skipped.append((self.line, "assert(" + a + ")"))
            return
        if a == "valid == true":
            return
        parts = split_and(a)
        if len(parts) > 1:
            for p in parts:
                self.assertion(p)
            return
        m = re.fullmatch(r"(\w+)\.Inside\((.+)\)\s*==\s*EInside::(\w+)", re.sub(r"vecgeom::", "", a))
        if m:
            return self.record("Inside", "==", float(INSIDE[m.group(3)]), m.group(1), list(self.ev(m.group(2)).v))
        m = re.fullmatch(r"ApproxEqual\(normal,\s*(.+)\)", a)
        if m:
            ref = self.env["normal"]
            if ref is None:
                self.skipped.append((self.line, "assert(" + a + ")  (normal at a query's exit point)"))
                return
            if self.shape_type != "gentrap":
                self.skipped.append((self.line, "assert(" + a + ")  (Normal is not on the query path)"))
                return
            return self.record("Normal", "approx_vec", self.ev(m.group(1)).v, ref.shape, ref.at.v)
        m = re.fullmatch(r"ApproxEqual\((minExtent|maxExtent),\s*(Vec_t\(.*\))\)", a)
        if m:
            shape = self.env["__extent__"][0]
            q = "ExtentMin" if m.group(1) == "minExtent" else "ExtentMax"
            return self.record(q, "approx_vec", self.ev(m.group(2)).v, shape)
        if re.fullmatch(r"ApproxEqual\((minExtent|maxExtent),\s*(minBBox|maxBBox)\)", a):
            self.skipped.append((self.line, "assert(" + a + ")  (the cached box is the extent)"))
            return
        m = re.fullmatch(r"ApproxEqual<Precision>\((\w+),\s*(.+)\)", a)
        if m:
            ref, other = self.env[m.group(1)], self.ev(m.group(2))
            if isinstance(other, QueryRef):
                self.record_query(ref, "any", 0.0)
                self.record_query(other, "any", 0.0)
                self.pairs.append({"a": len(self.cases) - 2, "b": len(self.cases) - 1, "kind": "approx",
                                   "line": self.line})
                return
            return self.record_query(ref, "approx", float(other))
        m = re.fullmatch(r"(\w+)\s*(<=|<|>=|>)\s*(.+)", a)
        if m and isinstance(self.env.get(m.group(1)), QueryRef):
            return self.record_query(self.env[m.group(1)], m.group(2), float(self.ev(m.group(3))))
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


def split_and(a):
    """Top-level && operands of an assert expression."""
    out, depth, cur, k = [], 0, "", 0
    while k < len(a):
        ch = a[k]
        depth += ch in "(["
        depth -= ch in ")]"
        if depth == 0 and a.startswith("&&", k):
            out.append(cur.strip())
            cur, k = "", k + 2
            continue
        cur += ch
        k += 1
    out.append(cur.strip())
    return out


def extract(root, name):
    func, cls, typ, note = FILES[name]
    path = os.path.join(root, "test", "unit_tests", "Test%s.cpp" % name)
    src = strip_comments(open(path).read())
    m = re.search(r"bool %s\(\)\s*\{" % func, src)
    depth, k = 1, m.end()
    while depth:
        depth += {"{": 1, "}": -1}.get(src[k], 0)
        k += 1
    body = src[m.end():k - 1]
    first_line = src[:m.end()].count("\n") + 1  # the line of the opening brace: body line 0
    it = Interp(cls, typ)
    it.run(body, first_line)
    return {"source": "test/unit_tests/Test%s.cpp" % name, "shapes": it.shapes, "cases": it.cases,
            "pairs": it.pairs, "skipped_statements": [{"line": l, "text": t} for l, t in it.skipped], "note": note}


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VECGEOM_SOURCE_DIR")
    out_dir = sys.argv[2] if len(sys.argv) > 2 else os.path.dirname(os.path.abspath(__file__))
    if not root:
        sys.exit(__doc__)
    for name in FILES:
        doc = extract(root, name)
        with open(os.path.join(out_dir, "unit_%s.json" % name), "w") as f:
            json.dump(doc, f, indent=1)
        print("%s: %d cases, %d pairs, %d skipped" % (name, len(doc["cases"]), len(doc["pairs"]),
                                                       len(doc["skipped_statements"])))


if __name__ == "__main__":
    main()
