"""Extract the known answers of VecGeom's boolean unit test into a JSON fixture.

Reads test/unit_tests/TestBooleans.cpp of a VecGeom source tree AS TEXT (nothing of it is
compiled or run) and records the geometry the test builds (boxes and tubes, their logical
volumes and placements, the booleans made of placed volumes: a union of two tubes, a box
minus that union, a union of the tube union and a rotated slab) and every assert on a
query result of those placed volumes:

    volume, query (Contains, DistanceToIn, DistanceToOut, PlacedDistanceToOut), point,
    direction, comparison (truth, ==, ApproxEqual, <, >) and expected value

An assert that compares two query results with each other (ApproxEqual(dt1, d)) is kept
as a pair. The capacity, surface-area and bounding-box asserts are not on the query path
and are skipped, as are commented-out checks.

Usage: python tests/golden/extract_booleans.py <VecGeom source tree> [out dir]
       (or set VECGEOM_SOURCE_DIR). Writes tests/golden/unit_Booleans.json.
"""
import json
import math
import os
import re
import sys

DBL_MAX = sys.float_info.max


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
        depth += ch in "(["
        depth -= ch in ")]"
        cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def euler_rotation(phi, theta, psi):
    """Transformation3D::SetRotation(phi, theta, psi) in degrees (source/Transformation3D.cpp:129-148)."""
    d = math.pi / 180.0
    sf, cf = math.sin(d * phi), math.cos(d * phi)
    st, ct = math.sin(d * theta), math.cos(d * theta)
    sp, cp = math.sin(d * psi), math.cos(d * psi)
    return [cp * cf - ct * sf * sp, -sp * cf - ct * sf * cp, st * sf,
            cp * sf + ct * cf * sp, -sp * sf + ct * cf * cp, -st * cf,
            sp * st, cp * st, ct]


class Extractor:
    def __init__(self):
        self.scalars = {}
        self.shapes = {}   # name -> {"type", "args"} (box, tube, union, subtraction)
        self.lvs = {}      # name -> shape name
        self.pvs = {}      # name -> {"lv", "trans", "rot"}
        self.order = []    # creation order: ("shape"|"lv"|"pv", name)
        self.calls = {}    # variable -> call description
        self.cases = []
        self.anon = 0

    # ---------------------------------------------------------------- expressions
    def num(self, expr):
        e = expr.strip()
        e = re.sub(r"vecgeom::kTwoPi|kTwoPi", repr(2.0 * math.pi), e)
        e = e.replace("kInfLength", repr(DBL_MAX))
        e = re.sub(r"\b(\w+)\.rmax\(\)", lambda m: repr(self.shapes[m.group(1)]["args"][1]), e)
        e = re.sub(r"std::sqrt|sqrt", "math.sqrt", e)
        e = re.sub(r"<\w+>", "", e)
        return float(eval(e, {"math": math}, dict(self.scalars)))

    def vec(self, expr):
        m = re.match(r"Vec3D_t\((.*?)\)(\.Normalized\(\))?$", expr.strip())
        v = [self.num(a) for a in split_args(m.group(1))]
        if m.group(2):
            n = math.sqrt(sum(c * c for c in v))
            v = [c / n for c in v]
        return v

    def transform(self, arg):
        """`new Transformation3D(...)` -> (translation, rotation)."""
        m = re.match(r"new Transformation3D\((.*)\)$", arg.strip())
        a = [self.num(x) for x in split_args(m.group(1))]
        rot = euler_rotation(*a[3:6]) if len(a) == 6 else [1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0]
        return a[:3], rot

    def place(self, name, lv, targs):
        trans, rot = self.transform(targs) if targs.strip() else ([0.0, 0.0, 0.0], [1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0])
        self.pvs[name] = {"lv": lv, "trans": trans, "rot": rot}
        self.order.append(("pv", name))

    def operand(self, expr):
        m = re.match(r"(\w+)\.Place\((.*)\)$", expr.strip())
        if m:
            self.anon += 1
            name = "_placed%d" % self.anon
            self.place(name, m.group(1), m.group(2))
            return name
        return expr.strip()

    # ---------------------------------------------------------------- statements
    def statement(self, st, line):
        st = re.split(r"[{}]", st)[-1].strip()  # drop block braces and the function header
        if not st:
            return
        m = re.match(r"(UnplacedBox|GenericUnplacedTube)\s+(\w+)\((.*)\)$", st, re.S)
        if m:
            kind = "box" if m.group(1) == "UnplacedBox" else "tube"
            self.shapes[m.group(2)] = {"type": kind, "args": [self.num(a) for a in split_args(m.group(3))]}
            self.order.append(("shape", m.group(2)))
            return
        m = re.match(r"UnplacedBooleanVolume<k(Union|Subtraction)>\s+(\w+)\(k\w+,\s*(.*)\)$", st, re.S)
        if m:
            left, right = split_args(m.group(3))
            self.shapes[m.group(2)] = {"type": m.group(1).lower(), "args": [self.operand(left), self.operand(right)]}
            self.order.append(("shape", m.group(2)))
            return
        m = re.match(r'LogicalVolume\s+(\w+)\("[^"]*",\s*&(\w+)\)$', st)
        if m:
            self.lvs[m.group(1)] = m.group(2)
            self.order.append(("lv", m.group(1)))
            return
        m = re.match(r'auto\s+(\w+)\s*=\s*\(new LogicalVolume\("[^"]*",\s*&(\w+)\)\)->Place\(\)$', st)
        if m:
            lv = "_lv_" + m.group(1)
            self.lvs[lv] = m.group(2)
            self.order.append(("lv", lv))
            self.place(m.group(1), lv, "")
            return
        m = re.match(r"auto\s+(\w+)\s*=\s*(\w+)\.Place\((.*)\)$", st, re.S)
        if m:
            self.place(m.group(1), m.group(2), m.group(3))
            return
        m = re.match(r"(?:bool|double)\s+(\w+)\s*=\s*(\w+)->(Contains|DistanceToIn|DistanceToOut|PlacedDistanceToOut)"
                     r"\((.*)\)$", st, re.S)
        if m:
            args = split_args(m.group(4))
            self.calls[m.group(1)] = {"volume": m.group(2), "query": m.group(3), "p": self.vec(args[0]),
                                      "d": self.vec(args[1]) if len(args) > 1 else None}
            return
        m = re.match(r"(?:double|auto)\s+(\w+)\s*=\s*(.+)$", st, re.S)
        if m and "->" not in st and not re.search(r"[A-Za-z_]\w*\.[A-Za-z_]\w*\(", m.group(2)):
            try:
                self.scalars[m.group(1)] = self.num(m.group(2))
            except Exception:
                pass
            return
        m = re.match(r"assert\((.*)\)$", st, re.S)
        if m:
            self.assertion(m.group(1).strip(), line)

    def case(self, var, kind, expected, line):
        c = dict(self.calls[var])
        c.update(kind=kind, expected=expected, line=line)
        self.cases.append(c)

    def assertion(self, e, line):
        if re.fullmatch(r"!?\w+", e) and e.lstrip("!") in self.calls:
            self.case(e.lstrip("!"), "==", 0.0 if e.startswith("!") else 1.0, line)
            return
        m = re.fullmatch(r"ApproxEqual(?:<\w+>)?\((.*)\)", e, re.S)
        if m:
            a, b = split_args(m.group(1))
            if a in self.calls and b in self.calls:
                self.cases.append({"kind": "approx_pair", "a": self.calls[a], "b": self.calls[b], "line": line})
            elif a in self.calls:
                self.case(a, "approx", self.num(b), line)
            elif b in self.calls:
                self.case(b, "approx", self.num(a), line)
            return
        for part in e.split("&&"):
            m = re.fullmatch(r"\s*(\w+)\s*(==|<=|>=|<|>)\s*(.+?)\s*", part)
            if m and m.group(1) in self.calls:
                self.case(m.group(1), m.group(2), self.num(m.group(3)), line)

    def run(self, src):
        text = strip_comments(src)
        body = text[text.index("int TestBooleans()"):]
        pos, line0 = 0, text[:text.index("int TestBooleans()")].count("\n") + 1
        for st in body.split(";"):
            self.statement(st, line0 + body[:pos].count("\n") + st[:len(st) - len(st.lstrip())].count("\n"))
            pos += len(st) + 1


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VECGEOM_SOURCE_DIR")
    if not root:
        sys.exit("usage: extract_booleans.py <VecGeom source tree> [output dir] (or set VECGEOM_SOURCE_DIR)")
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(root, "test", "unit_tests", "TestBooleans.cpp")) as f:
        src = f.read()
    ex = Extractor()
    ex.run(src)
    doc = {"source": "test/unit_tests/TestBooleans.cpp", "shapes": ex.shapes, "lvs": ex.lvs, "pvs": ex.pvs,
           "order": ex.order, "cases": ex.cases,
           "note": "line numbers are those of the source file; placed volumes named _placed<k> are placements "
                   "written inline in a boolean's constructor"}
    with open(os.path.join(out, "unit_Booleans.json"), "w") as f:
        json.dump(doc, f, indent=0)
    print("Booleans %d cases, %d shapes, %d placed volumes" % (len(ex.cases), len(ex.shapes), len(ex.pvs)))


if __name__ == "__main__":
    main()
