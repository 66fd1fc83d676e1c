"""Extract known-answer vectors from VecGeom's shape unit tests into JSON fixtures.

Reads test/unit_tests/Test{Box,Tube,Cons,Polycone,Torus2,Trd,Polyhedra,Trap,Sphere}.cpp of a VecGeom
source tree AS TEXT (nothing of it is compiled or run) and records, for every assert that checks
a query result of a shape constructed in the test:

    shape constructor arguments, query name, point, direction, expected value, comparison

Checks written as asserts are "hard"; checks that only print a mismatch (TestCons's
`if (OutRange(...)) std::cout << ...`) are recorded with "soft": true, because the
reference's own run does not enforce them.

A small evaluator follows each test body statement by statement: vector and scalar
declarations, arrays, shape constructions, `X = shape.Query(args)` assignments, and the
asserts on X (ApproxEqual with the tests' own tolerance, ==, <, <=, >, >=) or directly on
`shape.Inside(p)`. Statements it cannot evaluate (loops, helpers, unsupported shapes and
queries) are skipped and counted. `if (testvecgeom)` blocks are taken as the tests' main()
sets that flag for the VecGeom types; `if (!testvecgeom)` blocks are dropped.

Usage: python tests/golden/extract_unit_vectors.py <vecgeom source root> [out dir]
Writes tests/golden/unit_<Shape>.json. Run in a checkout of the reference; the fixtures
are committed so that the tests need no reference tree.
"""
import json
import math
import os
import re
import sys

DBL_MAX = sys.float_info.max
FILES = {
    "Box": ("TestBox.cpp", {"Box_t": "box"}),
    "Tube": ("TestTube.cpp", {"Tube_t": "tube"}),
    "Cons": ("TestCons.cpp", {"Cone_t": "cone", "Tube_t": "tube"}),
    "Polycone": ("TestPolycone.cpp", {"Polycone_t": "polycone"}),
    "Torus2": ("TestTorus2.cpp", {"Torus_t": "torus2"}),
    "Trd": ("TestTrd.cpp", {"Trd_t": "trd"}),
    "Polyhedra": ("TestPolyhedra.cpp", {"Polyhedra_t": "polyhedron"}),
    "Trap": ("TestTrap.cpp", {"Trap_t": "trap", "vecgeom::UnplacedTrapezoid": "trap"}),
    "Sphere": ("TestSphere.cpp", {"Sphere_t": "sphere"}),
}
# object-like macros of a test file, expanded textually (unparenthesised, as the
# preprocessor does) before the file is evaluated
MACROS = {
    "TestSphere.cpp": [("deg", "PI / 180."), ("PI", "3.14159265358979323846")],
}
# unplaced shapes constructed without a label argument
NO_LABEL = {"vecgeom::UnplacedTrapezoid"}
QUERIES = {"Inside", "Contains", "DistanceToIn", "DistanceToOut", "SafetyToIn", "SafetyToOut"}
# Extent(lo, hi) results are recorded as the queries "ExtentMin" / "ExtentMax" (no point;
# the expected value is a vector compared component-wise with ApproxEqual)


class V:
    """Minimal Vector3D for evaluating test expressions."""

    def __init__(self, x=0.0, y=0.0, z=0.0):
        self.v = (float(x), float(y), float(z))

    def x(self):
        return self.v[0]

    def y(self):
        return self.v[1]

    def z(self):
        return self.v[2]

    def __add__(self, o):
        return V(*(a + b for a, b in zip(self.v, o.v)))

    def __sub__(self, o):
        return V(*(a - b for a, b in zip(self.v, o.v)))

    def __neg__(self):
        return V(*(-a for a in self.v))

    def __mul__(self, s):
        if isinstance(s, V):
            return sum(a * b for a, b in zip(self.v, s.v))
        return V(*(a * s for a in self.v))

    __rmul__ = __mul__

    def __truediv__(self, s):
        return V(*(a / s for a in self.v))

    def Mag2(self):
        return sum(a * a for a in self.v)

    def Mag(self):
        return math.sqrt(self.Mag2())

    def Perp2(self):
        return self.v[0] ** 2 + self.v[1] ** 2

    def Perp(self):
        return math.sqrt(self.Perp2())

    def Unit(self):
        m = self.Mag()
        return V(*(a / m for a in self.v)) if m > 0 else V(*self.v)

    def Normalized(self):
        return self.Unit()

    def Dot(self, o):
        return self * o


BASE_ENV = {
    "V": V, "sqrt": math.sqrt, "cos": math.cos, "sin": math.sin, "tan": math.tan, "atan": math.atan,
    "atan2": math.atan2, "acos": math.acos, "asin": math.asin, "fabs": abs, "abs": abs, "pow": math.pow,
    "kPi": math.pi, "kTwoPi": 2 * math.pi, "kHalfPi": 0.5 * math.pi, "kDegToRad": math.pi / 180.0,
    "kRadToDeg": 180.0 / math.pi, "kInfLength": DBL_MAX, "kTolerance": 1e-9, "kHalfTolerance": 5e-10,
    "kInside": 1, "kSurface": 2, "kOutside": 3, "INF": DBL_MAX, "kSqrt2": math.sqrt(2.0),
    "float": float, "max": max, "min": min,
}


def strip_comments(src):
    src = re.sub(r"/\*.*?\*/", lambda m: "\n" * m.group(0).count("\n"), src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    # drop #if 0 ... #endif blocks, keep other preprocessor-free code
    out, skip = [], 0
    for line in src.split("\n"):
        s = line.strip()
        if s.startswith("#if 0"):
            skip += 1
            out.append("")
            continue
        if skip:
            if s.startswith("#if"):
                skip += 1
            elif s.startswith("#endif"):
                skip -= 1
            out.append("")
            continue
        if s.startswith("#"):
            out.append("")
            continue
        out.append(line)
    return "\n".join(out)


def match_brace(s, i):
    """Index of the brace closing the one at s[i]."""
    depth = 0
    for k in range(i, len(s)):
        if s[k] == "{":
            depth += 1
        elif s[k] == "}":
            depth -= 1
            if depth == 0:
                return k
    return len(s) - 1


def resolve_flag_blocks(s):
    """Replace `if (testvecgeom) {A} else {B}` by A and `if (!testvecgeom) {A} [else {B}]` by B."""
    pat = re.compile(r"if\s*\(\s*(!?)\s*testvecgeom\s*\)\s*\{")
    while True:
        m = pat.search(s)
        if not m:
            return s
        neg = m.group(1) == "!"
        a0 = m.end() - 1
        a1 = match_brace(s, a0)
        then_body = s[a0 + 1:a1]
        rest = s[a1 + 1:]
        else_body = ""
        m2 = re.match(r"\s*else\s*\{", rest)
        end = a1 + 1
        if m2:
            b0 = a1 + 1 + m2.end() - 1
            b1 = match_brace(s, b0)
            else_body = s[b0 + 1:b1]
            end = b1 + 1
        keep = else_body if neg else then_body
        s = s[:m.start()] + keep + s[end:]


def split_top(s, sep=","):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [p.strip() for p in parts]


def strip_parens(s):
    """Remove parentheses that enclose the whole expression."""
    s = s.strip()
    while s.startswith("("):
        depth = 0
        for k, ch in enumerate(s):
            depth += ch == "("
            depth -= ch == ")"
            if depth == 0:
                break
        if k != len(s) - 1:
            break
        s = s[1:-1].strip()
    return s


def find_top(s, ops):
    """First operator of `ops` outside parentheses that is not part of `->`; (index, op)."""
    depth = 0
    for k, ch in enumerate(s):
        depth += ch in "([{"
        depth -= ch in ")]}"
        if depth:
            continue
        for op in ops:
            if s.startswith(op, k):
                if op in (">", ">=") and k > 0 and s[k - 1] == "-":
                    continue
                if op == "-" and s.startswith("->", k):
                    continue
                if op in ("<", ">") and (s.startswith("<=", k) or s.startswith(">=", k)):
                    continue
                return k, op
    return -1, None


def to_py(expr):
    e = expr.strip()
    e = re.sub(r"\bstatic_cast<[^>]*>", "", e)
    e = re.sub(r"\((?:Precision|double|float|int)\)", "", e)
    e = re.sub(r"\bvecgeom::InfinityLength<[^>]*>\(\)", "kInfLength", e)
    e = re.sub(r"\b(?:std|vecgeom|vecCore|math|EInside|Vec_t::)::", "", e)
    e = re.sub(r"\b(?:std|vecgeom|vecCore|math|EInside|VECGEOM_NAMESPACE)::", "", e)
    e = re.sub(r"\bVec_t\s*\(", "V(", e)
    e = re.sub(r"\bVector3D<[^>]*>\s*\(", "V(", e)
    e = re.sub(r"\bPrecision\s*\(", "float(", e)
    e = re.sub(r"(\d)[fF]\b", r"\1", e)
    e = re.sub(r"(\d\.)[fF]\b", r"\1", e)
    e = e.replace("&&", " and ").replace("||", " or ")
    e = re.sub(r"!(?!=)", " not ", e)
    # C++ integer division between integer literals
    e = re.sub(r"(?<![\w.])(\d+)\s*/\s*(\d+)(?![\w.])", r"(\1//\2)", e)
    return e


class Extractor:
    def __init__(self, shape_types):
        self.shape_types = shape_types
        self.env = dict(BASE_ENV)
        self.shapes = {}   # var -> {"type", "args"}
        self.lvs = {}      # logical-volume var -> shape var
        self.uninit = set()  # vectors declared without a value and not assigned since
        self.results = {}  # var -> pending query descriptor
        self.cases = []
        self.skipped = 0
        self.used_shapes = {}

    def ev(self, expr):
        return eval(to_py(expr), {"__builtins__": {}}, self.env)

    def query_call(self, text):
        m = re.match(r"^\s*([A-Za-z_]\w*)\s*(?:\.|->)\s*(\w+)\s*\((.*)\)\s*$", text, flags=re.S)
        if not m or m.group(2) not in QUERIES or m.group(1) not in self.shapes:
            return None
        args = split_top(m.group(3))
        q = m.group(2)
        p = self.ev(args[0])
        if not isinstance(p, V):
            return None
        d = None
        if q in ("DistanceToIn", "DistanceToOut"):
            if len(args) < 2:
                return None
            d = self.ev(args[1])
            if not isinstance(d, V):
                return None
        return {"shape": m.group(1), "query": q, "p": list(p.v), "d": list(d.v) if d else None}

    def emit(self, qd, kind, value, line, soft=False):
        name = qd["shape"]
        self.used_shapes[name] = self.shapes[name]
        c = dict(qd, kind=kind, expected=value, line=line, soft=soft)
        self.cases.append(c)

    def handle_fabs(self, term, line):
        """`fabs(CALL - value) < tol` or `fabs(CALL) < tol` (TestPolyhedra.cpp style)."""
        m = re.match(r"^(?:std::)?fabs\s*\((.*)\)\s*<\s*(.+)$", term, flags=re.S)
        if not m:
            return False
        inner = strip_parens(m.group(1))
        k, op = find_top(inner, ["-"])
        call, val = (strip_parens(inner[:k]), inner[k + 1:].strip()) if k > 0 else (inner, "0")
        qd = self.results.get(call) if re.match(r"^\w+$", call) else self.query_call(call)
        if qd is None:
            return False
        tol = float(self.ev(m.group(2)))
        self.emit(qd, "absdiff", float(self.ev(val)), line)
        self.cases[-1]["tol"] = tol
        return True

    def handle_assert(self, body, line):
        if len(split_top(body, "|")) > 1:
            return False  # alternatives: no single known answer
        ok = False
        for term in split_top(body, "&"):
            term = term.strip().strip("&").strip()
            if not term:
                continue
            if self.handle_fabs(term, line):
                ok = True
                continue
            m = re.match(r"^ApproxEqual(?:<[^>]*>)?\s*\((.*)\)$", term, flags=re.S)
            if m:
                a = split_top(m.group(1))
                if len(a) != 2:
                    continue
                lhs = a[0]
                qd = self.results.get(lhs) if re.match(r"^\w+$", lhs) else self.query_call(lhs)
                if qd is None:
                    continue
                try:
                    val = self.ev(a[1])
                except Exception:
                    continue
                if isinstance(val, V):
                    # an expected vector must be a value the test states, not another
                    # output (e.g. GetBBox into a vector declared without a value)
                    if qd["query"].startswith("Extent") and a[1].strip() not in self.uninit:
                        self.emit(qd, "approx_vec", list(val.v), line)
                        ok = True
                    continue
                if qd["query"].startswith("Extent"):
                    continue
                self.emit(qd, "approx", float(val), line)
                ok = True
                continue
            neg = term.startswith("!")
            qd = self.query_call(strip_parens(term[1:] if neg else term))
            if qd is not None and qd["query"] == "Contains":
                self.emit(qd, "==", 0.0 if neg else 1.0, line)
                ok = True
                continue
            k, op = find_top(term, ["==", "!=", "<=", ">=", "<", ">"])
            if k > 0:
                lhs, rhs = strip_parens(term[:k]), strip_parens(term[k + len(op):])
                qd = self.results.get(lhs) if re.match(r"^\w+$", lhs) else self.query_call(lhs)
                if qd is None:
                    continue
                try:
                    val = self.ev(rhs)
                except Exception:
                    continue
                if isinstance(val, V):
                    continue
                self.emit(qd, op, float(val), line)
                ok = True
        return ok

    def handle_condition(self, cond, line):
        """Soft checks of the form `if (OutRange(X, wanted) || ...)` or
        `if ((X = shape.Query(...)) != wanted)`: the wanted value is a known answer."""
        for term in split_top(cond, "|"):
            term = term.strip().strip("|").strip()
            if not term:
                continue
            m = re.match(r"^OutRange\s*\((.*)\)$", term, flags=re.S)
            if m:
                a = split_top(m.group(1))
                if len(a) == 2:
                    qd = self.results.get(a[0]) if re.match(r"^\w+$", a[0]) else self.query_call(a[0])
                    if qd is not None:
                        val = self.ev(a[1])
                        if not isinstance(val, V):
                            self.emit(qd, "range", float(val), line, soft=True)
                continue
            m = re.match(r"^\(\s*\(\s*(\w+)\s*=\s*(.*)\)\s*!=\s*(.*)\)?$", "(" + term + ")", flags=re.S)
            m = m or re.match(r"^\(\s*(\w+)\s*=\s*(.*)\)\s*!=\s*(.*)$", term, flags=re.S)
            if m:
                qd = self.query_call(m.group(2))
                if qd is not None:
                    self.results[m.group(1)] = qd
                    rhs = m.group(3).strip()
                    while rhs.endswith(")") and rhs.count(")") > rhs.count("("):
                        rhs = rhs[:-1]
                    val = self.ev(rhs)
                    if not isinstance(val, V):
                        self.emit(qd, "==", float(val), line, soft=True)
                continue
            m = re.match(r"^(\w+)\s*!=\s*(.*)$", term, flags=re.S)
            if m and m.group(1) in self.results:
                val = self.ev(m.group(2))
                if not isinstance(val, V):
                    self.emit(self.results[m.group(1)], "==", float(val), line, soft=True)

    def statement(self, st, line):
        st = st.strip()
        if not st:
            return
        # shape construction
        types = "|".join(re.escape(t) for t in self.shape_types)
        m = re.match(r"^(?:const\s+)?(" + types + r")\s+(.*)$", st, flags=re.S)
        if m:
            for decl in split_top(m.group(2)):
                mm = re.match(r"^\*?\s*(\w+)\s*(?:=\s*new\s+(?:" + types + r")\s*)?\((.*)\)$", decl, flags=re.S)
                if not mm:
                    self.skipped += 1
                    continue
                args = split_top(mm.group(2))
                try:
                    vals = []
                    for a in args[0 if m.group(1) in NO_LABEL else 1:]:
                        v = self.ev(a)
                        if isinstance(v, list):
                            v = [list(e.v) if isinstance(e, V) else float(e) for e in v]
                        vals.append(v if isinstance(v, list) else float(v))
                    self.shapes[mm.group(1)] = {"type": self.shape_types[m.group(1)], "args": vals}
                except Exception:
                    self.skipped += 1
            return
        # arrays: double name[] = {...};  Precision name[N] = {...};
        m = re.match(r"^(?:const\s+)?(?:static\s+)?(?:double|Precision|float|int)\s+(\w+)\s*\[[^\]]*\]\s*=\s*\{(.*)\}$",
                     st, flags=re.S)
        if m:
            try:
                self.env[m.group(1)] = [float(self.ev(a)) for a in split_top(m.group(2)) if a]
            except Exception:
                self.skipped += 1
            return
        m = re.match(r"^(?:const\s+)?(?:double|Precision|float)\s+(\w+)\s*\[\s*(\w+)\s*\]$", st)
        if m:
            try:
                self.env[m.group(1)] = [0.0] * int(self.ev(m.group(2)))
            except Exception:
                self.skipped += 1
            return
        m = re.match(r"^(\w+)\s*\[\s*(\w+)\s*\]\s*=\s*(.*)$", st, flags=re.S)
        if m and isinstance(self.env.get(m.group(1)), list):
            try:
                val = self.ev(m.group(3))
                self.env[m.group(1)][int(self.ev(m.group(2)))] = val if isinstance(val, V) else float(val)
            except Exception:
                self.env.pop(m.group(1), None)
                self.skipped += 1
            return
        # vector arrays: Vec_t name[N] = {Vec_t(...), ...};  Vec_t name[N];
        m = re.match(r"^(?:const\s+)?Vec_t\s+(\w+)\s*\[\s*(\w*)\s*\]\s*(?:=\s*\{(.*)\})?$", st, flags=re.S)
        if m:
            try:
                if m.group(3) is not None:
                    self.env[m.group(1)] = [self.ev(a) for a in split_top(m.group(3)) if a]
                else:
                    self.env[m.group(1)] = [V() for _ in range(int(self.ev(m.group(2))))]
            except Exception:
                self.skipped += 1
            return
        # a logical volume of a shape, and its placement at the identity (same answers)
        m = re.match(r"^(?:vecgeom::)?LogicalVolume\s+(\w+)\s*\(\s*\"[^\"]*\"\s*,\s*&\s*(\w+)\s*\)$", st)
        if m:
            if m.group(2) in self.shapes:
                self.lvs[m.group(1)] = m.group(2)
            return
        m = re.match(r"^(?:auto\s+)?(\w+)\s*=\s*(\w+)\s*\.\s*Place\s*\(\s*\)$", st)
        if m:
            if m.group(2) in self.lvs:
                self.shapes[m.group(1)] = self.shapes[self.lvs[m.group(2)]]
            return
        # vector declarations
        m = re.match(r"^(?:const\s+)?(?:Vec_t|Vector3D<[^>]*>|vecgeom::Vector3D<[^>]*>)\s+(.*)$", st, flags=re.S)
        if m:
            for decl in split_top(m.group(1)):
                mm = re.match(r"^(\w+)\s*\((.*)\)$", decl, flags=re.S)
                try:
                    if mm:
                        a = split_top(mm.group(2))
                        self.env[mm.group(1)] = V(*(float(self.ev(x)) for x in a)) if len(a) == 3 else self.ev(
                            mm.group(2))
                    else:
                        mm = re.match(r"^(\w+)\s*=\s*(.*)$", decl, flags=re.S)
                        if mm:
                            self.env[mm.group(1)] = self.ev(mm.group(2))
                        else:
                            self.env[decl] = V()
                            self.uninit.add(decl)  # declared without a value
                except Exception:
                    self.skipped += 1
            return
        # scalar declarations
        m = re.match(r"^(?:const\s+)?(?:static\s+)?(?:double|Precision|float|int|auto|bool|vecgeom::Precision)\s+(.*)$",
                     st, flags=re.S)
        if m and "(" not in m.group(1).split("=")[0]:
            for decl in split_top(m.group(1)):
                mm = re.match(r"^(\w+)\s*=\s*(.*)$", decl, flags=re.S)
                if mm:
                    qd = self.query_call(mm.group(2)) if "." in mm.group(2) or "->" in mm.group(2) else None
                    if qd:
                        self.results[mm.group(1)] = qd
                        continue
                    try:
                        self.env[mm.group(1)] = self.ev(mm.group(2))
                    except Exception:
                        self.results.pop(mm.group(1), None)
                        self.skipped += 1
            return
        # Inside_t / EInside declarations holding an Inside() result
        m = re.match(r"^(?:vecgeom::)?(?:Inside_t|EInside|int)\s+(\w+)\s*=\s*(.*)$", st, flags=re.S)
        if m:
            qd = self.query_call(m.group(2))
            if qd:
                self.results[m.group(1)] = qd
            return
        # compound assignment: evaluate, or forget the variable (its value is unknown,
        # e.g. it depends on a query result), so later uses are skipped, not wrong
        m = re.match(r"^(\w+)\s*([-+*/])=\s*(.*)$", st, flags=re.S)
        if m:
            var = m.group(1)
            try:
                self.env[var] = self.ev("(%s) %s (%s)" % (var, m.group(2), m.group(3)))
            except Exception:
                self.env.pop(var, None)
                self.skipped += 1
            self.results.pop(var, None)
            return
        # assignment of a query result or a scalar
        m = re.match(r"^(\w+)\s*=\s*(.*)$", st, flags=re.S)
        if m:
            var, rhs = m.group(1), m.group(2)
            self.uninit.discard(var)
            qd = None
            try:
                qd = self.query_call(rhs)
            except Exception:
                qd = None
            if qd:
                self.results[var] = qd
                return
            self.results.pop(var, None)
            try:
                self.env[var] = self.ev(rhs)
            except Exception:
                self.env.pop(var, None)
            return
        # shape.Extent(lo, hi): the two vectors become pending results (known answers follow)
        m = re.match(r"^(\w+)\s*(?:\.|->)\s*Extent\s*\(\s*(\w+)\s*,\s*(\w+)\s*\)$", st)
        if m:
            if m.group(1) in self.shapes:
                for var, q in ((m.group(2), "ExtentMin"), (m.group(3), "ExtentMax")):
                    self.results[var] = {"shape": m.group(1), "query": q, "p": None, "d": None}
                    self.env.pop(var, None)
            else:
                self.skipped += 1
            return
        # in-place vector mutators
        m = re.match(r"^(\w+)\s*\.\s*(Normalize|Set)\s*\((.*)\)$", st, flags=re.S)
        if m and isinstance(self.env.get(m.group(1)), V):
            if m.group(2) == "Normalize":
                self.env[m.group(1)] = self.env[m.group(1)].Unit()
            else:
                self.env[m.group(1)] = V(*(float(self.ev(a)) for a in split_top(m.group(3))))
            return
        m = re.match(r"^assert\s*\((.*)\)$", st, flags=re.S)
        if m:
            try:
                if not self.handle_assert(m.group(1), line):
                    self.skipped += 1
            except Exception:
                self.skipped += 1
            return

    def run(self, src):
        src = resolve_flag_blocks(strip_comments(src))
        # brace-initialised vectors: `Vec_t p{a, b, c}` -> `Vec_t p(a, b, c)`
        src = re.sub(r"(\bVec_t\s+\w+)\s*\{([^{}]*)\}", r"\1(\2)", src)
        # statements: split on ';' outside braces of initialisers, tracking line numbers
        pos, depth, start = 0, 0, 0
        stmts = []
        for i, ch in enumerate(src):
            if ch == "{":
                # an initialiser follows '=' (possibly with spaces)
                j = i - 1
                while j >= 0 and src[j] in " \t\n":
                    j -= 1
                if depth > 0 or (j >= 0 and src[j] == "="):
                    depth += 1
                else:
                    stmts.append((src[start:i], start))
                    start = i + 1
            elif ch == "}":
                if depth > 0:
                    depth -= 1
                else:
                    stmts.append((src[start:i], start))
                    start = i + 1
            elif ch == ";" and depth == 0:
                stmts.append((src[start:i], start))
                start = i + 1
        for st, off in stmts:
            st = st.strip()
            line = src.count("\n", 0, off) + 1
            # a control header (`if (...)`, `else`) is examined for soft checks, then dropped
            st = re.sub(r"^else\s*", "", st)
            m = re.match(r"^if\s*\(", st)
            if m:
                k, depth = m.end() - 1, 0
                for k2 in range(k, len(st)):
                    depth += st[k2] == "("
                    depth -= st[k2] == ")"
                    if depth == 0:
                        break
                try:
                    self.handle_condition(st[k + 1:k2], line)
                except Exception:
                    self.skipped += 1
                st = st[k2 + 1:].strip()
            if st.startswith("for") or st.startswith("while") or st.startswith("return"):
                self.skipped += 1
                continue
            try:
                self.statement(st, line)
            except Exception:
                self.skipped += 1


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VECGEOM_SOURCE_DIR")
    if not root:
        sys.exit("usage: extract_unit_vectors.py <VecGeom source tree> [output dir] "
                 "(or set VECGEOM_SOURCE_DIR)")
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.dirname(os.path.abspath(__file__))
    for shape, (fname, types) in FILES.items():
        path = os.path.join(root, "test", "unit_tests", fname)
        with open(path) as f:
            src = f.read()
        for name, body in MACROS.get(fname, []):
            src = re.sub(r"^\s*#define\s+%s\b[^\n]*$" % name, "", src, flags=re.M)
            src = re.sub(r"\b%s\b" % name, body, src)
        ex = Extractor(types)
        ex.run(src)
        doc = {"source": "test/unit_tests/" + fname, "shapes": ex.used_shapes, "cases": ex.cases,
               "skipped_statements": ex.skipped,
               "note": "line numbers count lines of the file after comments and disabled blocks were removed"}
        with open(os.path.join(out, "unit_%s.json" % shape), "w") as f:
            json.dump(doc, f, indent=0)
        print("%-9s %4d cases, %3d shapes, %4d statements skipped" % (shape, len(ex.cases), len(ex.used_shapes),
                                                                     ex.skipped))


if __name__ == "__main__":
    main()
