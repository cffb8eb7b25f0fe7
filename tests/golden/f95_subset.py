"""A small interpreter for the subset of Fortran 95 the reference's hot-path
routines are written in, used only to generate golden fixtures: the
reference's own statements are run, in order, in float64 on seeded inputs,
and their results are compared with the oracle's restatement.

Supported: SUBROUTINE / FUNCTION (with RESULT) units found anywhere in a file
(module procedures included); declarations (scalars and arrays with explicit,
deferred or (lo:hi) bounds; PARAMETER values; OPTIONAL dummies with
PRESENT); assignment to scalars, array elements, sections and whole arrays;
block and logical IF; DO (counted, WHILE, bare) with EXIT / CYCLE; SELECT
CASE (values, ranges, DEFAULT); CALL with by-reference arguments; RETURN;
ALLOCATE / DEALLOCATE; array constructors (/ ... /); intrinsics (ABS, SQRT,
EXP, LOG, MAX, MIN, SUM, REAL, DBLE, INT, NINT, FLOOR, MOD, ISNAN, SIGN,
MAXVAL, MINVAL, SIZE, PRESENT, ANY, ALL) and elementwise comparisons of
array sections.  WRITE, PRINT, FORMAT and USE are no-ops; statement labels
are dropped (a caller rewrites the one GO TO it meets).

Arguments are passed as by reference: scalars and array elements are copied
in and written back only when the procedure assigned them (two dummies may
name one actual element, as outlet_bc's do on the shifted lattice), whole
arrays are shared, and an explicit-shape dummy array takes its declared
shape and bounds over the actual's elements (sequence association).

Arithmetic follows Fortran where the routines depend on it: integer / integer
truncates toward zero, and a real literal without a D exponent is a default
(single precision) REAL, rounded to float32 before it enters a float64
expression.  The source is case-folded; comments and continuation lines are
removed before parsing.
"""
from __future__ import annotations

import math
import re
from collections import ChainMap

import numpy as np


# ---------------------------------------------------------------------------
# values
# ---------------------------------------------------------------------------
class FInt(int):
    """A Fortran INTEGER: division truncates toward zero; results stay integers."""

    def _w(self, v):
        return FInt(v) if isinstance(v, int) and not isinstance(v, bool) else v

    def __add__(self, o):
        return self._w(int.__add__(self, o)) if isinstance(o, int) else float(self) + o

    __radd__ = __add__

    def __sub__(self, o):
        return self._w(int.__sub__(self, o)) if isinstance(o, int) else float(self) - o

    def __rsub__(self, o):
        return self._w(int.__rsub__(self, o)) if isinstance(o, int) else o - float(self)

    def __mul__(self, o):
        return self._w(int.__mul__(self, o)) if isinstance(o, int) else float(self) * o

    __rmul__ = __mul__

    def __truediv__(self, o):
        if isinstance(o, int):
            q = abs(int(self)) // abs(int(o))
            return FInt(q if (int(self) >= 0) == (int(o) >= 0) else -q)
        return float(self) / o

    def __rtruediv__(self, o):
        if isinstance(o, int):
            return FInt(o).__truediv__(self)
        return o / float(self)

    def __pow__(self, o):
        if isinstance(o, int):
            if int(o) < 0:
                return FInt(1 if abs(int(self)) == 1 else 0) if int(self) != 0 else float("inf")
            return FInt(int(self) ** int(o))
        return float(self) ** o

    def __rpow__(self, o):
        return o ** int(self)

    def __neg__(self):
        return FInt(-int(self))

    def __pos__(self):
        return self


def f32(x: float) -> float:
    """A default-kind REAL literal: its float32 value, exactly, as a float64."""
    return float(np.float32(x))


class FArray:
    """A Fortran array: numpy storage plus lower bounds; a(i, j) reads an
    element (or a section with slices), arithmetic acts on the whole array."""

    def __init__(self, data, lb=None):
        self.a = data
        self.lb = tuple(lb) if lb is not None else (1,) * data.ndim

    def _index(self, idx):
        out = []
        for k, i in enumerate(idx):
            lb = self.lb[k]
            if isinstance(i, slice):
                lo = lb if i.start is None else int(i.start)
                hi = (self.a.shape[k] + lb - 1) if i.stop is None else int(i.stop)
                out.append(slice(lo - lb, hi - lb + 1))
            else:
                j = int(i) - lb
                if not 0 <= j < self.a.shape[k]:
                    raise IndexError(f"index {int(i)} outside ({lb}:{self.a.shape[k] + lb - 1})")
                out.append(j)
        return tuple(out)

    def __call__(self, *idx):
        v = self.a[self._index(idx)]
        if isinstance(v, np.ndarray):
            return FArray(v)
        return FInt(int(v)) if self.a.dtype.kind in "iu" else float(v)

    def set(self, idx, value):
        self.a[self._index(idx)] = value.a if isinstance(value, FArray) else value

    def fill(self, value):
        self.a[...] = value.a if isinstance(value, FArray) else value

    # whole-array arithmetic
    def _bin(self, o, f):
        return FArray(f(self.a, o.a if isinstance(o, FArray) else o))

    def __add__(self, o):
        return self._bin(o, np.add)

    def __radd__(self, o):
        return self._bin(o, lambda a, b: b + a)

    def __sub__(self, o):
        return self._bin(o, np.subtract)

    def __rsub__(self, o):
        return self._bin(o, lambda a, b: b - a)

    def __mul__(self, o):
        return self._bin(o, np.multiply)

    def __rmul__(self, o):
        return self._bin(o, lambda a, b: b * a)

    def __truediv__(self, o):
        return self._bin(o, np.true_divide)

    def __pow__(self, o):
        return self._bin(o, np.power)

    def __neg__(self):
        return FArray(-self.a)

    # elementwise comparisons (for ANY / ALL over sections)
    def __lt__(self, o):
        return self._bin(o, np.less)

    def __le__(self, o):
        return self._bin(o, np.less_equal)

    def __gt__(self, o):
        return self._bin(o, np.greater)

    def __ge__(self, o):
        return self._bin(o, np.greater_equal)


def _S(lo, hi):
    return slice(lo, hi)


def _arr(items):
    flat = []
    for v in items:
        flat.extend(v.a.ravel().tolist() if isinstance(v, FArray) else [v])
    if all(isinstance(v, int) and not isinstance(v, bool) for v in flat):
        return FArray(np.array([int(v) for v in flat], np.int64))
    return FArray(np.array([float(v) for v in flat], np.float64))


def _val(x):
    return x.a if isinstance(x, FArray) else x


def _real(x, kind=None):
    if isinstance(x, FArray):
        return FArray(x.a.astype(np.float64))
    return float(x)


def _int(x, kind=None):
    if isinstance(x, FArray):
        return FArray(np.trunc(x.a).astype(np.int64))
    return FInt(math.trunc(x))


def _max(*a):
    vals = [float(v) if not isinstance(v, int) else v for v in a]
    m = max(vals)
    return FInt(m) if all(isinstance(v, int) for v in a) else float(m)


def _min(*a):
    vals = [float(v) if not isinstance(v, int) else v for v in a]
    m = min(vals)
    return FInt(m) if all(isinstance(v, int) for v in a) else float(m)


def _sum(x, dim=None):
    s = np.sum(_val(x))
    return FInt(int(s)) if np.asarray(_val(x)).dtype.kind in "iu" else float(s)


def _abs(x):
    if isinstance(x, FArray):
        return FArray(np.abs(x.a))
    return FInt(abs(int(x))) if isinstance(x, int) else abs(x)


def _mod(a, p):
    if isinstance(a, int) and isinstance(p, int):
        return FInt(int(math.fmod(int(a), int(p))))
    return math.fmod(a, p)


def _sign(a, b):
    return abs(a) if b >= 0 else -abs(a)


def _elemental(f):
    def g(x):
        return FArray(f(x.a)) if isinstance(x, FArray) else float(f(x))
    return g


INTRINSICS = {
    "abs": _abs, "dabs": _abs,
    "sqrt": _elemental(np.sqrt), "dsqrt": _elemental(np.sqrt),
    "exp": _elemental(np.exp), "dexp": _elemental(np.exp),
    "log": _elemental(np.log), "dlog": _elemental(np.log),
    "max": _max, "min": _min, "dmax1": _max, "dmin1": _min, "amax1": _max, "amin1": _min,
    "sum": _sum, "real": _real, "dble": _real, "int": _int,
    "nint": lambda x, kind=None: FInt(int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))),
    "floor": lambda x, kind=None: FInt(math.floor(x)),
    "mod": _mod, "isnan": lambda x: bool(math.isnan(x)), "sign": _sign,
    "maxval": lambda x: float(np.max(_val(x))), "minval": lambda x: float(np.min(_val(x))),
    "size": lambda x, dim=None: FInt(np.asarray(_val(x)).size if dim is None else np.asarray(_val(x)).shape[dim - 1]),
    "_S": _S, "_arr": _arr, "True": True, "False": False,
    "selected_real_kind": lambda p=6, r=37: FInt(8 if p > 6 or r > 37 else 4),
    "selected_int_kind": lambda r=9: FInt(8 if r > 9 else 4),
    "kind": lambda x: FInt(8),
    "any": lambda x: bool(np.any(_val(x))), "all": lambda x: bool(np.all(_val(x))),
}

PY_RESERVED = {"lambda", "in", "is", "if", "else", "for", "while", "and", "or", "not", "def", "class", "return",
               "import", "from", "as", "with", "try", "except", "pass", "print", "global", "del", "yield", "raise",
               "finally", "none", "true", "false", "assert", "break", "continue", "elif", "async", "await",
               "nonlocal"}


def pyname(n: str) -> str:
    return "v_" + n if n in PY_RESERVED else n


# ---------------------------------------------------------------------------
# source -> logical lines
# ---------------------------------------------------------------------------
def _strip_comment(line: str) -> str:
    out, q = [], None
    for ch in line:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        elif ch == "!":
            break
        else:
            out.append(ch)
    return "".join(out).rstrip()


def logical_lines(text: str):
    """(first physical line number, statement) pairs: comments dropped,
    continuations joined, case folded, ';'-separated statements split."""
    out, buf, start = [], "", None
    for no, raw in enumerate(text.splitlines(), 1):
        s = _strip_comment(raw).strip()
        if not s:
            continue
        if buf and s.startswith("&"):
            s = s[1:].lstrip()
        if start is None:
            start = no
        if s.endswith("&"):
            buf += s[:-1] + " "
            continue
        buf += s
        for part in buf.split(";"):
            part = re.sub(r"^\d+\s+", "", part.strip())  # statement label
            if part:
                out.append((start, part.lower()))
        buf, start = "", None
    return out


# ---------------------------------------------------------------------------
# expressions
# ---------------------------------------------------------------------------
_TOK = re.compile(r"""
    (?P<ws>\s+)
  | (?P<real>(\d+\.\d*|\.\d+|\d+)([de][+-]?\d+)(_\w+)? | (\d+\.\d*|\.\d+)(_\w+)?)
  | (?P<int>\d+)
  | (?P<dotop>\.(and|or|not|eq|ne|lt|le|gt|ge|true|false|eqv|neqv)\.)
  | (?P<arrl>\(/)
  | (?P<arrr>/\))
  | (?P<op>\*\*|==|/=|<=|>=|<|>|\*|/|\+|-|\(|\)|,|:|=|%)
  | (?P<name>[a-z_][a-z0-9_]*)
  | (?P<str>'[^']*'|"[^"]*")
""", re.X)

_DOTOPS = {".and.": " and ", ".or.": " or ", ".not.": " not ", ".eq.": "==", ".ne.": "!=", ".lt.": "<",
           ".le.": "<=", ".gt.": ">", ".ge.": ">=", ".true.": "True", ".false.": "False", ".eqv.": "==",
           ".neqv.": "!="}


def tokens(s: str):
    pos, out = 0, []
    while pos < len(s):
        m = _TOK.match(s, pos)
        if not m:
            raise SyntaxError(f"cannot tokenise {s[pos:pos + 20]!r} in {s!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind != "ws":
            out.append((kind, m.group(kind)))
    return out


def _real_literal(t: str) -> str:
    m = re.fullmatch(r"(\d+\.\d*|\.\d+|\d+)(?:([de])([+-]?\d+))?(?:_(\w+))?", t)
    mant, ek, ex, kind = m.groups()
    v = float(mant + ("e" + ex if ex else ""))
    if ek == "d" or kind is not None:
        return repr(v)
    return repr(f32(v))


def translate(expr: str) -> str:
    """Fortran expression -> Python expression over FInt/FArray values."""
    toks = tokens(expr)
    out = []
    depth_kinds = []  # per open paren: True if inside an array-ref/call argument list
    for k, (kind, t) in enumerate(toks):
        if kind == "real":
            out.append(_real_literal(t))
        elif kind == "int":
            out.append(f"FInt({t})")
        elif kind == "dotop":
            out.append(_DOTOPS[t])
        elif kind == "arrl":
            out.append("_arr([")
            depth_kinds.append("arr")
        elif kind == "arrr":
            out.append("])")
            depth_kinds.pop()
        elif kind == "name":
            if t == "present" and k + 3 < len(toks) and toks[k + 1][1] == "(" and toks[k + 3][1] == ")":
                out.append("_present")
                toks[k + 2] = ("str", repr(pyname(toks[k + 2][1])))
            else:
                out.append(pyname(t))
        elif kind == "str":
            out.append(t)
        else:  # op
            if t == "(":
                prev = toks[k - 1] if k else None
                is_call = prev is not None and prev[0] == "name"
                depth_kinds.append("call" if is_call else "paren")
                out.append("(")
            elif t == ")":
                depth_kinds.pop()
                out.append(")")
            elif t == "/=":
                out.append("!=")
            elif t == ":":
                out.append(":")
            elif t == "%":
                raise SyntaxError(f"derived-type component in {expr!r}")
            else:
                out.append(t)
    py = "".join(out).strip()
    return _slices(py)


def _split_args(inner: str):
    parts, level, cur = [], 0, ""
    for c in inner:
        if c in "([":
            level += 1
        elif c in ")]":
            level -= 1
        if c == "," and level == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += c
    parts.append(cur)
    return parts


def _slices(s: str) -> str:
    """Inside parenthesised argument lists, a:b -> _S(a, b) (either side may be empty)."""
    pairs, st = {}, []
    for i, c in enumerate(s):
        if c == "(":
            st.append(i)
        elif c == ")":
            pairs[st.pop()] = i

    def build(a, b):
        out, k = [], a
        while k < b:
            if s[k] == "(":
                e = pairs[k]
                out.append("(" + conv(build(k + 1, e)) + ")")
                k = e + 1
            else:
                out.append(s[k])
                k += 1
        return "".join(out)

    def conv(inner):
        new = []
        for p in _split_args(inner):
            lvl, pos = 0, -1
            for q, c in enumerate(p):
                if c in "([":
                    lvl += 1
                elif c in ")]":
                    lvl -= 1
                elif c == ":" and lvl == 0:
                    pos = q
                    break
            if pos >= 0:
                lo, hi = p[:pos].strip(), p[pos + 1:].strip()
                new.append(f"_S({lo or 'None'}, {hi or 'None'})")
            else:
                new.append(p)
        return ",".join(new)

    return build(0, len(s))


# ---------------------------------------------------------------------------
# statements
# ---------------------------------------------------------------------------
def split_paren(s: str, start: int):
    """Index just past the parenthesis group that opens at s[start] == '('."""
    depth = 0
    for i in range(start, len(s)):
        if s[i] == "(":
            depth += 1
        elif s[i] == ")":
            depth -= 1
            if depth == 0:
                return i + 1
    raise SyntaxError(f"unbalanced parentheses in {s!r}")


def split_top(s: str, sep=","):
    parts, depth, cur, q = [], 0, "", None
    for c in s:
        if q:
            cur += c
            if c == q:
                q = None
            continue
        if c in "'\"":
            q = c
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
        if c == sep and depth == 0:
            parts.append(cur.strip())
            cur = ""
        else:
            cur += c
    if cur.strip():
        parts.append(cur.strip())
    return parts


class Node:
    def __init__(self, kind, line, **kw):
        self.kind, self.line = kind, line
        self.__dict__.update(kw)


_DECL = re.compile(r"^(real|integer|logical|double\s+precision|character|type\s*\()")
_NOOP = re.compile(r"^(use\b|implicit\b|save\b|private\b|public\b|write\s*\(|print\b|format\b|continue$|"
                   r"include\b|contains$|intrinsic\b|external\b|nullify\b|end\s*$|flush\b)")


def parse_block(lines, i, enders):
    """Parse statements from lines[i] until one matching `enders` (a regex);
    returns (list of nodes, index of the ending line)."""
    body = []
    while i < len(lines):
        no, s = lines[i]
        if re.match(enders, s):
            return body, i
        node, i = parse_stmt(lines, i)
        if node is not None:
            body.append(node)
    raise SyntaxError(f"missing end matching {enders}")


def parse_stmt(lines, i):
    no, s = lines[i]
    if _NOOP.match(s):
        return None, i + 1
    if _DECL.match(s) and "::" in s:
        return Node("decl", no, text=s), i + 1
    if re.match(r"^(real|integer|logical|double\s+precision)\b", s) and not re.match(r"^\w+\s*\(.*\)\s*=", s):
        return Node("decl", no, text=s), i + 1
    m = re.match(r"^if\s*\(", s)
    if m:
        e = split_paren(s, s.index("("))
        cond, rest = s[s.index("(") + 1:e - 1], s[e:].strip()
        if rest == "then":
            arms = []
            body, j = parse_block(lines, i + 1, r"^(else\s*if\s*\(.*\)\s*then|else$|end\s*if)")
            arms.append((cond, body))
            while True:
                _, t = lines[j]
                if re.match(r"^end\s*if", t):
                    return Node("if", no, arms=arms), j + 1
                if t == "else":
                    body, j = parse_block(lines, j + 1, r"^end\s*if")
                    arms.append((None, body))
                    continue
                e2 = split_paren(t, t.index("("))
                c2 = t[t.index("(") + 1:e2 - 1]
                body, j = parse_block(lines, j + 1, r"^(else\s*if\s*\(.*\)\s*then|else$|end\s*if)")
                arms.append((c2, body))
        sub, _ = parse_stmt([(no, rest)], 0)
        return Node("if", no, arms=[(cond, [sub] if sub else [])]), i + 1
    m = re.match(r"^do\s+while\s*\((.*)\)$", s)
    if m:
        body, j = parse_block(lines, i + 1, r"^end\s*do")
        return Node("dowhile", no, cond=m.group(1), body=body), j + 1
    m = re.match(r"^do\s+(\w+)\s*=\s*(.*)$", s)
    if m:
        parts = split_top(m.group(2))
        body, j = parse_block(lines, i + 1, r"^end\s*do")
        return Node("do", no, var=m.group(1), lo=parts[0], hi=parts[1], step=parts[2] if len(parts) > 2 else None,
                    body=body), j + 1
    if s == "do":
        body, j = parse_block(lines, i + 1, r"^end\s*do")
        return Node("dowhile", no, cond=".true.", body=body), j + 1
    m = re.match(r"^select\s+case\s*\((.*)\)$", s)
    if m:
        cases = []
        j = i + 1
        while not re.match(r"^end\s*select", lines[j][1]):
            t = lines[j][1]
            if re.match(r"^case\s+default", t):
                sel = None
            else:
                mm = re.match(r"^case\s*\((.*)\)$", t)
                if not mm:
                    raise SyntaxError(f"line {lines[j][0]}: {t!r}")
                sel = split_top(mm.group(1))
            body, j = parse_block(lines, j + 1, r"^(case\b|end\s*select)")
            cases.append((sel, body))
        return Node("select", no, expr=m.group(1), cases=cases), j + 1
    m = re.match(r"^call\s+(\w+)\s*(\((.*)\))?$", s)
    if m:
        return Node("call", no, name=m.group(1), args=split_top(m.group(3) or "")), i + 1
    if s in ("return", "exit", "cycle"):
        return Node(s, no), i + 1
    if s.startswith("stop"):
        return Node("stop", no, text=s), i + 1
    m = re.match(r"^(allocate|deallocate)\s*\((.*)\)$", s)
    if m:
        return Node(m.group(1), no, items=split_top(m.group(2))), i + 1
    # assignment
    depth = 0
    for k, c in enumerate(s):
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
        elif c == "=" and depth == 0 and s[k + 1:k + 2] != "=" and s[k - 1:k] not in ("<", ">", "/", "="):
            return Node("assign", no, lhs=s[:k].strip(), rhs=s[k + 1:].strip()), i + 1
    raise SyntaxError(f"line {no}: unsupported statement {s!r}")


class Proc:
    def __init__(self, kind, name, args, result, body, decls, line):
        self.kind, self.name, self.args, self.result, self.body, self.decls, self.line = (
            kind, name, args, result, body, decls, line)


_UNIT = re.compile(r"^(?:(?:recursive|pure|elemental)\s+)*(?:(?:real|integer|logical)(?:\s*\([^)]*\))?\s+)?"
                   r"(subroutine|function)\s+(\w+)\s*(?:\(([^)]*)\))?\s*(?:result\s*\((\w+)\))?$")


def parse_units(lines, only=None):
    """The SUBROUTINE and FUNCTION units of a file; with `only`, the named ones
    (the others are skipped up to their END SUBROUTINE / END FUNCTION)."""
    procs, i = {}, 0
    while i < len(lines):
        no, s = lines[i]
        m = _UNIT.match(s)
        if not m:
            i += 1
            continue
        kind, name, args, result = m.groups()
        if only is not None and name not in only:
            j = i + 1
            while j < len(lines) and not re.match(rf"^end\s*{kind}\b", lines[j][1]):
                j += 1
            i = j + 1
            continue
        body, j = parse_block(lines, i + 1, rf"^end\s*({kind}\b|$)|^end$")
        decls = [n for n in body if n.kind == "decl"]
        procs[name] = Proc(kind, name, [a.strip() for a in (args or "").split(",") if a.strip()],
                           result or name, [n for n in body if n.kind != "decl"], decls, no)
        i = j + 1
    return procs


# ---------------------------------------------------------------------------
# execution
# ---------------------------------------------------------------------------
class _Return(Exception):
    pass


class _Exit(Exception):
    pass


class _Cycle(Exception):
    pass


class Ref:
    """A by-reference actual argument: a variable of a scope, or an array element."""

    def __init__(self, scope, name, idx=None):
        self.scope, self.name, self.idx = scope, name, idx

    def get(self):
        v = self.scope[self.name]
        return v(*self.idx) if self.idx is not None else v

    def set(self, v):
        if self.idx is not None:
            self.scope[self.name].set(self.idx, v)
        elif isinstance(self.scope.get(self.name), FArray) and isinstance(v, FArray):
            self.scope[self.name].fill(v)
        else:
            self.scope[self.name] = v


class Interp:
    def __init__(self, procs: dict, globals_: dict):
        self.procs = procs
        self.globals = globals_
        self._code = {}

    # -- expressions --
    def ev(self, expr: str, scope):
        code = self._code.get(expr)
        if code is None:
            code = compile(translate(expr), f"<{expr}>", "eval")
            self._code[expr] = code
        return eval(code, {"FInt": FInt, "__builtins__": {}}, scope)

    def scope_for(self, local):
        funcs = {n: self._callable(n) for n, p in self.procs.items() if isinstance(p, Proc) and p.kind == "function"}
        return ChainMap(local, self.globals, funcs, INTRINSICS)

    def _callable(self, name):
        def f(*args, **kw):
            return self.call(name, list(args), kw)
        return f

    # -- declarations --
    def declare(self, decl: str, local, scope, dummies):
        head, _, rest = decl.partition("::")
        if not _:
            m = re.match(r"^(real(?:\s*\([^)]*\))?|integer(?:\s*\([^)]*\))?|logical|double\s+precision)\s+(.*)$",
                         decl)
            head, rest = m.group(1), m.group(2)
        head = head.strip()
        is_int = head.startswith("integer")
        is_log = head.startswith("logical")
        is_param = "parameter" in head
        dim_attr = re.search(r"dimension\s*\(([^)]*)\)", head)
        for item in split_top(rest):
            init = None
            if "=" in item and not item.split("=")[0].strip().endswith(("<", ">", "/")):
                item, init = item.split("=", 1)
                item, init = item.strip(), init.strip()
            m = re.match(r"^(\w+)\s*(\((.*)\))?$", item)
            name, dims = m.group(1), m.group(3) or (dim_attr.group(1) if dim_attr else None)
            pname = pyname(name)
            if pname in dummies:
                # an explicit-shape dummy array takes its declared shape and bounds over the actual's
                # elements (sequence association: a section a(i,j,k,1:n) passed to b(i:i,j:j,k:k,1:n))
                act = local.get(pname)
                if dims is not None and isinstance(act, FArray) and not re.fullmatch(r"[:,\s*]*", dims):
                    shape, lbs = [], []
                    for d in split_top(dims):
                        if ":" in d:
                            lo, hi = d.split(":")
                            lo_v = int(self.ev(lo, scope)) if lo.strip() else 1
                            hi_v = int(self.ev(hi, scope))
                        else:
                            lo_v, hi_v = 1, int(self.ev(d, scope))
                        shape.append(hi_v - lo_v + 1)
                        lbs.append(lo_v)
                    if int(np.prod(shape)) == act.a.size and (tuple(shape) != act.a.shape or tuple(lbs) != act.lb):
                        data = act.a if tuple(shape) == act.a.shape else act.a.reshape(shape, order="F")
                        local[pname] = FArray(data, lbs)
                continue
            if dims is not None and not re.fullmatch(r"[:,\s]*", dims):
                shape, lbs = [], []
                for d in split_top(dims):
                    if ":" in d:
                        lo, hi = d.split(":")
                        lo_v = int(self.ev(lo, scope)) if lo.strip() else 1
                        hi_v = int(self.ev(hi, scope))
                    else:
                        lo_v, hi_v = 1, int(self.ev(d, scope))
                    shape.append(hi_v - lo_v + 1)
                    lbs.append(lo_v)
                arr = np.zeros(shape, np.int64) if is_int else (
                    np.zeros(shape, bool) if is_log else np.full(shape, np.nan))
                local[pname] = FArray(arr, lbs)
                if init is not None:
                    local[pname].fill(self.ev(init, scope))
            elif dims is not None:
                local[pname] = None  # allocatable / deferred shape: set at ALLOCATE
            else:
                if init is not None:
                    v = self.ev(init, scope)
                    local[pname] = FInt(int(v)) if is_int else (bool(v) if is_log else float(v))
                else:
                    local[pname] = FInt(0) if is_int else (False if is_log else float("nan"))
            if is_param:
                pass

    # -- calls --
    def call(self, name, actuals, kw=None):
        p = self.procs[name]
        if not isinstance(p, Proc):  # a Python stand-in (e.g. a recording wrapper)
            return p(*actuals, **(kw or {}))
        return self.call_proc(p, actuals, kw)

    def call_proc(self, p, actuals, kw=None):
        local = {}
        dummies = {pyname(a) for a in p.args}
        present = set()
        refs = {}
        entry = {}
        for a, v in zip(p.args, actuals):
            if isinstance(v, Ref):
                refs[pyname(a)] = v
                local[pyname(a)] = entry[pyname(a)] = v.get()
            else:
                local[pyname(a)] = v
            present.add(pyname(a))
        for a, v in (kw or {}).items():
            local[a] = v
            present.add(a)
        for a in p.args:
            if pyname(a) not in local:
                local[pyname(a)] = None
        scope = self.scope_for(local)
        local["_present"] = lambda nm, _p=present: nm in _p
        for d in p.decls:
            self.declare(d.text, local, scope, dummies)
        if p.kind == "function" and pyname(p.result) not in local:
            local[pyname(p.result)] = float("nan")
        try:
            self.run(p.body, local, scope)
        except _Return:
            pass
        # copy-out of the arguments the procedure assigned: an argument passed by reference that
        # the procedure leaves alone does not write (two dummies may name one actual element, as
        # outlet_bc's fout_outl and fout_opp do on the shifted lattice, where opp(i) = i)
        for a, r in refs.items():
            new, old = local[a], entry[a]
            if new is old or (not isinstance(new, FArray) and type(new) is type(old) and new == old):
                continue
            r.set(new)
        if p.kind == "function":
            return local[pyname(p.result)]
        return None

    def _actual(self, expr, scope):
        m = re.fullmatch(r"(\w+)", expr.strip())
        if m and pyname(m.group(1)) in scope and not callable(scope[pyname(m.group(1))]):
            owner = _owner(scope, pyname(m.group(1)))
            return Ref(owner, pyname(m.group(1)))
        m = re.fullmatch(r"(\w+)\s*\((.*)\)", expr.strip())
        if m and isinstance(scope.get(pyname(m.group(1))), FArray) and ":" not in m.group(2):
            owner = _owner(scope, pyname(m.group(1)))
            idx = tuple(self.ev(x, scope) for x in split_top(m.group(2)))
            return Ref(owner, pyname(m.group(1)), idx)
        return self.ev(expr, scope)

    # -- statements --
    def assign(self, lhs, value, local, scope):
        m = re.fullmatch(r"(\w+)\s*(\((.*)\))?", lhs)
        name = pyname(m.group(1))
        owner = _owner(scope, name)
        if m.group(2):
            idx = tuple(self.ev(x, scope) if ":" not in x else self._slice(x, scope) for x in split_top(m.group(3)))
            owner[name].set(idx, value)
        else:
            cur = owner.get(name)
            if isinstance(cur, FArray):
                cur.fill(value)
            elif isinstance(cur, FInt) or (isinstance(cur, int) and not isinstance(cur, bool)):
                owner[name] = FInt(math.trunc(value)) if not isinstance(value, bool) else value
            elif isinstance(cur, float) and isinstance(value, int) and not isinstance(value, bool):
                owner[name] = float(value)
            else:
                owner[name] = value

    def _slice(self, x, scope):
        lo, hi = x.split(":")
        return slice(self.ev(lo, scope) if lo.strip() else None, self.ev(hi, scope) if hi.strip() else None)

    def run(self, body, local, scope):
        for n in body:
            k = n.kind
            try:
                if k == "assign":
                    self.assign(n.lhs, self.ev(n.rhs, scope), local, scope)
                elif k == "if":
                    for cond, blk in n.arms:
                        if cond is None or self.ev(cond, scope):
                            self.run(blk, local, scope)
                            break
                elif k == "do":
                    lo, hi = int(self.ev(n.lo, scope)), int(self.ev(n.hi, scope))
                    st = int(self.ev(n.step, scope)) if n.step else 1
                    owner = _owner(scope, pyname(n.var))
                    v = lo
                    while (v <= hi) if st > 0 else (v >= hi):
                        owner[pyname(n.var)] = FInt(v)
                        try:
                            self.run(n.body, local, scope)
                        except _Cycle:
                            pass
                        except _Exit:
                            break
                        v += st
                    else:
                        owner[pyname(n.var)] = FInt(v)
                elif k == "dowhile":
                    guard = 0
                    while self.ev(n.cond, scope):
                        guard += 1
                        if guard > 10_000_000:
                            raise RuntimeError(f"line {n.line}: loop did not end")
                        try:
                            self.run(n.body, local, scope)
                        except _Cycle:
                            pass
                        except _Exit:
                            break
                elif k == "select":
                    v = self.ev(n.expr, scope)
                    for sel, blk in n.cases:
                        if sel is None or any(_case_match(v, c, self, scope) for c in sel):
                            self.run(blk, local, scope)
                            break
                elif k == "call":
                    if n.name not in self.procs:
                        hook = self.globals.get("__call_" + n.name)
                        if hook is None:
                            raise KeyError(f"line {n.line}: no subroutine {n.name}")
                        hook(*[self.ev(a, scope) for a in n.args])
                        continue
                    acts, kws = [], {}
                    target = self.procs[n.name]
                    dummies = {pyname(x) for x in target.args} if isinstance(target, Proc) else set()
                    for a in n.args:
                        mm = re.fullmatch(r"(\w+)\s*=\s*(.*)", a)
                        if mm and mm.group(1) in dummies:
                            kws[mm.group(1)] = self.ev(mm.group(2), scope)
                        else:
                            acts.append(self._actual(a, scope))
                    self.call(n.name, acts, kws)
                elif k == "return":
                    raise _Return()
                elif k == "exit":
                    raise _Exit()
                elif k == "cycle":
                    raise _Cycle()
                elif k == "stop":
                    raise RuntimeError(f"line {n.line}: {n.text}")
                elif k == "allocate":
                    for it in n.items:
                        mm = re.fullmatch(r"(\w+)\s*\((.*)\)", it)
                        name = pyname(mm.group(1))
                        shape, lbs = [], []
                        for d in split_top(mm.group(2)):
                            if ":" in d:
                                lo_s, hi_s = d.split(":")
                                lo_v, hi_v = int(self.ev(lo_s, scope)), int(self.ev(hi_s, scope))
                            else:
                                lo_v, hi_v = 1, int(self.ev(d, scope))
                            shape.append(hi_v - lo_v + 1)
                            lbs.append(lo_v)
                        ints = self.globals.get("__int_arrays", set())
                        data = np.zeros(shape, np.int64) if name in ints else np.full(shape, np.nan)
                        _owner(scope, name)[name] = FArray(data, lbs)
                elif k == "deallocate":
                    pass
                else:
                    raise RuntimeError(f"line {n.line}: cannot run {k}")
            except (_Return, _Exit, _Cycle):
                raise
            except Exception as e:
                if not getattr(e, "_located", False):
                    e.args = (f"line {n.line}: {e}",) + e.args[1:]
                    e._located = True
                raise


def _owner(scope: ChainMap, name: str):
    """The scope level holding a name; a name declared nowhere is a module variable."""
    for m in scope.maps:
        if name in m:
            return m
    return scope.maps[1] if len(scope.maps) > 1 else scope.maps[0]


def _case_match(v, c, interp, scope):
    if ":" in c:
        lo, hi = c.split(":")
        return (not lo.strip() or v >= interp.ev(lo, scope)) and (not hi.strip() or v <= interp.ev(hi, scope))
    return v == interp.ev(c, scope)


def load_procs(*paths) -> dict:
    procs = {}
    for p in paths:
        procs.update(parse_units(logical_lines(open(p).read())))
    return procs


def module_parameters(path, scope=None) -> dict:
    """PARAMETER values declared in a module file (evaluated in order)."""
    out = {}
    interp = Interp({}, {})
    sc = ChainMap(out, scope or {}, INTRINSICS)
    for no, s in logical_lines(open(path).read()):
        if "parameter" in s and "::" in s and _DECL.match(s):
            interp.declare(s, out, sc, set())
    return out
