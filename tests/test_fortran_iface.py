"""The ISO_C_BINDING module (fortran/elbm_gb300_iface.f90) against the C header
(include/elbm_gb300.h), checked as text (no Fortran compiler is available):
every entry point of the header has an interface with the same bind(c) name,
the same number of arguments in the same order and a Fortran kind that
matches each C parameter (by value or by reference), and every bind(c)
derived type has the fields of its C struct in the same order, kinds and
element counts.  The constants the module exports have the header's values."""
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "elbm_gb300.h"
MODULE = ROOT / "university-of-cincinnati-lattice-boltzmann-solver_gb300" / "fortran" / "elbm_gb300_iface.f90"

STRUCTS = ("elbm_d3q27_params", "elbm_d3q39_params", "elbm_d3q39_bc", "elbm_plot3d_header", "elbm_stats")

# C scalar type -> Fortran kind
KIND = {"int": "c_int", "int32_t": "c_int32_t", "uint32_t": "c_int32_t", "int64_t": "c_int64_t",
        "uint64_t": "c_int64_t", "double": "c_double", "float": "c_float", "uint8_t": "c_int8_t", "char": "c_char"}


def _c_text():
    t = HEADER.read_text()
    t = re.sub(r"/\*.*?\*/", " ", t, flags=re.S)
    return re.sub(r"//[^\n]*", " ", t)


def c_functions():
    out = {}
    for m in re.finditer(r"(int|void|const\s+char\s*\*)\s+(elbm_\w+)\s*\(([^)]*)\)\s*;", _c_text()):
        ret, name, args = m.group(1), m.group(2), m.group(3)
        params = []
        for a in [x.strip() for x in args.split(",") if x.strip()]:
            a = re.sub(r"\bconst\b", "", a).strip()
            stars = a.count("*")
            base = a.replace("*", " ").split()[0]
            params.append((base, stars))
        out[name] = (re.sub(r"\s+", " ", ret), params)
    return out


def c_structs():
    out = {}
    for m in re.finditer(r"typedef\s+struct\s*\{(.*?)\}\s*(\w+)\s*;", _c_text(), re.S):
        fields = []
        for decl in [d.strip() for d in m.group(1).split(";") if d.strip()]:
            parts = decl.split(None, 1)
            base, rest = parts[0], parts[1]
            for item in [x.strip() for x in rest.split(",")]:
                dims = [int(x) for x in re.findall(r"\[(\d+)\]", item)]
                n = 1
                for d in dims:
                    n *= d
                fields.append((re.match(r"\w+", item).group(0), KIND[base], n))
        out[m.group(2)] = fields
    return out


def _f_lines():
    out, buf = [], ""
    for raw in MODULE.read_text().splitlines():
        s = raw.split("!", 1)[0].rstrip()
        if not s.strip():
            continue
        if buf:
            s = s.lstrip()
            if s.startswith("&"):
                s = s[1:]
        if s.endswith("&"):
            buf += s[:-1] + " "
            continue
        out.append((buf + s).strip().lower())
        buf = ""
    return out


def f_interfaces():
    lines = _f_lines()
    out, i = {}, 0
    head = re.compile(r"^(?:(integer\(c_int\)|type\(c_ptr\))\s+function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*"
                      r"bind\(c,\s*name=\"(\w+)\"\)$")
    while i < len(lines):
        m = head.match(lines[i])
        if not m:
            i += 1
            continue
        ret, name, args, cname = m.group(1), m.group(2), m.group(3), m.group(4)
        dummies = [a.strip() for a in args.split(",") if a.strip()]
        decl = {}
        i += 1
        while not re.match(r"^end\s+(function|subroutine)", lines[i]):
            d = lines[i]
            m2 = re.match(r"^(integer\((\w+)\)|real\((\w+)\)|type\((\w+)\)|character\(kind=(\w+)\))\s*(,[^:]*)?::(.*)$",
                          d)
            if m2:
                kind = m2.group(2) or m2.group(3) or m2.group(5) or m2.group(4)
                attrs = m2.group(6) or ""
                for item in re.findall(r"(\w+)\s*(\([^)]*\))?", m2.group(7)):
                    decl[item[0]] = (kind, "value" in attrs, bool(item[1]))
            i += 1
        out[cname] = (ret or "subroutine", name, [(a, decl.get(a)) for a in dummies])
        i += 1
    return out


def f_types():
    lines = _f_lines()
    out, i = {}, 0
    while i < len(lines):
        m = re.match(r"^type,\s*bind\(c\),\s*public\s*::\s*(\w+)$", lines[i])
        if not m:
            i += 1
            continue
        fields = []
        i += 1
        while lines[i] != "end type":
            m2 = re.match(r"^(?:integer|real)\((\w+)\)\s*::\s*(.*)$", lines[i])
            for name, dims in re.findall(r"(\w+)\s*(\([^)]*\))?", m2.group(2)):
                n = 1
                for d in re.findall(r"\d+", dims):
                    n *= int(d)
                fields.append((name, m2.group(1), n))
            i += 1
        out[m.group(1)] = fields
        i += 1
    return out


def f_constants():
    out = {}
    for s in _f_lines():
        m = re.match(r"^integer\(c_int\),\s*parameter,\s*public\s*::\s*(.*)$", s)
        if m:
            for name, val in re.findall(r"(\w+)\s*=\s*(-?\d+)", m.group(1)):
                out[name.upper()] = int(val)
    return out


def test_every_entry_point_is_bound():
    cf, fi = c_functions(), f_interfaces()
    assert len(cf) >= 40
    missing = sorted(set(cf) - set(fi))
    assert not missing, f"no Fortran interface for {missing}"
    assert not sorted(set(fi) - set(cf)), "interfaces without a C entry point"


@pytest.mark.parametrize("name", sorted(c_functions()))
def test_arguments_match(name):
    ret, params = c_functions()[name]
    fret, _, dummies = f_interfaces()[name]
    expect_ret = {"int": "integer(c_int)", "void": "subroutine", "const char *": "type(c_ptr)",
                  "const char*": "type(c_ptr)"}[ret]
    assert fret == expect_ret, (name, ret, fret)
    assert len(dummies) == len(params), (name, [d for d, _ in dummies], params)
    for (dname, decl), (base, stars) in zip(dummies, params):
        assert decl is not None, (name, dname, "not declared")
        kind, by_value, _ = decl
        if base == "elbm_ctx":
            assert kind == "c_ptr" and by_value == (stars == 1), (name, dname, decl)
        elif stars == 0:
            assert by_value and kind == KIND[base], (name, dname, decl, base)
        elif base in STRUCTS:
            assert kind == base and not by_value, (name, dname, decl)
        else:
            # by reference with the C element kind, or an explicit c_ptr passed by value (optional arrays)
            assert (kind == KIND[base] and not by_value) or (kind == "c_ptr" and by_value), (name, dname, decl, base)


@pytest.mark.parametrize("struct", STRUCTS)
def test_struct_layouts_match(struct):
    """Same kinds and element counts, field by field, in the same order (names may differ in case)."""
    c, f = c_structs()[struct], f_types()[struct]
    assert [(k, n) for _, k, n in c] == [(k, n) for _, k, n in f], (c, f)
    assert [x.lower() for x, _, _ in c] == [x for x, _, _ in f]


def test_constants_match():
    text = HEADER.read_text()
    defs = {m.group(1): int(m.group(2), 0) for m in re.finditer(r"#define\s+(ELBM_\w+)\s+(-?(?:0x[0-9a-f]+|\d+))u?",
                                                                 text, re.I)}
    fc = f_constants()
    assert len(fc) >= 20
    for name, val in fc.items():
        assert name in defs and defs[name] == val, (name, val, defs.get(name))
