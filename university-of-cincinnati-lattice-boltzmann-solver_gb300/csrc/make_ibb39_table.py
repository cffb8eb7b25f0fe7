"""Generates ibb39_table.h: the non-equilibrium parts of the D3Q39 interpolated
wall closure on the unshifted lattice as coefficient tables.

The reference writes that closure (interpolative_bounceback_bc.f95:834-2838,
one `case` per direction 2..39) as hand-expanded formulas, each with its own
grouping and its own deviations from the generic Grad form (for example
`3/cv_const` where cv_const = 1/const_vol).  To reproduce them exactly without
per-direction code, this script reads the formulas, expands them with sympy
into sums of monomials and writes, per direction, the exact coefficients:

  fi_neq = k_fi * sum_t c_t * D_t * u^a v^b w^c * T^e * beta_1^p * beta_2^q * C_v^r
  gi_neq = k_gi * (the same form with its own terms)

D_t is one of the twelve wall-stencil derivatives (du/dx .. dT/dz) and T the
target temperature.  Each term's exponents are packed into one int32:
derivative (bits 0-3), u, v, w (2 bits each from bit 4), T + 4 (3 bits from
bit 10), beta_1 + 2, beta_2 + 2 (2 bits each from bit 13), C_v + 2 (3 bits
from bit 17).  The derivative rule of each direction (which derivatives are
the one-sided wall form, up or down) is checked against the rule the library
implements: wall form on the axes where the direction has a component, "up"
when that component is positive.

Run:  python make_ibb39_table.py <reference root>   (rewrites ibb39_table.h)
"""
from __future__ import annotations

import pathlib
import re
import sys

import sympy as sp

HERE = pathlib.Path(__file__).resolve().parent
SRC_REL = "boundary_conditions/interpolative_bc/interpolative_bounceback_bc.f95"
FIRST, LAST = 834, 2838  # 1-based lines of the unshifted D3Q39 cases
DERIVS = ["dudx", "dudy", "dudz", "dvdx", "dvdy", "dvdz", "dwdx", "dwdy", "dwdz", "dTdx", "dTdy", "dTdz"]
# unshifted D3Q39 velocities, 1-based direction order of the reference
CX = [0, 1, 0, 0, -1, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 2, 0, 0, -2, 0, 0, 2, 2, 0, -2, -2, 2, 2, -2, -2, 0, 0, 0,
      3, 0, 0, -3, 0, 0]
CY = [0, 0, 1, 0, 0, -1, 0, 1, 1, -1, -1, 1, 1, -1, -1, 0, 2, 0, 0, -2, 0, 2, 0, 2, 2, -2, -2, 0, 0, 0, 2, -2, -2,
      0, 3, 0, 0, -3, 0]
CZ = [0, 0, 0, 1, 0, 0, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 2, 0, 0, -2, 0, 2, 2, 0, 0, 0, -2, -2, 2, -2, -2, 2,
      0, 0, 3, 0, 0, -3]


def parse_cases(path: pathlib.Path):
    """{direction (1-based): (derivative calls, [(lhs, rhs), ...])} from the case blocks."""
    lines = path.read_text().splitlines()[FIRST - 1:LAST]
    stmts, buf = [], ""
    for ln in lines:
        s = ln.split("!")[0].rstrip()
        if not s.strip():
            continue
        s = (buf + " " + s.strip()) if buf else s.strip()
        buf = ""
        if s.endswith("&"):
            buf = s[:-1]
            continue
        stmts.append(s)
    cases, cur = {}, None
    for s in stmts:
        m = re.match(r"case\s*\((\d+)\)", s, re.I)
        if m:
            cur = int(m.group(1))
            cases[cur] = ({}, [])
            continue
        if re.match(r"end select", s, re.I):
            cur = None
            continue
        if cur is None:
            continue
        lhs, rhs = (x.strip() for x in s.split("=", 1))
        if lhs in DERIVS:
            m = re.match(r"(d\w+?)_(ibb|local)\((.*)\)$", rhs)
            if not m or m.group(1) != lhs:
                raise ValueError(f"case {cur}: unexpected derivative call {s}")
            cases[cur][0][lhs] = (m.group(2), m.group(3).replace(" ", ""))
        else:
            cases[cur][1].append((lhs, rhs))
    return cases


def check_rule(d: int, calls) -> None:
    """The derivative calls of direction d follow the library's unshifted wall rule."""
    comp = {"x": CX[d - 1], "y": CY[d - 1], "z": CZ[d - 1]}
    nb = {"x": ("5", "2"), "y": ("6", "3"), "z": ("7", "4")}
    for name, (kind, args) in calls.items():
        q, ax = name[1:-2], name[-1]
        c = comp[ax]
        if c != 0:
            tgt = "temp_tgt" if q == "T" else f"{q}_tgt"
            wall = "temp_tgt" if q == "T" else "0.0D0"
            want = ",".join([tgt, wall, "upwind" if c > 0 else "downwind", "dir_state", "i"])
            if kind != "ibb" or args != want:
                raise ValueError(f"direction {d} {name}: {kind} {args}")
        else:
            loc = "loc_temp" if q == "T" else f"loc_{q}"
            up, down = nb[ax]
            want = ",".join([f"{loc}(1)", f"{loc}({up})", f"{loc}({down})", "rest_state(a,b,c,1)",
                             f"rest_state(a,b,c,{up})", f"rest_state(a,b,c,{down})"])
            if kind != "local" or args != want:
                raise ValueError(f"direction {d} {name}: {kind} {args}")


SYM = {d: sp.Symbol(d) for d in DERIVS}
T, U, V, W, B1, B2, C = sp.symbols("temp_tgt u_tgt v_tgt w_tgt beta_1 beta_2 const_vol")
KFI, KGI, FEQ, GEQ, EPS = sp.symbols("k_fi k_gi loc_fieq loc_gieq loc_epsilon")


def _sympify(rhs: str) -> str:
    rhs = re.sub(r"(\d+\.\d*)[dD]([+-]?\d+)", lambda m: "Rational('%s')" % sp.nsimplify(float(m.group(1) + "e" +
                                                                                             m.group(2))), rhs)
    return re.sub(r"(?<![\w.'])(\d+)(?![\w.'])", r"Integer(\1)", rhs)


def expand_case(exprs):
    env = dict(SYM, temp_tgt=T, u_tgt=U, v_tgt=V, w_tgt=W, beta_1=B1, beta_2=B2, const_vol=C, cv_const=1 / C,
               cv_const_2=2 / C, k_fi=KFI, k_gi=KGI, loc_fieq=FEQ, loc_gieq=GEQ, loc_epsilon=EPS,
               dimensions=sp.Integer(3))
    for lhs, rhs in exprs:
        env[lhs] = eval(_sympify(rhs), {"Rational": sp.Rational, "Integer": sp.Integer}, env)
    fn = sp.expand((env["loc_fout"] - FEQ) / (EPS * KFI))
    gn = sp.expand((env["loc_gout"] - GEQ) / (EPS * KGI))
    for e in (fn, gn):
        if e.has(EPS) or e.has(KFI) or e.has(KGI) or e.has(FEQ) or e.has(GEQ):
            raise ValueError("closure not of the form f_eq + eps k (...)")
    return fn, gn


def terms(expr):
    out = []
    for t in expr.as_ordered_terms():
        coeff, rest = t.as_coeff_Mul()
        pw = rest.as_powers_dict()
        ds = [k for k in range(12) if SYM[DERIVS[k]] in pw]
        if len(ds) != 1 or pw[SYM[DERIVS[ds[0]]]] != 1:
            raise ValueError(f"term {t} is not linear in one derivative")
        e = [int(pw.get(s, 0)) for s in (U, V, W, T, B1, B2, C)]
        known = {SYM[DERIVS[ds[0]]], U, V, W, T, B1, B2, C}
        if any(s not in known for s in pw):
            raise ValueError(f"term {t}: unexpected symbol")
        eu, ev, ew, eT, eb1, eb2, eC = e
        if not (0 <= eu <= 3 and 0 <= ev <= 3 and 0 <= ew <= 3 and -4 <= eT <= 3 and -2 <= eb1 <= 1 and
                -2 <= eb2 <= 1 and -2 <= eC <= 5):
            raise ValueError(f"term {t}: exponents out of the packed range")
        packed = ds[0] | eu << 4 | ev << 6 | ew << 8 | (eT + 4) << 10 | (eb1 + 2) << 13 | (eb2 + 2) << 15 | \
            (eC + 2) << 17
        out.append((float(coeff), packed, str(t)))
    return out


def generate(ref_root: pathlib.Path) -> str:
    cases = parse_cases(ref_root / SRC_REL)
    if sorted(cases) != list(range(2, 40)):
        raise ValueError(f"expected cases 2..39, found {sorted(cases)}")
    f_terms, g_terms, f_off, g_off = [], [], [0, 0], [0, 0]
    for d in range(2, 40):
        calls, exprs = cases[d]
        check_rule(d, calls)
        fn, gn = expand_case(exprs)
        f_terms += terms(fn)
        g_terms += terms(gn)
        f_off.append(len(f_terms))
        g_off.append(len(g_terms))

    def arr(name, ts):
        body = ",\n".join(f"    {{{c!r}, {p}}}" for c, p, _ in ts)
        return f"IBB39_QUAL ibb39_term {name}[{len(ts)}] = {{\n{body}\n}};\n"

    return (
        "/* Generated by make_ibb39_table.py from the unshifted D3Q39 cases of\n"
        " * interpolative_bounceback_bc.f95:834-2838: per direction d (0-based, 1..38)\n"
        " * the terms [off[d], off[d + 1]) of fi_neq / k_fi and gi_neq / k_gi.  Packed\n"
        " * exponents: derivative (bits 0-3: du/dx, du/dy, du/dz, dv/dx .. dT/dz), u, v, w\n"
        " * (2 bits each from bit 4), T + 4 (3 bits from bit 10), beta_1 + 2, beta_2 + 2\n"
        " * (2 bits each from bit 13), C_v + 2 (3 bits from bit 17).  Do not edit. */\n"
        "#ifndef IBB39_TABLE_H\n#define IBB39_TABLE_H\n#include <stdint.h>\n"
        "#ifndef IBB39_QUAL\n#define IBB39_QUAL static const\n#endif\n"
        "typedef struct { double c; int32_t e; } ibb39_term;\n"
        f"IBB39_QUAL int ibb39_f_off[40] = {{{', '.join(map(str, f_off))}}};\n"
        f"IBB39_QUAL int ibb39_g_off[40] = {{{', '.join(map(str, g_off))}}};\n"
        + arr("ibb39_f_terms", f_terms) + arr("ibb39_g_terms", g_terms) + "#endif\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_ibb39_table.py <reference root>")
    root = pathlib.Path(sys.argv[1])
    (HERE / "ibb39_table.h").write_text(generate(root))
    print("wrote", HERE / "ibb39_table.h")
