"""Golden values of the unshifted D3Q39 wall closure, evaluated straight from the
reference's formulas (interpolative_bounceback_bc.f95:834-2838, one case per
direction): the select-case block is parsed and run by the Fortran-subset
interpreter (tests/golden/f95_subset.py; independent of the table generator's
own reader) in float64 on seeded random derivatives and targets, with k_fi =
k_gi = eps = 1 and f_eq = g_eq = 0, so that loc_fout = fi_neq / k_fi and
loc_gout = gi_neq / k_gi.  The derivative calls of each case return the seeded
derivative values.

Run: python make_ibb39_unshifted_golden.py <reference root>   (writes ibb39_unshifted_golden.json)
"""
import json
import pathlib
import random
import re
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import f95_subset as F  # noqa: E402

SRC_REL = "boundary_conditions/interpolative_bc/interpolative_bounceback_bc.f95"
FIRST = 834  # 1-based line of the D3Q39 branch; its unshifted select-case block follows
DERIVS = ["dudx", "dudy", "dudz", "dvdx", "dvdy", "dvdz", "dwdx", "dwdy", "dwdz", "dtdx", "dtdy", "dtdz"]


def unshifted_cases(root: pathlib.Path):
    """The select-case node of the unshifted D3Q39 closures (direction -> statements)."""
    lines = F.logical_lines((root / SRC_REL).read_text())
    k = next(j for j, (no, s) in enumerate(lines) if no >= FIRST and re.match(r"^select\s+case\s*\(i\)$", s))
    node, _ = F.parse_stmt(lines, k)
    return node


def main(root: pathlib.Path) -> None:
    sel = unshifted_cases(root)
    rng = random.Random(20240611)
    out = {}
    cases = {int(sel_[0]): body for sel_, body in sel.cases if sel_ is not None}
    for d in sorted(cases):
        rows = []
        for _ in range(3):
            D = [rng.uniform(-0.05, 0.05) for _ in range(12)]
            u, v, w = rng.uniform(-0.3, 0.3), rng.uniform(-0.2, 0.2), rng.uniform(-0.2, 0.2)
            T, b1, b2, cv = rng.uniform(0.25, 0.45), rng.uniform(0.7, 0.99), rng.uniform(0.7, 0.99), 2.5
            g = dict(temp_tgt=T, u_tgt=u, v_tgt=v, w_tgt=w, beta_1=b1, beta_2=b2, const_vol=cv, cv_const=1 / cv,
                     cv_const_2=2 / cv, k_fi=1.0, k_gi=1.0, loc_fieq=0.0, loc_gieq=0.0, loc_epsilon=1.0,
                     dimensions=F.FInt(3), i=F.FInt(d), a=F.FInt(1), b=F.FInt(1), c=F.FInt(1), upwind=F.FInt(1),
                     downwind=F.FInt(-1), dir_state=F.FInt(0), temperature=T,
                     rest_state=F.FArray(np.zeros((1, 1, 1, 39), np.int64), [1, 1, 1, 1]))
            for name in ("loc_u", "loc_v", "loc_w", "loc_temp"):
                g[name] = F.FArray(np.zeros(39))
            # each derivative function returns its seeded value
            for name, val in zip(DERIVS, D):
                for form in ("ibb", "local"):
                    g[f"{name}_{form}"] = (lambda val: (lambda *args: val))(val)
            interp = F.Interp({}, g)
            local = {}
            interp.run(cases[d], local, interp.scope_for(local))
            rows.append({"D": D, "u": u, "v": v, "w": w, "T": T, "b1": b1, "b2": b2, "cv": cv,
                         "fpoly": float(g["loc_fout"]), "gpoly": float(g["loc_gout"])})
        out[str(d - 1)] = rows  # 0-based direction
    (HERE / "ibb39_unshifted_golden.json").write_text(json.dumps(out, indent=0))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_ibb39_unshifted_golden.py <reference root>")
    main(pathlib.Path(sys.argv[1]))
