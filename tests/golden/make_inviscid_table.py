"""Writes inviscid_table.json: the reference's specular-reflection table for
D3Q39 inviscid links (boundary_conditions/inviscid_edge.f95), run through the
f95_subset interpreter: for each direction i (1-based) and every combination
of the state components its SELECT CASE branch consults being -11 (the rest
0), the direction the population goes to (inviscid_dir; null where no branch
assigns it) and the displacement (loc_cx, loc_cy, loc_cz) of the receiving
node; once for the unshifted lattice and once for the shifted one with the
primary flow along +x (the routine then adds the shift to the displacement).

Run: python make_inviscid_table.py <reference root>   (writes inviscid_table.json here)"""
import itertools
import json
import pathlib
import re
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import f95_subset as F  # noqa: E402


def consulted(src: str):
    """Per direction, the loc_state components its CASE branch reads."""
    out, case = {}, None
    for raw in src.split("\n"):
        line = raw.split("!")[0].strip()
        m = re.match(r"CASE\s*\((\d+)\)", line, re.I)
        if m:
            case = int(m.group(1))
            out[case] = set()
            continue
        if re.match(r"END\s*SELECT", line, re.I):
            break
        if case is not None:
            out[case] |= {int(x) for x in re.findall(r"loc_state\((\d+)\)", line, re.I)}
    return out


def main(root: pathlib.Path) -> None:
    src = (root / "boundary_conditions" / "inviscid_edge.f95").read_text()
    procs = F.parse_units(F.logical_lines(src), only={"inviscid_edge"})
    table = {}
    for name, shifted in (("unshifted", False), ("shifted", True)):
        interp = F.Interp(procs, {"dir": F.FInt(39), "dp": F.FInt(8), "shifted": shifted,
                                  "primary_flow_dir": F.FInt(1)})
        table[name] = cases(interp, src)
    (HERE / "inviscid_table.json").write_text(json.dumps(table, indent=0))
    print({k: sum(len(v) for v in t.values()) for k, t in table.items()})


def cases(interp, src):
    table = {}
    for i, comps in sorted(consulted(src).items()):
        comps = sorted(comps)
        entries = []
        for r in range(len(comps) + 1):
            for walls in itertools.combinations(comps, r):
                state = np.zeros(39, np.int64)
                state[i - 1] = -11
                for c in walls:
                    state[c - 1] = -11
                v = {"f": 0.0, "fo": 0.0, "g": 0.0, "go": 0.0, "j": F.FInt(-999), "x": F.FInt(7), "y": F.FInt(7),
                     "z": F.FInt(7)}
                interp.call("inviscid_edge", [F.Ref(v, "f"), F.Ref(v, "fo"), F.Ref(v, "g"), F.Ref(v, "go"), F.FInt(i),
                                              F.FInt(-11), F.FArray(state.copy()), F.Ref(v, "j"), F.Ref(v, "x"),
                                              F.Ref(v, "y"), F.Ref(v, "z")])
                j = int(v["j"])
                entries.append({"walls": list(walls), "dir": None if j == -999 else j,
                                "loc": [int(v["x"]), int(v["y"]), int(v["z"])]})
        table[str(i)] = entries
    return table


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_inviscid_table.py <reference root>")
    main(pathlib.Path(sys.argv[1]))
