"""Writes inviscid_table.json: the reference's specular-reflection table for
D3Q39 inviscid links (boundary_conditions/inviscid_edge.f95): for each
direction (1-based) the ordered IF chain of its SELECT CASE branch, each entry
the state components that must equal -11, the reflected direction and the
displacement (loc_cx, loc_cy, loc_cz) of the node that receives it.

Run: python make_inviscid_table.py <reference root>   (writes inviscid_table.json here)"""
import json
import pathlib
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_inviscid_table.py <reference root>")
SRC = pathlib.Path(sys.argv[1]) / "boundary_conditions" / "inviscid_edge.f95"
cases, case, cond, cur = {}, None, [], None
for raw in SRC.read_text().split("\n"):
    line = raw.split("!")[0].strip()
    m = re.match(r"CASE\s*\((\d+)\)", line, re.I)
    if m:
        case, cond = int(m.group(1)), []
        cases[case] = []
        continue
    if case is None:
        continue
    if re.match(r"END SELECT", line, re.I):
        break
    if re.match(r"(ELSE\s*)?IF\s*\(", line, re.I):
        cond = sorted(int(x) for x in re.findall(r"loc_state\((\d+)\)\s*==\s*-11", line))
        continue
    m = re.match(r"inviscid_dir\s*=\s*(\d+)", line)
    if m:
        cur = {"cond": cond, "dir": int(m.group(1)), "loc": [0, 0, 0]}
        cases[case].append(cur)
        continue
    for a, ax in enumerate("xyz"):
        m = re.match(r"loc_c%s\s*=\s*(-?\d+)" % ax, line)
        if m and cur is not None:
            cur["loc"][a] = int(m.group(1))
pathlib.Path(__file__).with_name("inviscid_table.json").write_text(json.dumps(cases, indent=0))
print(len(cases), sum(len(v) for v in cases.values()))
