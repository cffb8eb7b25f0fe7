"""Writes ibb_deriv_table.json: for each D3Q39 direction (1-based) and axis
(card 1 x, 2 y, 3 z), the derivative form the reference's
first_order_shifted_vel_cond_unknown and first_order_shifted_temp_cond_unknown
(derivatives/modules/derivatives.f95) select: the wall form dudx_ibb with its
up-wind flag, or the local difference dudx_local.

Run: python make_ibb_deriv_table.py <reference root>   (writes ibb_deriv_table.json here)"""
import json
import pathlib
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_ibb_deriv_table.py <reference root>")
SRC = pathlib.Path(sys.argv[1]) / "derivatives" / "modules" / "derivatives.f95"


def table(lines, fname):
    start = next(k for k, l in enumerate(lines) if ("function " + fname) in l)
    end = next(k for k in range(start + 1, len(lines)) if lines[k].strip().startswith("end function"))
    out, case, card, winds = [], None, None, None
    for raw in lines[start:end]:
        l = raw.split("!")[0]
        m = re.match(r"\s*case\((\d+)\)", l)
        if m:
            case = int(m.group(1))
            continue
        m = re.search(r"card == (\d)", l)
        if m:
            card, winds = int(m.group(1)), None
            continue
        m = re.search(r"winds = \.(true|false)\.", l)
        if m:
            winds = m.group(1) == "true"
            continue
        if "dudx_ibb" in l:
            out.append({"dir": case, "card": card, "form": "wall", "up": winds})
        elif "dudx_local" in l:
            out.append({"dir": case, "card": card, "form": "local"})
    return sorted(out, key=lambda e: (e["dir"], e["card"]))


lines = SRC.read_text().split("\n")
data = {"velocity": table(lines, "first_order_shifted_vel_cond_unknown"),
        "temperature": table(lines, "first_order_shifted_temp_cond_unknown")}
pathlib.Path(__file__).with_name("ibb_deriv_table.json").write_text(json.dumps(data, indent=0))
print(len(data["velocity"]), len(data["temperature"]))
