"""Golden values of the unshifted D3Q39 wall closure, evaluated straight from the
reference's formulas (interpolative_bounceback_bc.f95:834-2838, one case per
direction): each case's statements are run in order in float64 on seeded
random derivatives and targets, with k_fi = k_gi = eps = 1 and f_eq = g_eq = 0,
so that loc_fout = fi_neq / k_fi and loc_gout = gi_neq / k_gi.

Run: python make_ibb39_unshifted_golden.py [reference root]  (writes ibb39_unshifted_golden.json)
"""
import importlib.util
import json
import math
import pathlib
import random
import re
import sys

HERE = pathlib.Path(__file__).resolve().parent
GEN = HERE.parents[1] / "university-of-cincinnati-lattice-boltzmann-solver_gb300" / "csrc" / "make_ibb39_table.py"


def _fortran_to_python(rhs: str) -> str:
    return re.sub(r"(\d+\.\d*)[dD]([+-]?\d+)", r"\1e\2", rhs)


def main(root: pathlib.Path) -> None:
    spec = importlib.util.spec_from_file_location("make_ibb39_table", GEN)
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    cases = gen.parse_cases(root / gen.SRC_REL)
    rng = random.Random(20240611)
    out = {}
    for d in sorted(cases):
        rows = []
        for _ in range(3):
            D = [rng.uniform(-0.05, 0.05) for _ in range(12)]
            env = dict(zip(gen.DERIVS, D))
            u, v, w = rng.uniform(-0.3, 0.3), rng.uniform(-0.2, 0.2), rng.uniform(-0.2, 0.2)
            T, b1, b2, cv = rng.uniform(0.25, 0.45), rng.uniform(0.7, 0.99), rng.uniform(0.7, 0.99), 2.5
            env.update(temp_tgt=T, u_tgt=u, v_tgt=v, w_tgt=w, beta_1=b1, beta_2=b2, const_vol=cv, cv_const=1 / cv,
                       cv_const_2=2 / cv, k_fi=1.0, k_gi=1.0, loc_fieq=0.0, loc_gieq=0.0, loc_epsilon=1.0,
                       dimensions=3)
            for lhs, rhs in cases[d][1]:
                env[lhs] = eval(_fortran_to_python(rhs), {"abs": abs, "sqrt": math.sqrt}, env)
            rows.append({"D": D, "u": u, "v": v, "w": w, "T": T, "b1": b1, "b2": b2, "cv": cv,
                         "fpoly": env["loc_fout"], "gpoly": env["loc_gout"]})
        out[str(d - 1)] = rows  # 0-based direction
    (HERE / "ibb39_unshifted_golden.json").write_text(json.dumps(out, indent=0))


if __name__ == "__main__":
    main(pathlib.Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference"))
