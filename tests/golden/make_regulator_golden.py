"""Generate tests/golden/rational_exp_regulator.json from DiFfRG's RationalExpRegulator.

Source: DiFfRG/include/DiFfRG/physics/regulators.hh, struct RationalExpRegulator: get_f(x) and
get_df(x) are written there as one rational expression per order 1..16 in x, c and b0.  This
script reads those expressions as text, evaluates them in Python (double precision) at the
sample points below, and stores f and f' per order, option set and x.  The drop-in's regulator
builds f from its defining construction instead of the per-order expressions; the test
(tests/test_boundary_headers.py) compares the two.

Run with the path of a DiFfRG checkout (the project root):
    python tests/golden/make_regulator_golden.py /path/to/DiFfRG-project-root
"""
import json
import os
import re
import sys

OPTIONS = [(2.0, 0.0), (1.5, 0.25), (3.0, 0.1)]  # (c, b0)
XS = [1e-3, 0.05, 0.3, 0.9, 1.7, 4.0, 10.0]


def powr(n, y):
    return y ** n


def expressions(block, fname):
    start = block.index(fname + "(const auto x)")
    body = block[start:]
    body = body[:body.index("static_assert")]
    out = {}
    for order, expr in re.findall(r"if constexpr \(order == (\d+)\)\s*return\s*(.*?);", body, flags=re.S):
        out[int(order)] = re.sub(r"powr<(-?\d+)>\(", r"powr(\1, ", " ".join(expr.split()))
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_regulator_golden.py /path/to/DiFfRG-project-root")
    path = os.path.join(sys.argv[1], "DiFfRG/include/DiFfRG/physics/regulators.hh")
    text = open(path).read()
    block = text[text.index("struct RationalExpRegulator {"):]
    block = block[:block.index("struct PolynomialExpRegulatorOpts")]
    f_expr, df_expr = expressions(block, "get_f"), expressions(block, "get_df")
    assert sorted(f_expr) == list(range(1, 17)) and sorted(df_expr) == list(range(1, 17))
    cases = []
    for order in range(1, 17):
        for c, b0 in OPTIONS:
            for x in XS:
                env = {"powr": powr, "x": x, "c": c, "b0": b0}
                cases.append({"order": order, "c": c, "b0": b0, "x": x,
                              "f": float(eval(f_expr[order], env)), "df": float(eval(df_expr[order], env))})
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rational_exp_regulator.json")
    with open(out, "w") as fh:
        json.dump({"source": "DiFfRG/include/DiFfRG/physics/regulators.hh RationalExpRegulator::get_f/get_df",
                   "cases": cases}, fh, indent=0)
    print("wrote", out, len(cases), "cases")


if __name__ == "__main__":
    main()
