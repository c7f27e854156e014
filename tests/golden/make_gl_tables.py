"""Generate tests/golden/gl_tables.json from DiFfRG's constexpr Gauss-Legendre tables.

Source: DiFfRG/include/DiFfRG/common/quadrature/gauss_legendre.hh (GLQuadrature<N, ctype>,
nodes x[i] and weights w[i] on [0,1]).  The reference's own quadrature test compares
make_quadrature against exactly these tables for N = 4, 8, 16, 32, 64, 128
(DiFfRG/tests/common/quadrature/test_quadrature.cc:10-33); the same orders are extracted here.

Run with the path of a DiFfRG checkout (the project root):
    python tests/golden/make_gl_tables.py /path/to/DiFfRG-project-root
The JSON keeps the decimal strings of the header (30+ digits), parsed to float at test time.
"""
import json
import os
import re
import sys

ORDERS = [4, 8, 16, 32, 64, 128]


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_gl_tables.py /path/to/DiFfRG-project-root")
    root = sys.argv[1]
    path = os.path.join(root, "DiFfRG/include/DiFfRG/common/quadrature/gauss_legendre.hh")
    text = open(path).read()
    blocks = re.split(r"template <typename ctype> struct GLQuadrature<(\d+), ctype>", text)
    tables = {}
    for i in range(1, len(blocks), 2):
        n = int(blocks[i])
        if n not in ORDERS:
            continue
        body = blocks[i + 1]
        xs = dict((int(a), b) for a, b in re.findall(r"\bx\[(\d+)\]\s*=\s*([0-9eE.+-]+);", body))
        ws = dict((int(a), b) for a, b in re.findall(r"\bw\[(\d+)\]\s*=\s*([0-9eE.+-]+);", body))
        assert len(xs) == n and len(ws) == n, n
        tables[str(n)] = {"x": [xs[j] for j in range(n)], "w": [ws[j] for j in range(n)]}
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gl_tables.json")
    with open(out, "w") as f:
        json.dump({"source": "DiFfRG/include/DiFfRG/common/quadrature/gauss_legendre.hh",
                   "interval": [0, 1], "tables": tables}, f, indent=0)
    print("wrote", out, sorted(int(k) for k in tables))


if __name__ == "__main__":
    main()
