"""Writes minimax_errors.json: published maximum errors of the best k-term
exponential sums for 1/x on [1, R] (Hackbusch's tables, as shipped with
megalochem in src/math/laplace/data/init_error.txt, tokens 1_xkKK_RRRR).
Kept: k <= 10, R <= 1e5, errors >= 3e-9 (the range a double-precision
Remez iteration resolves).  Run once where the reference tree is present,
with the root of that tree as the only argument:
    python tests/golden/make_minimax_fixture.py <megalochem source root>
"""
import json
import os
import sys


def parse_token(tok):
    k = int(tok[4:6])
    rs = tok[7:]
    if rs[1] == "E":
        R = int(rs[0]) * 10 ** int(rs[2:])
    else:
        R = int(rs[0]) + int(rs[1:]) / 1000.0
    return k, R


def main(root):
    path = os.path.join(root, "src/math/laplace/data/init_error.txt")
    out = []
    for line in open(path):
        if not line.startswith("1_xk"):
            continue
        tok, val = line.split()
        k, R = parse_token(tok)
        err = float(val)
        if k <= 10 and R <= 1e5 and err >= 3e-9:
            out.append({"k": k, "R": R, "err": err})
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "minimax_errors.json")
    with open(dst, "w") as f:
        json.dump({"source": "src/math/laplace/data/init_error.txt", "entries": out}, f, indent=0)
    print(len(out), "entries ->", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_minimax_fixture.py <megalochem source root>")
    main(sys.argv[1])
