"""Extracts the literal known answers of the reference's own tests for the
angular-momentum algebra on the hot path (Wigner 3j / 6j, Clebsch-Gordan; used by
the spin-mixing and general-F tensor steps) into known_answers.json.

Reads the Julia test files as text (nothing of the reference is executed); run it
where the reference is mounted:

    python tests/golden/make_golden.py /root/reference

Each record keeps the source file and line, the function, its integer arguments,
the comparison (== or approx) and the expected value evaluated from the Julia
expression (numbers, + - * /, sqrt, pi)."""

import ast
import json
import math
import re
import sys
from pathlib import Path

FILES = ["test/test_clebsch_gordan.jl"]
FUNCS = {"wigner_3j", "wigner_6j", "clebsch_gordan"}
LINE = re.compile(r"@test\s+(\w+)\(([-0-9,\s]+)\)\s*(≈|==)\s*(.+?)(?:\s+(atol|rtol)\s*=\s*([0-9.eE-]+))?\s*$")


def _eval(expr: str) -> float:
    tree = ast.parse(expr.replace("π", "pi"), mode="eval")

    def ev(n):
        if isinstance(n, ast.Expression):
            return ev(n.body)
        if isinstance(n, ast.Constant) and isinstance(n.value, (int, float)):
            return float(n.value)
        if isinstance(n, ast.Name) and n.id == "pi":
            return math.pi
        if isinstance(n, ast.UnaryOp) and isinstance(n.op, ast.USub):
            return -ev(n.operand)
        if isinstance(n, ast.BinOp) and isinstance(n.op, (ast.Add, ast.Sub, ast.Mult, ast.Div)):
            a, b = ev(n.left), ev(n.right)
            return {ast.Add: a + b, ast.Sub: a - b, ast.Mult: a * b, ast.Div: a / b}[type(n.op)]
        if isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and n.func.id == "sqrt" and len(n.args) == 1:
            return math.sqrt(ev(n.args[0]))
        raise ValueError(f"unsupported expression {expr!r}")

    return ev(tree)


def main(ref: str) -> None:
    out = []
    for rel in FILES:
        for no, line in enumerate((Path(ref) / rel).read_text().splitlines(), start=1):
            m = LINE.search(line.strip())
            if not m or m.group(1) not in FUNCS:
                continue
            rec = {"source": f"{rel}:{no}", "func": m.group(1),
                   "args": [int(a) for a in m.group(2).split(",")], "op": m.group(3),
                   "expected": _eval(m.group(4))}
            if m.group(5):
                rec[m.group(5)] = float(m.group(6))
            out.append(rec)
    dst = Path(__file__).with_name("known_answers.json")
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print(f"{len(out)} known answers -> {dst}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
