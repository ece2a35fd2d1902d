"""Generate tests/golden/expr_cases.json by running the reference's own expression compiler.

lmweather's builders compile expression strings with lmnum::Expr (cpp/expr.hpp, a header with no dependencies).
This script writes a small C++ driver, compiles it here against that header where it lies in the reference
checkout, evaluates every case below with it and records the result bits (C99 hex float) or the exact error text.
It runs only where the reference checkout exists (given as the argument, or $LMW_REFERENCE_DIR, or a checkout named
`reference` beside this repository); the fixture it writes is committed so the tests need neither.

    python tests/golden/make_expr_golden.py [<lmweather checkout>]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from oracle_lib import reference_dir  # noqa: E402
OUT = os.path.join(HERE, "expr_cases.json")

DRIVER = r"""
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>
#include "expr.hpp"
// one case per line: text \x1f name,name,... \x1f v1,v2,...; prints the result as %a or "ERR <message>"
int main() {
  std::string line;
  while (std::getline(std::cin, line)) {
    size_t a = line.find('\x1f'), b = line.find('\x1f', a + 1);
    std::string text = line.substr(0, a), names = line.substr(a + 1, b - a - 1), vals = line.substr(b + 1);
    std::vector<std::string> vars = lmnum::split_names(names);
    std::vector<double> x;
    for (const auto &s : lmnum::split_names(vals)) x.push_back(std::strtod(s.c_str(), nullptr));
    try {
      lmnum::Expr e(text, vars);
      std::printf("%a\n", e.eval(x.data()));
    } catch (const std::exception &ex) {
      std::printf("ERR %s\n", ex.what());
    }
  }
}
"""

X = {"x": 0.7, "y": -1.3}
CASES = [
    # precedence, signs, powers
    ("1 + 2 * 3", {}), ("(1 + 2) * 3", {}), ("2^3^2", {}), ("2**3**2", {}), ("-2^2", {}), ("2^-1", {}), ("--3", {}),
    ("+-3", {}), ("- - x", X), ("x ** -2", X), ("2 ^ - x", X), ("1 - 2 - 3", {}), ("8 / 4 / 2", {}), ("2 * -3", {}),
    ("x*y - y/x + x^y", X), ("-x^2 + (-x)^2", X), ("3.", {}), (".5", {}), ("1.5e3", {}), ("2E-3", {}), ("0x1p3", {}),
    ("  x  +  y  ", X), ("sin (x)", X), ("1/0", {}), ("-1/0", {}), ("0/0", {}),
    # names and constants
    ("pi", {}), ("e", {}), ("pi * x", X), ("e ^ y", X), ("x1 + _b2", {"x1": 2.0, "_b2": 0.25}),
    ("lat * lon", {"lon": 1.25, "lat": -0.5}),
    # functions
    ("sin(x)", X), ("cos(x)", X), ("tan(x)", X), ("asin(0.3)", {}), ("acos(0.3)", {}), ("atan(2)", {}), ("sinh(1.1)", {}),
    ("cosh(1.1)", {}), ("tanh(0.4)", {}), ("exp(-x*x)", X), ("log(e)", {}), ("ln(2)", {}), ("log10(1000)", {}),
    ("sqrt(2)", {}), ("sqrt(-1)", {}), ("abs(y)", X), ("floor(-2.5)", {}), ("ceil(2.1)", {}), ("sign(y)", X), ("sign(0)", {}),
    ("atan2(y, x)", X), ("pow(2, 0.5)", {}), ("min(x, y)", X), ("max(x, y)", X), ("mod(-7, 3)", {}), ("mod(7.5, 2)", {}),
    ("5960.0 - 1500.0 * pow(2.718281828459045, -((x - 3.0) * (x - 3.0) * cos(y) * cos(y) + y * y) / 0.1)", X),
    ("500.0 * (1 + cos(pi * min(1.0, 3.0 * acos(cos(y) * cos(x - 1.5 * pi)))))", X),
    ("2000.0 * (1 - sqrt(min((pi / 9) * (pi / 9), (x - 1.5 * pi) * (x - 1.5 * pi) + (y - pi / 6) * (y - pi / 6))) / (pi / 9))", X),
    # errors
    ("2 +* 3", {}), ("foo", {}), ("foo(1)", {}), ("sin(1, 2)", {}), ("atan2(1)", {}), ("pow()", {}), ("(1", {}), ("1)", {}),
    ("", {}), ("   ", {}), ("1e400", {}), ("-1e400", {}), ("1e-400", {}), (".", {}), ("..5", {}), ("2 3", {}), ("x +", X),
    ("sin(", {}), ("sin(1", {}), ("min(1,)", {}), ("1 # 2", {}), ("x $", X), ("1 ** * 2", {}),
    ("(" * 99 + "1" + ")" * 99, {}), ("(" * 100 + "1" + ")" * 100, {}), ("(" * 300 + "1" + ")" * 300, {}),
    ("-" * 199 + "1", {}), ("-" * 200 + "1", {}), ("1" + "+1" * 1999, {}), ("1" + "+1" * 2000, {}),
    ("x + " * 40 + "unknown_name_here", X), ("sin(1 + foo)", {}), ("foo(1 +* 2)", {}),
]


def main() -> None:
    ref = sys.argv[1] if len(sys.argv) > 1 else reference_dir()
    if not ref or not os.path.isfile(os.path.join(ref, "cpp", "expr.hpp")):
        sys.exit("the reference checkout is absent: the committed fixture stands")
    REF_CPP = os.path.join(ref, "cpp")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "expr_driver.cpp")
        exe = os.path.join(d, "expr_driver")
        with open(src, "w") as f:
            f.write(DRIVER)
        subprocess.run(["g++", "-std=c++17", "-O2", "-I" + REF_CPP, src, "-o", exe], check=True)
        lines = []
        for text, env in CASES:
            names = ",".join(env)
            vals = ",".join(repr(float(v)) for v in env.values())
            lines.append(f"{text}\x1f{names}\x1f{vals}")
        r = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    outs = r.stdout.splitlines()
    assert len(outs) == len(CASES)
    fixture = []
    for (text, env), out in zip(CASES, outs):
        item = {"text": text, "vars": {k: float(v) for k, v in env.items()}}
        if out.startswith("ERR "):
            item["error"] = out[4:]
        else:
            item["value"] = out
        fixture.append(item)
    with open(OUT, "w") as f:
        json.dump(fixture, f, indent=1)
        f.write("\n")
    print(f"{len(fixture)} cases -> {OUT}")


if __name__ == "__main__":
    main()
