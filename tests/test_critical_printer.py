"""CPU test of the critical printer (include/ivarp/critical_printer.hpp): for a critical cuboid it prints the
variables and the interval value of every printable_expression, as the reference's CriticalPrinter does
(critical_printer.hpp:44-57, float_interval_print.hpp:30-40: max_digits10 digits, '~' when possibly
undefined). The values come from the host evaluator include/ivarp/sid_fe/host_eval.hpp; here they are
checked for enclosure against 300-bit mpmath on the printed box."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)

PROGRAM = r"""
#include <ivarp/critical_printer.hpp>
#include <iostream>
using namespace ivarp;
int main() {
    const auto x = args::x0;
    const auto y = args::x1;
    auto sys = constraint_system(variable(x, "x", 0, 1), variable(y, "y", 0, 2), x + y <= 3_Z);
    auto p = critical_printer(std::cout, sys, printable_expression("f", x * y + sqrt(y) - 0.1_X / (y + 1_Z)),
                              printable_expression("g", acos(x) * square(y)),
                              printable_expression("h", 1_Z / (x - 0.3_X)),
                              printable_expression("m", maximum(x, y - 1_Z, sqrt(2_Z))));
    IDouble box[2] = {IDouble(0.25, 0.5), IDouble(1.0, 4.0)};
    p(0, box);
}
"""


def test_critical_printer_prints_enclosing_expression_values(tmp_path):
    mpmath = pytest.importorskip("mpmath")
    src = tmp_path / "cp.cpp"
    src.write_text(PROGRAM)
    exe = str(tmp_path / "cp")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(REPO, "include"), str(src), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines()
    assert out[0] == "Critical:"
    assert out[1] == "\tx: [0.25, 0.5]" and out[2] == "\ty: [1, 4]"
    vals = {}
    for line in out[3:]:
        name, iv = line.strip().split(": ")
        und = iv.startswith("~")
        lo, hi = iv.lstrip("~")[1:-1].split(", ")
        vals[name] = (float(lo), float(hi), und)
    mpmath.mp.prec = 300
    iv = mpmath.iv
    X, Y = iv.mpf([0.25, 0.5]), iv.mpf([1.0, 4.0])
    exact = {"f": X * Y + iv.sqrt(Y) - iv.mpf("0.1") / (Y + 1),
             "g": iv.mpf([mpmath.acos(0.5), mpmath.acos(0.25)]) * Y ** 2,
             "m": iv.mpf([max(0.25, 0.0, float(mpmath.sqrt(2))), max(0.5, 3.0, float(mpmath.sqrt(2)))])}
    for name in ("f", "g"):
        lo, hi, und = vals[name]
        assert not und
        assert lo <= exact[name].a and exact[name].b <= hi, name
        assert exact[name].a - lo <= 1e-9 and hi - exact[name].b <= 1e-9, name   # tight as well
    assert vals["h"][2] and vals["h"][0] == float("-inf") and vals["h"][1] == float("inf")
    lo, hi, und = vals["m"]
    assert lo <= mpmath.sqrt(2) <= hi and hi == 3.0 and not und
