"""The wx.* operator surface without a GPU (cpp/main.cpp:62-145, cpp/expr.hpp): the registry's schema is byte for
byte lmweather's schema/lmweather.dsl.json, the expression compiler gives the reference's results bit for bit and its
error texts exactly (golden fixture made by the reference's own compiler, tests/golden/make_expr_golden.py), the Wx
context methods and the argument checks that run before any engine call behave and fail as the reference's do
(test.sh:176-213), and the registrations compile against the reference's scripting VM interface."""
import hashlib
import json
import math
import os
import shutil
import subprocess

import pytest

from lmweather_gb300.wx import Wx, WxError, eval_expression
from oracle_lib import reference_dir

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF = reference_dir() or ""
# sha256 of lmweather 0.1.4's schema/lmweather.dsl.json (12,049 bytes: 8 Wx, 44 Sphere and 29 Plane methods)
SCHEMA_SHA256 = "62a74d57af48db2325d29b44ccf5e7d9546820c3f56e5a5d321d1fbaa99ac21b"


@pytest.fixture(scope="module")
def wx():
    with Wx() as w:
        yield w


def test_schema_is_the_reference_schema(wx):
    s = wx.schema()
    assert len(s) == 12049
    assert hashlib.sha256(s).hexdigest() == SCHEMA_SHA256
    d = json.loads(s)
    assert {t: len(v["methods"]) for t, v in d["types"].items()} == {"Wx": 8, "Sphere": 44, "Plane": 29}
    path = os.path.join(REF, "schema", "lmweather.dsl.json")
    if os.path.exists(path):
        with open(path, "rb") as f:
            assert f.read() == s


def _same_bits(got: float, want: str) -> bool:
    if want.lstrip("-") == "nan":
        return math.isnan(got)
    w = float(want) if want.lstrip("-") == "inf" else float.fromhex(want)
    return got == w and math.copysign(1.0, got) == math.copysign(1.0, w)


def test_expressions_against_the_reference_compiler():
    with open(os.path.join(HERE, "golden", "expr_cases.json")) as f:
        cases = json.load(f)
    assert len(cases) >= 90
    for c in cases:
        if "value" in c:
            got = eval_expression(c["text"], **c["vars"])
            assert _same_bits(got, c["value"]), (c["text"], got, c["value"])
        else:
            with pytest.raises(WxError) as e:
                eval_expression(c["text"], **c["vars"])
            assert str(e.value) == c["error"], c["text"]


def test_context_methods(wx, tmp_path, capfd):
    assert wx.version() == "lmweather 0.1.4"
    assert wx.assert_close(1.0, 1.05, 0.1) is None
    wx.assert_true(True)
    wx.print("hello from a script")
    assert "hello from a script\n" in capfd.readouterr().out
    p = tmp_path / "t.txt"
    wx.save_text(str(p), "a b\n")
    assert p.read_text() == "a b\n"
    with pytest.raises(WxError, match=r"^assert_close failed: 1 vs 2 \(tolerance 0.10000000000000001\)$"):
        wx.assert_close(1.0, 2.0, 0.1)
    with pytest.raises(WxError, match="assert_close failed"):
        wx.assert_close(1.0, 1.0, -1.0)
    with pytest.raises(WxError, match="assert_close failed"):
        wx.assert_close(float("nan"), 1.0, 10.0)


# test.sh:176-213, the cases that fail before an engine object exists
@pytest.mark.parametrize(
    "call, fragment",
    [
        (lambda w: w.sphere(2), "truncation"),
        (lambda w: w.sphere(171), "Wx.sphere: truncation must be between 4 and 170"),
        (lambda w: w.planet(10, 0.0, 0.0001, 9.8), "radius"),
        (lambda w: w.planet(10, 6.4e6, -1.0, 9.8), "omega not negative"),
        (lambda w: w.plane(2, 2, 1.0, 1.0), "4..4000"),
        (lambda w: w.plane(4000, 2001, 1.0, 1.0), "at most 8 million cells"),
        (lambda w: w.plane(10, 10, 0.0, 1.0), "domain"),
        (lambda w: w.save_text("/nonexistent-dir/x.csv", "x"), "cannot write"),
        (lambda w: w.assert_close(1.0, 2.0, 0.1), "assert_close failed"),
        (lambda w: w.assert_true(False), "assert_true failed"),
        (lambda w: w.sphere(10.0), "Wx.sphere argument 1 must be int"),
        (lambda w: w.plane(10, 10, 1, 1.0), "Wx.plane argument 3 must be float"),
        (lambda w: w.assert_true(1), "Wx.assert_true argument 1 must be bool"),
        (lambda w: w.print(3.0), "Wx.print argument 1 must be string"),
    ],
)
def test_errors_before_any_engine_call(wx, call, fragment):
    with pytest.raises(WxError, match=fragment):
        call(wx)


def test_call_errors(wx):
    with pytest.raises(ValueError, match="unknown method Wx.nothing"):
        wx.nothing()
    with pytest.raises(ValueError, match="Wx.version takes 0 argument"):
        wx.version(1)
    with pytest.raises(ValueError, match="unknown method Sphere.fly"):
        wx._call("Sphere", None, "fly", ())
    with pytest.raises(ValueError, match="the receiver is not a Sphere of this host"):
        wx._call("Sphere", 12345, "time", ())


def test_registrations_compile_against_the_reference_vm(tmp_path):
    """register_host<VM> instantiated with the reference's own scripting VM types (cpp/dslvm.hpp): the host program
    keeps its registry and calls this layer's register_host in place of its own."""
    vm = os.path.join(REF, "cpp", "dslvm.hpp")
    if not os.path.exists(vm) or shutil.which("g++") is None:
        pytest.skip("the reference checkout (its VM header) is absent")
    src = tmp_path / "bind.cpp"
    src.write_text(
        '#include "dslvm.hpp"\n#include "lmweather_wx.hpp"\n'
        "struct DslvmVM { using Registry = dslvm::Registry; using Value = dslvm::Value; using Args = dslvm::Args; "
        "using Error = dslvm::Error; };\n"
        "void bind(dslvm::Registry &r, lmweather_gb300::wx::Host &h) { lmweather_gb300::wx::register_host<DslvmVM>(r, h); }\n"
    )
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I" + os.path.join(REF, "cpp"), "-I" + os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
