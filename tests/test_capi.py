"""The drop-in boundary without a GPU: the library builds, loads and exports every entry point that
include/*.h declares; the Python mirror fails loudly when asked to run without a device; the host-side
argument checks answer with the reference's messages before any device work."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    inc = os.path.join(ROOT, "include")
    for fn in sorted(os.listdir(inc)):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(lmw_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(engine):
    lib = ctypes.CDLL(engine.library_path())
    names = declared_symbols()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_error_channel(engine):
    lib = engine.load_library()
    assert lib.lmw_version().decode().startswith("lmweather-gb300")
    assert lib.lmw_last_error() is not None


def test_header_is_plain_c():
    # the boundary carries no torch or C++ types: it compiles as C
    import subprocess
    import tempfile

    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        with open(src, "w") as f:
            f.write('#include "lmweather_gb300.h"\n#include "lmweather_wx.h"\nint main(void) { return lmw_version() == 0; }\n')
        r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-c", "-I", os.path.join(ROOT, "include"), src, "-o",
                            os.path.join(d, "t.o")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_null_handles_are_rejected(engine):
    lib = engine.load_library()
    assert lib.lmw_sphere_step(None, 10.0) == 1
    assert "null sphere handle" in lib.lmw_last_error().decode()
    assert lib.lmw_plane_run(None, 10.0, 1.0) == 1
    assert "null plane handle" in lib.lmw_last_error().decode()


def test_constructor_argument_checks_use_reference_messages(engine):
    # cpp/sphere.cpp:76 and cpp/plane.cpp:21-23: checked on the host before any device work
    with pytest.raises(ValueError, match="truncation must be between 4 and 170"):
        engine.Sphere(2)
    with pytest.raises(ValueError, match="truncation must be between 4 and 170"):
        engine.Sphere(171)
    with pytest.raises(ValueError, match="at least 4 x 4 and at most 8 million cells"):
        engine.Plane(2, 2, 1.0, 1.0)
    with pytest.raises(ValueError, match="domain sizes must be positive"):
        engine.Plane(8, 8, -1.0, 1.0)


def test_no_silent_cpu_path_without_a_device(engine):
    from conftest import gpu_available

    if gpu_available():
        pytest.skip("a GPU is present")
    with pytest.raises(engine.DeviceError):
        engine.Sphere(21)
    with pytest.raises(engine.DeviceError):
        engine.Plane(16, 8, 1e5, 5e4)
