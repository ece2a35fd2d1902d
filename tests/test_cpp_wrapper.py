"""The C++ classes over the C ABI (include/lmweather_gb300.hpp): the header compiles as C++17 on its own (CPU), and
a program using it the way lmweather's wx.* layer uses lmweather::Sphere / Plane runs on the GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_header_compiles():
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "wrapper_test.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_wrapper_program_on_gpu(engine, tmp_path):
    lib_dir = os.path.dirname(engine.library_path())
    exe = str(tmp_path / "wrapper_test")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "wrapper_test.cpp"),
                        "-L", lib_dir, "-llmw_gb300", f"-Wl,-rpath,{lib_dir}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0 and run.stdout.strip().endswith("ok"), run.stdout + run.stderr
