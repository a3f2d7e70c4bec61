"""The C++ shim (include/agb.hpp) compiles against the C ABI with g++ alone,
and on a GPU reproduces the tests/Solid KAT through the reference call shape."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "shim_example.cpp")


def compile_example(tmp_path):
    from alamo_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "shim_example")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", os.path.dirname(lib), "-lalamo_gb300", "-Wl,-rpath," + os.path.dirname(lib)]
    subprocess.check_call(cmd)
    return exe


def test_shim_compiles(tmp_path):
    assert os.path.exists(compile_example(tmp_path))


@pytest.mark.gpu
def test_shim_runs_kat(tmp_path):
    exe = compile_example(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
