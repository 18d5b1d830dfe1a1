"""The header-only C++ wrapper compiles and links against liballium_sweep.so
(CPU), and runs the constant-solution check on the GPU."""
import os
import subprocess

import pytest

from allium_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "tests", "cpp", "_build", "wrapper_demo")


def compile_demo():
    build.build()
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    libdir = os.path.dirname(build.LIB)
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "wrapper_demo.cpp"),
           "-L", libdir, "-lallium_sweep", f"-Wl,-rpath,{libdir}", "-o", EXE]
    subprocess.run(cmd, check=True)
    return EXE


def test_wrapper_compiles_and_links():
    assert os.path.exists(compile_demo())


@pytest.mark.gpu
def test_wrapper_constant_solution_on_gpu():
    r = subprocess.run([compile_demo()], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")
