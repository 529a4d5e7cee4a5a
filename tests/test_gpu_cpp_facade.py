"""The reference's program tests (isprings, cg, femTet) written in C++ against
the facade simit_gb300/cpp/simit.h (Set / FieldRef / Function::bind / init /
runSafe), compiled here and run on the GPU."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_program_tests(tmp_path):
    from simit_gb300 import _lib
    _lib.load()
    exe = str(tmp_path / "test_programs")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-std=c++17", "-O2", "-I", ROOT, "-I", os.path.join(cuda, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_programs.cpp"),
           "-L", os.path.join(ROOT, "simit_gb300"), "-lsimit_gb300",
           "-L", os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + os.path.join(ROOT, "simit_gb300"), "-o", exe]
    subprocess.check_call(cmd)
    r = subprocess.run([exe, os.path.join(ROOT, "tests", "golden")], capture_output=True,
                       text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all passed" in r.stdout
