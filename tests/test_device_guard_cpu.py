"""The C ABI's current-device guard, compiled with g++ against a fake device
API and run on the CPU (tests/cpp/test_device_guard.cpp): every entry point
that takes a context makes the context's device current and restores the
caller's device on return."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_device_guard_restores_callers_device(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "guard"
    subprocess.check_call([cxx, "-std=c++17", "-O1", "-o", str(exe),
                           os.path.join(HERE, "cpp", "test_device_guard.cpp")])
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert "device guard ok" in out.stdout
