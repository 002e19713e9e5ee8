"""The reference class mirror (include/emoopic.hpp), host-only parts: the
boundary factories' string registries (declare / lookup / types, the
Register*Boundary statics, the reference's error texts) resolve input.txt
names, user-registered ones included, to the device's boundary kinds.
Compiles tests/cpp_mirror_check.cpp with g++ and runs it; no GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_boundary_registries(tmp_path):
    exe = tmp_path / "cpp_mirror_check"
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp_mirror_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"
