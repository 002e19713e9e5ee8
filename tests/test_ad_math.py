"""The per-particle arithmetic of the differentiated step (csrc/ad_math.cuh),
compiled for the host: tangent-linear derivatives against central
differences, and the hand-written adjoints against the tangent-linear ones
(dot-product test). The same header is compiled into the GPU kernels."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "apc_524_project_gb300", "csrc")


def test_ad_math_tangent_and_adjoint(tmp_path):
    exe = str(tmp_path / "ad_math_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "ad_math_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASSED" in r.stdout
