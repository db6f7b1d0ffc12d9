"""Host unit test of the float-float arithmetic used by the complex128 fused
gate bodies (compiled with the host compiler; no GPU needed)."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_df64_split_rebuild_and_bodies():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "test_df64")
        subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "pennylane_lightning_gpu_gb300", "csrc",
                                                                         "kernels"),
                        os.path.join(ROOT, "tests", "native", "test_df64.cpp"), "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "bad 0" in r.stdout
