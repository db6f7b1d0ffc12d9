"""Host unit test of the integer-pipe FP64 multiply used by the complex128
gate kernels (compiled with the host compiler; no GPU needed)."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_emul_matches_ieee_product():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "test_emul")
        subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "pennylane_lightning_gpu_gb300", "csrc",
                                                                         "kernels"),
                        os.path.join(ROOT, "tests", "native", "test_emul.cpp"), "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "bad 0" in r.stdout
