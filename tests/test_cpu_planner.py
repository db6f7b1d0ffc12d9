"""Host unit tests of the gate lowering and the shared-memory fusion planner
(GateLowering.hpp), of the register-group split of a fused block
(lgpu_fused_plan.h), of the folding of diagonal gates into phase tables
(lgpu_fused_plan.h) and of the Pauli-word tile pass plan
(lgpu_pauli_plan.h): invariants, and state equivalence of the reordered
gates, on random inputs (compiled with the host compiler; no GPU needed)."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "include", "cuComplex.h")):
            return os.path.join(cand, "include")
    nvcc = shutil.which("nvcc")
    if nvcc:
        inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
        if os.path.exists(os.path.join(inc, "cuComplex.h")):
            return inc
    return None


def test_fusion_plan_keeps_the_state():
    inc = _cuda_include()
    if inc is None:
        pytest.skip("cuComplex.h not found")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "test_planner")
        subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "tests", "native"),
                        "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(ROOT, "pennylane_lightning_gpu_gb300", "csrc", "cpp"), "-I" + inc,
                        os.path.join(ROOT, "tests", "native", "test_planner.cpp"), "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "bad 0" in r.stdout


def test_register_groups_keep_the_state():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "test_fused_groups")
        subprocess.run(["g++", "-O2", "-std=c++17",
                        "-I" + os.path.join(ROOT, "pennylane_lightning_gpu_gb300", "csrc", "kernels"),
                        "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "native", "test_fused_groups.cpp"), "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "bad 0" in r.stdout


def test_pauli_tile_pass_plan():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "test_pauli_plan")
        subprocess.run(["g++", "-O2", "-std=c++17",
                        "-I" + os.path.join(ROOT, "pennylane_lightning_gpu_gb300", "csrc", "kernels"),
                        os.path.join(ROOT, "tests", "native", "test_pauli_plan.cpp"), "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "bad 0" in r.stdout


def test_lowering_matches_the_oracle():
    inc = _cuda_include()
    if inc is None:
        pytest.skip("cuComplex.h not found")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "test_lowering_vs_oracle")
        subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "tests", "native"),
                        "-I" + os.path.join(ROOT, "oracle"), "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(ROOT, "pennylane_lightning_gpu_gb300", "csrc", "cpp"), "-I" + inc,
                        os.path.join(ROOT, "tests", "native", "test_lowering_vs_oracle.cpp"), "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "bad 0" in r.stdout


def test_diagonal_folding_keeps_the_state():
    """Diagonal gates of float-float fused blocks folded into phase tables
    (lgpu_fused_plan.h::fold_diagonal_gates): 400 random blocks transform
    random states exactly as the unfolded gate lists do."""
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "test_diag_fold")
        subprocess.run(["g++", "-O2", "-std=c++17",
                        "-I" + os.path.join(ROOT, "pennylane_lightning_gpu_gb300", "csrc", "kernels"),
                        "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "native", "test_diag_fold.cpp"), "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "bad 0" in r.stdout



def test_adjoint_phase_group_plan():
    """Phase groups of the adjoint blocks
    (lgpu_adj_plan.h::plan_phase_groups): on 500 random runs of steps the
    planned sweep (a group's overlaps before its U^dag) gives every step's
    overlap and the final states of the original order."""
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "test_adj_plan")
        subprocess.run(["g++", "-O2", "-std=c++17",
                        "-I" + os.path.join(ROOT, "pennylane_lightning_gpu_gb300", "csrc", "kernels"),
                        os.path.join(ROOT, "tests", "native", "test_adj_plan.cpp"), "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "bad 0" in r.stdout
