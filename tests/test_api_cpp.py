"""The C++ template API compiled into a user program with nvcc (the way a
C++ caller of the reference's headers would switch over)."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def build_example(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "api_usage")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
           "--extended-lambda", "-I", os.path.join(REPO, "include"),
           "-I", os.path.join(REPO, "mgpu-shaders_gb300", "inc"),
           os.path.join(HERE, "cpp", "api_usage.cu"), "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_cpp_template_api(tmp_path):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    exe = build_example(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    for name in ["launch_transform", "mergesort_user_comparator", "merge_keys",
                 "scan_exclusive_in_place", "radix_sort_keys"]:
        assert "ok " + name in r.stdout
