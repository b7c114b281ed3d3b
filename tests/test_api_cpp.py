"""The C++ template API compiled into a user program with nvcc (the way a
C++ caller of the reference's headers would switch over)."""
import os
import shutil
import subprocess

import pytest

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


@pytest.mark.gpu
def test_cpp_template_api(tmp_path):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    exe = build_example(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    for name in ["launch_transform", "mergesort_user_comparator", "merge_keys",
                 "scan_exclusive_in_place", "radix_sort_keys", "radix_sort_keys_4bit",
                 "radix_sort_4bit_passes", "merge_path_partitions_memcache"]:
        assert "ok " + name in r.stdout


NONCOMMUTATIVE = r"""
#include "mgpu/gb300/scan.hxx"
struct first_t {   // keeps its left operand: associative, not commutative
  static __host__ __device__ int identity() { return 0; }
  __device__ int operator()(int a, int) const { return a; }
};
#ifdef OPT_IN
template<> struct mgpu::gb300::commutative_op<first_t> : std::true_type {};
#endif
mgpu::gb300::status_t f(mgpu::gb300::context_t& ctx, int* d, int64_t n) {
  return mgpu::gb300::scan(ctx, d, n, d, 0, first_t());
}
"""


def test_scan_rejects_an_operator_not_declared_commutative(tmp_path):
    """The scans combine partials out of element order, so an operator must
    be declared commutative (the built-ins are); an undeclared one is a
    compile-time error instead of a wrong result.  Compiles only (no GPU)."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    src = tmp_path / "op.cu"
    src.write_text(NONCOMMUTATIVE)
    base = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17",
            "--extended-lambda", "-I", os.path.join(REPO, "include"),
            "-I", os.path.join(REPO, "mgpu-shaders_gb300", "inc"), "-c", str(src),
            "-o", str(tmp_path / "op.o")]
    r = subprocess.run(base, capture_output=True, text=True)
    assert r.returncode != 0 and "commutative" in r.stdout + r.stderr
    r = subprocess.run(base[:1] + ["-DOPT_IN"] + base[1:], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_tuning_table_host_logic(tmp_path):
    """The tuning table (size buckets, lookup precedence, text round trip,
    malformed lines) is host code: compiled with the host compiler and run
    without a GPU."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "tuning_table")
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Werror",
                    "-I", os.path.join(REPO, "mgpu-shaders_gb300", "inc"),
                    os.path.join(HERE, "cpp", "tuning_table.cpp"), "-o", exe],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe, str(tmp_path / "table.txt")], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 0 and "ok tuning_table" in r.stdout, r.stdout + r.stderr

