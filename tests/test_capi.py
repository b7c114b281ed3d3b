"""CPU checks of the C ABI library: it builds for sm_103a, loads, and
exports every function include/mgpu_gb300.h declares.  No compute calls."""
import ctypes
import os

import pytest


def test_library_exports_declared_symbols(mgpu):
    from mgpu_gb300 import _lib
    names = _lib.declared_functions()
    assert len(names) >= 20
    handle = ctypes.CDLL(_lib.library_path())
    missing = [n for n in names if not hasattr(handle, n)]
    assert not missing, missing


def test_status_strings(mgpu):
    lib = mgpu.lib()
    for code in range(8):
        assert lib.mgpu_status_string(code)


def test_null_context_rejected(mgpu):
    lib = mgpu.lib()
    assert lib.mgpu_synchronize(None) == 1
    assert lib.mgpu_radix_sort(None, 1, None, 0, None, 0, None, None) == 1


def test_no_cpu_fallback_symbols(mgpu):
    """The product library does not link the oracle."""
    from mgpu_gb300 import _lib
    handle = ctypes.CDLL(_lib.library_path())
    for name in ("oracle_sort", "emu_radix_sort", "oracle_merge"):
        assert not hasattr(handle, name)


C_PROGRAM = r"""
#include "mgpu_gb300.h"
#include <stdio.h>
int main(void) {
  /* No device work: argument checks only. */
  size_t aux_size = 0;
  if(mgpu_radix_sort(NULL, MGPU_U32, NULL, 4, NULL, 10, NULL, &aux_size) != MGPU_ERR_INVALID_ARG)
    return 1;
  if(mgpu_radix_sort_count_on_device(NULL, MGPU_U32, NULL, 0, NULL, 10, NULL, NULL, NULL) !=
     MGPU_ERR_INVALID_ARG)
    return 2;
  printf("%s\n", mgpu_status_string(MGPU_ERR_INVALID_ARG));
  return 0;
}
"""


def test_header_is_c99_and_links(mgpu, tmp_path):
    """A C caller (gcc -std=c99 -pedantic, no CUDA headers) compiles against
    include/mgpu_gb300.h, links libmgpu_gb300.so and gets status codes back."""
    import shutil
    import subprocess
    from mgpu_gb300 import _lib
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "caller.c"
    src.write_text(C_PROGRAM)
    exe = str(tmp_path / "caller")
    libdir = os.path.dirname(_lib.library_path())
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
                    "-I", os.path.join(repo, "include"), str(src), "-L", libdir, "-lmgpu_gb300",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True, capture_output=True,
                   text=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stderr)
    assert out.stdout.strip()
