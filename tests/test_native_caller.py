"""The C ABI from compiled code: tests/native/matmul_caller.cpp (g++, include/spreg.h, libspreg.so)
drives MatMulSpecialized as the reference's C++ testbed does (SpMM_SOP.h:107-178)."""
import os
import shutil
import subprocess

import pytest

from spreg import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "native", "matmul_caller.cpp")


@pytest.fixture(scope="module")
def caller(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    _lib.lib()  # raises if the library has not been built
    lib = _lib.LIB_PATH
    out = str(tmp_path_factory.mktemp("native") / "matmul_caller")
    libdir = os.path.dirname(lib)
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", out,
                    f"-L{libdir}", "-l:" + os.path.basename(lib), f"-Wl,-rpath,{libdir}"],
                   check=True, capture_output=True, text=True)
    return out


def test_native_caller_argument_paths(caller):
    r = subprocess.run([caller, "cpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("ok cpu"), r.stderr


@pytest.mark.gpu
def test_native_caller_matmul_specialized(cuda, caller):
    r = subprocess.run([caller, "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok gpu"), r.stdout + r.stderr
