"""The C++ drop-in headers (include/mcleap/) compiled with nvcc into a program
that runs the reference's test drivers against libmcl_gb300.so."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_dropin_program():
    from mcleap_gb300 import build as B

    lib = B.build()
    out_dir = os.path.join(ROOT, "mcleap_gb300", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "test_dropin")
    cmd = [B.nvcc(), "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "test_dropin.cu"),
           "-L", os.path.dirname(lib), "-lmcl_gb300", "-Xlinker", "-rpath," + os.path.dirname(lib), "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout
