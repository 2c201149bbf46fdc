"""Banded LU with partial pivoting (the host solver of the shift-invert
preconditioner): compiled with g++ and checked by residual on random,
indefinite and pivoting-heavy banded matrices."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_banded_lu(tmp_path):
    exe = str(tmp_path / "banded_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", os.path.join(HERE, "cxx", "banded_check.cpp"),
                           "-I", os.path.join(ROOT, "helfem_gb300", "csrc"), "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stdout
