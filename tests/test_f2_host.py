"""The float-pair arithmetic of the mixed-precision column solve and stage updates
(fe-project_gb300/csrc/fedg_f2.cuh), compiled for the CPU with IEEE single-precision stand-ins
for the CUDA rounding intrinsics and checked against long-double references.

The certifying Newton residual relies on these operations to hold about 2^-44 relative accuracy
(the tolerance 1e-10 of the residual is then met with five orders of magnitude to spare).
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BOUNDS = {"split": 8e-15, "add": 6e-14, "mul": 6e-14, "mul_f": 6e-14, "add_f": 6e-14, "recip": 6e-14, "dot": 6e-14}


@pytest.mark.skipif(shutil.which("g++") is None or not os.path.exists("/usr/local/cuda/include/cuda_runtime.h"),
                    reason="needs g++ and the CUDA headers")
def test_float_pair_operations(tmp_path):
    exe = tmp_path / "f2_check"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I/usr/local/cuda/include",
                    "-I" + os.path.join(ROOT, "fe-project_gb300", "csrc"), os.path.join(ROOT, "tests", "host", "f2_check.cpp"),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    errs = {ln.split()[0]: float(ln.split()[1]) for ln in out.strip().splitlines()}
    assert set(errs) == set(BOUNDS)
    for name, bound in BOUNDS.items():
        assert errs[name] <= bound, (name, errs[name])
