"""The host planner (validation, ranks, bisection with OpenMP tasks, records, record check)
built with AddressSanitizer and UndefinedBehaviorSanitizer and run on grids up to 85k
entities, so the parallel bisection path runs too; the record check must also reject three
kinds of corrupted record. No GPU needed."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "ferrite.jl_gb300", "csrc")


def test_planner_clean_under_sanitizers(tmp_path):
    gxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if not gxx or not os.path.isdir(cuda_inc):
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path / "planner_sanitize")
    cmd = [gxx, "-std=c++17", "-O1", "-g", "-fopenmp", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
           "-fno-omit-frame-pointer", "-I", cuda_inc, "-include", "cuda_runtime.h", "-I", os.path.join(ROOT, "include"),
           "-I", CSRC, os.path.join(HERE, "planner_sanitize.cpp"), os.path.join(CSRC, "plan.cpp"),
           os.path.join(CSRC, "setup.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    if r.returncode != 0 and "sanitize" in r.stderr and "unrecognized" in r.stderr:
        pytest.skip("this g++ has no sanitizers")
    assert r.returncode == 0, r.stderr[-3000:]
    env = dict(os.environ, OMP_NUM_THREADS="4", ASAN_OPTIONS="detect_leaks=1")
    for args in (["6", "1"], ["12", "3"], ["20", "3", "8192"], ["44", "1"]):
        p = subprocess.run([exe] + args, capture_output=True, text=True, timeout=900, env=env)
        assert p.returncode == 0, (args, p.stdout[-500:], p.stderr[-3000:])
        assert "rc=0" in p.stdout and "ERROR" not in p.stderr and "runtime error" not in p.stderr, (args, p.stderr[-3000:])
        assert "corrupted records rejected: 3 of 3" in p.stdout, p.stdout[-500:]
