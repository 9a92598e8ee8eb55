"""The round-size rules of the schedule (heuristic_darts, cap_darts, class_darts, alive_darts in
rsa_mpi_gb300/csrc/host_common.h), compiled with g++ and checked on the host: no GPU is used."""
import os
import shutil
import subprocess

import pytest

from rsa_mpi_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_schedule.cpp")
OUT = os.path.join(ROOT, "rsa_mpi_gb300", "_build", "test_schedule")


def test_round_size_rules(tmp_path):
    lib = B.build()
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    if not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("no CUDA headers")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{os.path.join(ROOT, 'include')}", f"-I{cuda_inc}", SRC, "-o", OUT,
                    f"-L{libdir}", "-lrsagpu", f"-Wl,-rpath,{libdir}"], check=True)
    r = subprocess.run([OUT], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all checks passed" in r.stdout
