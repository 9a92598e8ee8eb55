"""The C++ facade include/rsa_gpu/user_interface.hxx: compiles against the C ABI (CPU) and runs the
reference's own user_interface scenario (test/test_python.cpp:8-31) on the GPU."""
import os
import subprocess

import pytest

from rsa_mpi_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_user_interface.cpp")
OUT = os.path.join(ROOT, "rsa_mpi_gb300", "_build", "test_user_interface")


def _compile():
    lib = B.build()
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O1", f"-I{os.path.join(ROOT, 'include')}", SRC, "-o", OUT, f"-L{libdir}", "-lrsagpu",
           f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True)
    return OUT


def test_facade_compiles_and_links():
    assert os.path.exists(_compile())


@pytest.mark.gpu
def test_facade_runs_reference_scenario(tmp_path):
    exe = _compile()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "spheres" in r.stdout
    # domain_log as the reference prints it on one rank (rsa_domain.ixx:151-162)
    log = " ==== log: domain [ 0 ] ==== \n == m_inf : 0,0,0\n == m_sup : 3.5,3.5,3.5\n == sbuffer size :  26\n"
    assert log in r.stdout, r.stdout
    vtp = tmp_path / "ParaviewOutput" / "rsa_mpi_0" / "rsa_mpi_0_0.vtp"
    assert (tmp_path / "ParaviewOutput" / "rsa_mpi_0.pvtp").exists() and vtp.exists()
    n = int(vtp.read_text().split('NumberOfPoints="')[1].split('"')[0])
    assert 600 <= n <= 760
