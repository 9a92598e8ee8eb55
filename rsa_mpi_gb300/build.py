"""Builds the sampler's shared library rsa_mpi_gb300/_build/librsagpu.so with nvcc for sm_103a.

The kernels are compiled once per space dimension (kernels.cu with -DRSA_DIM=2..7) in parallel,
then linked with the dimension-independent kernels and the host driver into one shared library
whose C ABI is include/rsagpu.h.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "librsagpu.so")
CLI = os.path.join(OUT, "rsa")  # the command-line sampler (csrc/rsa_cli.cpp), linked against LIB
ACTIVITY = os.path.join(OUT, "libactivity.so")  # GPU idle meter for bench.py --idle (csrc/activity.cpp, CUPTI)
DIMS = (2, 3, 4, 5, 6, 7)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no multiply-add contraction anywhere; the FP64 decisions also use explicit _rn intrinsics.
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         f"-I{os.path.join(ROOT, 'include')}"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))] + [
        os.path.join(ROOT, "include", "rsagpu.h")]


def _cli_sources():
    inc = os.path.join(ROOT, "include", "rsa_gpu")
    return [os.path.join(CSRC, "rsa_cli.cpp"), LIB] + [os.path.join(inc, f) for f in os.listdir(inc)]


def up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(CLI):
        return False
    t = os.path.getmtime(LIB)
    if not all(os.path.getmtime(s) <= t for s in _sources()):
        return False
    return all(os.path.getmtime(s) <= os.path.getmtime(CLI) for s in _cli_sources())


def build_cli() -> str:
    """g++ build of the command-line sampler; the library is found next to it at run time."""
    tmp = CLI + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", f"-I{os.path.join(ROOT, 'include')}", os.path.join(CSRC, "rsa_cli.cpp"),
           "-o", tmp, f"-L{OUT}", "-lrsagpu", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for rsa_cli.cpp:\n{r.stderr}")
    os.replace(tmp, CLI)
    return CLI


def build_activity() -> str | None:
    """g++ build of the CUPTI activity meter (bench.py --idle); None where the toolkit has no CUPTI."""
    src = os.path.join(CSRC, "activity.cpp")
    if os.path.exists(ACTIVITY) and os.path.getmtime(ACTIVITY) >= os.path.getmtime(src):
        return ACTIVITY
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    inc, libdir = os.path.join(cuda, "include"), os.path.join(cuda, "lib64")
    if not os.path.exists(os.path.join(inc, "cupti.h")):
        return None
    os.makedirs(OUT, exist_ok=True)
    tmp = f"{ACTIVITY}.{os.getpid()}.tmp"  # builds running side by side each write their own
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", f"-I{inc}", src, "-o", tmp, f"-L{libdir}",
                        "-lcupti", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(f"activity meter not built (bench.py --idle unavailable):\n{r.stderr}")
        return None
    os.replace(tmp, ACTIVITY)
    return ACTIVITY


def build(force: bool = False, verbose: bool = False) -> str:
    build_activity()
    if not force and up_to_date():
        return LIB
    lib_fresh = os.path.exists(LIB) and all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in _sources())
    if not force and lib_fresh:
        build_cli()
        return LIB
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    for d in DIMS:
        jobs.append(([nvcc(), *ARCH, *FLAGS, f"-DRSA_DIM={d}", "-c", os.path.join(CSRC, "kernels.cu"),
                      "-o", os.path.join(OUT, f"kernels_d{d}.o")], f"kernels_d{d}"))
    for name in ("kernels_common", "rsagpu", "batch", "noalloc", "mlp"):
        jobs.append(([nvcc(), *ARCH, *FLAGS, "-c", os.path.join(CSRC, f"{name}.cu"),
                      "-o", os.path.join(OUT, f"{name}.o")], name))

    def run(job):
        cmd, name = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return name

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(OUT, f"kernels_d{d}.o") for d in DIMS]
    objs += [os.path.join(OUT, f"{n}.o") for n in ("kernels_common", "rsagpu", "batch", "noalloc", "mlp")]
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    build_cli()
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
