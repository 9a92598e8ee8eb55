"""The C-ABI library builds, loads and exports every entry point include/rsagpu.h declares.
No compute call is made here (this runs without a GPU)."""
import ctypes as C
import os

import pytest

from rsa_mpi_gb300 import _lib
from rsa_mpi_gb300 import build as B


def test_library_builds_for_sm103a_and_loads():
    path = B.build()
    assert os.path.exists(path)
    L = _lib.lib()
    assert L.rsagpu_version().decode().startswith("rsagpu")


def test_every_header_symbol_is_exported():
    syms = _lib.header_symbols()
    assert len(syms) >= 30
    L = C.CDLL(B.build())
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    # and the ctypes signatures cover the whole header
    assert set(syms) <= set(_lib._SIGS), set(syms) - set(_lib._SIGS)


def test_errors_are_reported_without_a_gpu_call():
    L = _lib.lib()
    h = C.c_void_p()
    import numpy as np
    inf = np.zeros(2)
    sup = np.ones(2)
    # dimension out of range is rejected before any CUDA call
    rc = L.rsagpu_domain_create(9, _lib.ptr(inf, _lib._d), _lib.ptr(sup, _lib._d), 0.1, C.byref(h))
    assert rc == -1
    assert "dimension" in L.rsagpu_last_error().decode()
    rc = L.rsagpu_radgen_create_counts(2, None, None, None, 0, 0.0, C.byref(h))
    assert rc == -1
    # a negative exclusion distance could put the first radius under the next class's
    r = np.array([0.02, 0.01])
    n = np.array([10, 10], np.uint64)
    rc = L.rsagpu_radgen_create_counts(2, _lib.ptr(r, _lib._d), _lib.ptr(n, _lib._u64), None, 2, -0.03, C.byref(h))
    assert rc == -1 and "exclusion" in L.rsagpu_last_error().decode()
    rc = L.rsagpu_radgen_create_counts(2, _lib.ptr(r, _lib._d), _lib.ptr(n, _lib._u64), None, 2, 0.001, C.byref(h))
    assert rc == 0
    assert L.rsagpu_radgen_destroy(h) == 0


def test_python_module_mirrors_reference_names():
    from rsa_mpi_gb300 import rsa_mpi_py as m
    for dim in range(2, 8):
        for base in ("sphere", "throw_spheres", "rsa_domain", "radius_generator", "rsa_algo"):
            assert hasattr(m, f"{base}_{dim}D")
    assert callable(m.set_nb_threads)
    s = m.sphere_3D([0.1, 0.2, 0.3], 0.05, 2)
    assert s.center == [0.1, 0.2, 0.3] and s.radius == 0.05 and s.phase == 2


def test_activity_meter_builds_and_exports_its_entry_points():
    """bench.py --idle's CUPTI meter (csrc/activity.cpp): built beside the library where the toolkit has CUPTI."""
    path = B.build_activity()
    if path is None:
        pytest.skip("no CUPTI in this CUDA toolkit")
    L = C.CDLL(path)
    assert hasattr(L, "rsa_activity_start") and hasattr(L, "rsa_activity_stop")
